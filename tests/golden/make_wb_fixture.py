"""Generate the whole-body fixture from a reference checkout.

Reads the aliengo model that the SRBD controller's whole-body interface uses
(mpx/data/aliengo/aliengo.xml, named by mpx/config/config_srbd.py:6) with
mpx_gb300.mjcf, and the joint angles q0 and foot positions p_legs0 that
config_srbd.py:35,38-43 lists for it (the first, uncommented definitions; the
foot x coordinates are given to 8 digits, the y coordinates to 3).

Usage:  python tests/golden/make_wb_fixture.py /path/to/reference [out.npz]
Output: tests/golden/aliengo_wb.npz (committed; the tests only read it).
"""
import os
import re
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", ".."))
from mpx_gb300 import mjcf  # noqa: E402


def _array(text, name):
    """The first uncommented `name = jnp.array([...])` of a config module."""
    for m in re.finditer(r"^%s\s*=\s*jnp\.array\(\[(.*?)\]\)" % name, text, re.S | re.M):
        body = "\n".join(line.split("#")[0] for line in m.group(1).splitlines())
        return np.array([float(t) for t in re.split(r"[,\s]+", body) if t], dtype=np.float64)
    raise KeyError(name)


def main(ref, out):
    cfg = open(os.path.join(ref, "mpx", "config", "config_srbd.py")).read()
    model = mjcf.parse(os.path.join(ref, "mpx", "data", "aliengo", "aliengo.xml"), ["FL", "FR", "RL", "RR"],
                       ["FL_calf", "FR_calf", "RL_calf", "RR_calf"])
    mjcf.save_npz(model, out, q0=_array(cfg, "q0"), p_legs0=_array(cfg, "p_legs0"))
    print("wrote", out)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                             "aliengo_wb.npz")
    main(ref, out)
