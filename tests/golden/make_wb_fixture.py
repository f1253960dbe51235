"""Generate the whole-body model fixtures from a reference checkout.

For each whole-body configuration of the reference it reads the robot's MJCF
with mpx_gb300.mjcf, attaches the configuration's contact points, and saves
the model with the configuration's q0 and p0:

  * aliengo: mpx/data/aliengo/aliengo.xml, named by mpx/config/config_srbd.py:6
    for the SRBD controller's whole-body interface (and by config_aliengo.py).
    The file also keeps config_srbd.py's p_legs0, the aliengo foot positions
    at q0 (config_srbd.py:35,38-43), listed x to 8 digits and y to 3;
  * h1: the model of config_h1.py:8, feet FL, RL, FR, RR (config_h1.py:12).
    FL and RL are differentiated on the left ankle, FR and RR on the right
    (the body_id indices of h1_wb_dynamics, models.py:139-142);
  * talos: the model of config_talos.py:8, eight foot corners
    (config_talos.py:12-13), four on each ankle (talos_wb_dynamics,
    models.py:196-204).

Values are read from the config modules' own text: the first uncommented
`name = jnp.array([...])` or list literal.

Usage:  python tests/golden/make_wb_fixture.py /path/to/reference [outdir]
Output: tests/golden/{aliengo,h1,talos}_wb.npz (committed; the tests only
read them).
"""
import ast
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


def _list(text, name):
    """The first uncommented `name = [...]` list literal of a config module."""
    m = re.search(r"^%s\s*=\s*(\[.*?\])" % name, text, re.S | re.M)
    if m is None:
        raise KeyError(name)
    return ast.literal_eval(m.group(1))


def _model_path(ref, text):
    m = re.search(r"^model_path\s*=.*?'(/data/[^']+)'", text, re.M)
    return os.path.join(ref, "mpx") + m.group(1)


def main(ref, outdir):
    cfgdir = os.path.join(ref, "mpx", "config")
    srbd = open(os.path.join(cfgdir, "config_srbd.py")).read()
    model = mjcf.parse(_model_path(ref, srbd), _list(srbd, "contact_frame"), _list(srbd, "body_name"))
    mjcf.save_npz(model, os.path.join(outdir, "aliengo_wb.npz"), q0=_array(srbd, "q0"),
                  p_legs0=_array(srbd, "p_legs0"))
    for name, per_point in (("h1", [0, 0, 1, 1]), ("talos", [0] * 4 + [1] * 4)):
        text = open(os.path.join(cfgdir, "config_%s.py" % name)).read()
        bodies = _list(text, "body_name")
        model = mjcf.parse(_model_path(ref, text), _list(text, "contact_frame"), [bodies[i] for i in per_point])
        mjcf.save_npz(model, os.path.join(outdir, "%s_wb.npz" % name), q0=_array(text, "q0"), p0=_array(text, "p0"))
    print("wrote", outdir)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MPX_REFERENCE", "")
    if not ref or not os.path.isdir(os.path.join(ref, "mpx")):
        sys.exit("usage: make_wb_fixture.py <reference checkout containing mpx/> [out dir] (or set MPX_REFERENCE)")
    outdir = sys.argv[2] if len(sys.argv) > 2 else os.path.dirname(os.path.abspath(__file__))
    main(ref, outdir)
