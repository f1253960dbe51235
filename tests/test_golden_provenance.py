"""The committed golden fixtures are what the reference's own source gives.

Regenerates every fixture under tests/golden/ from the reference checkout
(tests/golden/make_golden.py and make_wb_fixture.py, in subprocesses, as a
maintainer would) and checks that each array equals the committed one bit for
bit.  Skipped where the reference checkout is absent (set MPX_REFERENCE to
point at one).
"""
import importlib.util
import os
import subprocess
import sys

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _reference():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    root = mod.reference_root()
    if not root or not os.path.isdir(os.path.join(root, "mpx")):
        pytest.skip("no reference checkout (MPX_REFERENCE)")
    return root


def _same(committed, regenerated):
    a, b = np.load(committed), np.load(regenerated)
    assert sorted(a.files) == sorted(b.files), os.path.basename(committed)
    for k in a.files:
        assert a[k].dtype == b[k].dtype and a[k].shape == b[k].shape and np.array_equal(a[k], b[k]), \
            (os.path.basename(committed), k)


def _run(*args):
    subprocess.run([sys.executable] + list(args), check=True, capture_output=True, timeout=600)


def test_srbd_and_whole_body_vectors_regenerate_bit_for_bit(tmp_path):
    ref = _reference()
    _run(os.path.join(GOLDEN, "make_golden.py"), ref, str(tmp_path / "srbd.npz"))
    _same(os.path.join(GOLDEN, "srbd_golden.npz"), tmp_path / "srbd.npz")
    _run(os.path.join(GOLDEN, "make_golden.py"), ref, "--wb", str(tmp_path / "wb.npz"))
    _same(os.path.join(GOLDEN, "wb_golden.npz"), tmp_path / "wb.npz")
    _run(os.path.join(GOLDEN, "make_golden.py"), ref, "--wbref", str(tmp_path / "wbref.npz"))
    _same(os.path.join(GOLDEN, "wb_refgen.npz"), tmp_path / "wbref.npz")


def test_robot_model_fixtures_regenerate_bit_for_bit(tmp_path):
    ref = _reference()
    _run(os.path.join(GOLDEN, "make_wb_fixture.py"), ref, str(tmp_path))
    for name in ("aliengo_wb.npz", "h1_wb.npz", "talos_wb.npz"):
        _same(os.path.join(GOLDEN, name), tmp_path / name)
