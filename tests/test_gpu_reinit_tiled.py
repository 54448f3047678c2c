"""The tiled mixed reinitialisation sweep equals the per-node one bit for bit (it forms
the same FP64 differences once per tile instead of once per node).  The per-node kernel
is selected with GB2D_REINIT_UNTILED=1 in a child process (the switch is read once)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = r"""
import sys, importlib, numpy as np
sys.path.insert(0, {root!r})
from tests.golden.cases import bubbles_case
gb = importlib.import_module("2d_engine_gb300")
out = {{}}
for ni, nj in ((33, 33), (100, 37), (257, 129)):
    c = bubbles_case(ni, nj, seed=3, x_max=1.0, y_max=(nj - 1) / (ni - 1))
    ctx = gb.Context(ni, nj, 0.0, 0.0, 1.0, (nj - 1) / (ni - 1), advection_precision=gb.PRECISION_MIXED)
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_UA, "ua"), (gb.FIELD_VA, "va")):
        ctx.set(f, c[k])
    ctx.levelset_rk3(0.5 / (ni - 1))
    out[f"{{ni}}x{{nj}}"] = ctx.get(gb.FIELD_PHI)
    ctx.close()
np.savez({path!r}, **out)
"""


def run(path, untiled):
    env = dict(os.environ)
    env.pop("GB2D_REINIT_UNTILED", None)
    if untiled:
        env["GB2D_REINIT_UNTILED"] = "1"
    r = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT, path=str(path))], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return np.load(path)


def test_tiled_equals_per_node(gb, tmp_path):
    a = run(tmp_path / "tiled.npz", False)
    b = run(tmp_path / "untiled.npz", True)
    for k in a.files:
        np.testing.assert_array_equal(a[k], b[k])
