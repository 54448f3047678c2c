"""Within an order-3 time step the level set is fixed through the three velocity stages, so
stages 2 and 3 keep the first projection's curvature, face weights, diagonal and solver
levels.  Two frames (CFL time steps, viscous term on) in both precisions must be bit for bit
what rebuilding everything gives (GB2D_ASM_REUSE=0, in a child process: the switch is read
once per process)."""
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
for n, aprec, sprec in ((97, gb.PRECISION_FP64, gb.PRECISION_FP64), (600, gb.PRECISION_MIXED, gb.PRECISION_MIXED)):
    case = bubbles_case(n, seed=6)
    c = gb.Context(n, n, advection_precision=aprec)
    c.set_flow_params(water_viscosity=1.0, air_viscosity=0.01, viscosity=True)
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p"), (gb.FIELD_UA, "ua"),
                 (gb.FIELD_VA, "va")):
        c.set(f, case[k])
    dt = 0.0
    its = []
    for _ in range(2):
        dt, st = c.advance_frame(cfl=1.0, prev_dt=dt, opts=gb.solve_opts(precision=sprec, tolerance=1e-9))
        its.append(st.iterations)
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p")):
        out[f"{{n}}_{{k}}"] = c.get(f)
    out[f"{{n}}_stats"] = np.array([dt] + its)
    c.close()
np.savez({path!r}, **out)
"""


def run(path, flag):
    env = dict(os.environ, GB2D_ASM_REUSE=flag)
    r = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT, path=str(path))], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    return np.load(path)


def test_stage_reuse_is_exact(gb, tmp_path):
    full = run(tmp_path / "full.npz", "0")
    reuse = run(tmp_path / "reuse.npz", "1")
    for k in full.files:
        np.testing.assert_array_equal(reuse[k], full[k], err_msg=k)
