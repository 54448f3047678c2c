"""The device-driven CG run (one graph launch whose WHILE node iterates until convergence,
started without the host's read of the starting norms) gives exactly what the host-checked
run gives: a projection in both precisions, a solve whose start is already converged (0
iterations), and a solve stopped at its iteration cap.  GB2D_DEVICE_LOOP forces either form
in a child process (the switch is read once per process)."""
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
n = 129
case = bubbles_case(n, seed=4)
dt = 0.5 / (n - 1)
for prec in (gb.PRECISION_FP64, gb.PRECISION_MIXED):
    c = gb.Context(n, n)
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p")):
        c.set(f, case[k])
    st = c.projection(dt, gb.solve_opts(precision=prec, tolerance=1e-10))
    out[f"p{{prec}}"] = c.get(gb.FIELD_P)
    out[f"it{{prec}}"] = np.array([st.iterations, st.outer_iterations, st.rel_residual])
    # the assembled system solved from zero, again from its own solution, and with a cap of 3
    bx, by, dg, rhs = c.poisson_assemble(dt)
    opts = gb.solve_opts(precision=prec, tolerance=1e-9)
    x, s1 = c.poisson_solve(rhs, None, opts)
    x2, s2 = c.poisson_solve(rhs, x, opts)
    x3, s3 = c.poisson_solve(rhs, None, gb.solve_opts(precision=prec, tolerance=1e-12, max_iterations=3), allow_max_iters=True)
    out[f"x{{prec}}"] = x
    out[f"x2{{prec}}"] = x2
    out[f"x3{{prec}}"] = x3
    out[f"s{{prec}}"] = np.array([s1.iterations, s2.iterations, s3.iterations, s1.rel_residual, s2.rel_residual, s3.rel_residual])
    c.close()
np.savez({path!r}, **out)
"""


def run(path, flag):
    env = dict(os.environ, GB2D_DEVICE_LOOP=flag)
    r = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT, path=str(path))], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    return np.load(path)


def test_device_loop_equals_host_loop(gb, tmp_path):
    host = run(tmp_path / "host.npz", "0")
    dev = run(tmp_path / "dev.npz", "1")
    for k in host.files:
        np.testing.assert_array_equal(dev[k], host[k], err_msg=k)
    for prec in (0, 1):
        s = host[f"s{prec}"]
        assert s[0] > 0 and s[1] == 0 and s[2] == 3, s  # converged start: 0 iterations; the cap: 3
