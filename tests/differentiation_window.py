"""Differentiation window at full size, run on a GPU:  python tests/differentiation_window.py N STEPS SECONDS

The rising bubble (radius 0.15 at (0.5, 0.3), densities 1 : 1000, viscosities 0.01 : 1, sigma
0.0728, gravity -9.8; seeded small velocities so that no ENO comparison ties) on an N x N grid;
the loss is the centroid height after STEPS whole order-3 time steps (reinitialisation off,
viscosity on, fixed dt 1.5e-4 below the viscous CFL limit at 256^2), checkpointed every 10 steps.
Prints one JSON line: the forward and backward times, dL/d water_density against a Richardson
central difference (h = 1), and as many seeded unit directions in the initial level set
(Richardson central differences, eps = 1e-6) as fit in SECONDS (at most 16)."""
import importlib
import json
import os
import sys
import time

import numpy as np
import torch
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from tests.golden.cases import rising_bubble_case
gb = importlib.import_module("2d_engine_gb300")
ag = importlib.import_module("2d_engine_gb300.autograd")
n, steps, budget = int(sys.argv[1]), int(sys.argv[2]), float(sys.argv[3])
case = rising_bubble_case(n, n, seed=31)
dt = 1.5e-4
opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-12, max_iterations=20000)
visc = dict(water_viscosity=1.0, air_viscosity=0.01)
u0, v0 = torch.from_numpy(case["u"]), torch.from_numpy(case["v"])
A = torch.tensor(1.0, dtype=torch.float64)


def loss(phi, w, grad=False):
    P = torch.from_numpy(phi.copy()).requires_grad_(grad)
    W = torch.tensor(w, dtype=torch.float64, requires_grad=grad)
    L = ag.time_step_window_loss(gb, n, n, P, u0, v0, W, A, dt, steps, 10, opts, viscosity=visc, p0=case["p"])
    if not grad:
        return float(L)
    t = time.time()
    L.backward()
    return float(L.detach()), P.grad.numpy().copy(), float(W.grad), time.time() - t


out = {"n": n, "steps": steps, "dt": dt}
t0 = time.time()
L0, g_phi, g_w, t_bwd = loss(case["phi"], 1000.0, grad=True)
out.update(loss=L0, t_forward_backward=time.time() - t0, t_backward=t_bwd, dL_dwater=g_w)
t = time.time()
with torch.no_grad():
    loss(case["phi"], 1000.0)
out["t_forward"] = time.time() - t
q = lambda s: (loss(case["phi"], 1000.0 + s) - loss(case["phi"], 1000.0 - s)) / (2 * s)
with torch.no_grad():
    fd = (4 * q(0.5) - q(1.0)) / 3
out["water"] = [g_w, fd, abs(g_w - fd) / abs(fd)]
rng = np.random.default_rng(32)
it = (slice(2, 2 + n), slice(2, 2 + n))
dirs = []
while time.time() - t0 < budget and len(dirs) < 16:
    d = np.zeros_like(case["phi"])
    d[it] = rng.standard_normal((n, n))
    d /= np.linalg.norm(d)
    with torch.no_grad():
        qq = lambda s: (loss(case["phi"] + s * d, 1000.0) - loss(case["phi"] - s * d, 1000.0)) / (2 * s)
        fd = (4 * qq(0.5e-6) - qq(1e-6)) / 3
    ad = float(np.sum(g_phi * d))
    dirs.append([ad, fd, abs(ad - fd) / max(abs(fd), 1e-300)])
out["phi_dirs"] = dirs
out["t_total"] = time.time() - t0
print(json.dumps(out))
