"""The checkpointed whole-time-step differentiation window (autograd.time_step_window_loss).

Small case: 25^2 nodes, 4 whole order-3 time steps with the explicit viscosity on,
checkpointed every 2 steps.  Its forward and its gradients (initial level set, initial
x-velocity, water density) equal those of the same steps run as one plain autograd graph,
only the level-set context stays open on the GPU between the forward and the backward
pass, and the water-density derivative matches a central difference of the window."""
import gc
import importlib

import numpy as np
import pytest

from tests.golden.cases import rising_bubble_case

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N, STEPS, EVERY = 25, 4, 2
VISC = dict(water_viscosity=0.5, air_viscosity=0.05)


def _inputs():
    case = rising_bubble_case(N, N, seed=23)
    rng = np.random.default_rng(24)
    u0 = case["u"] * 5.0 + 0.1 * rng.standard_normal(case["u"].shape)
    v0 = case["v"] * 5.0 + 0.1 * rng.standard_normal(case["v"].shape)
    return case, u0, v0


def _open_contexts(gb):
    return sum(1 for o in gc.get_objects() if isinstance(o, gb.Context) and getattr(o, "h", None))


def test_checkpointed_window_equals_plain_graph(gb):
    ag = importlib.import_module("2d_engine_gb300.autograd")
    case, u0, v0 = _inputs()
    dt = 0.1 / (N - 1)
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-13, max_iterations=20000)
    kw = dict(surface_tension=0.5, reinit_iterations=0, advection_precision=gb.PRECISION_FP64)

    def leaves():
        return (torch.from_numpy(case["phi"].copy()).requires_grad_(True), torch.from_numpy(u0.copy()).requires_grad_(True),
                torch.from_numpy(v0.copy()), torch.tensor(3.0, dtype=torch.float64, requires_grad=True),
                torch.tensor(1.0, dtype=torch.float64))

    # checkpointed
    P, U, V, W, A = leaves()
    gc.collect()
    before = _open_contexts(gb)
    L = ag.time_step_window_loss(gb, N, N, P, U, V, W, A, dt, STEPS, EVERY, opts, surface_tension=0.5, viscosity=VISC,
                                 p0=case["p"])
    gc.collect()
    held = _open_contexts(gb) - before
    L.backward()
    got = (float(L), P.grad.numpy().copy(), U.grad.numpy().copy(), float(W.grad))
    assert held <= 1, held  # the level-set context only; no per-operation context survives the forward

    # the same steps as one plain graph
    P, U, V, W, A = leaves()

    def make(w, a):
        return gb.Context(N, N, water_density=w, air_density=a, **kw)

    ls = gb.Context(N, N, **kw)
    state = {"p": case["p"].copy()}
    p, uu, vv, ua, va = P, U, V, ag.advecting_copy(U), ag.advecting_copy(V)
    for _ in range(STEPS):
        p, uu, vv, ua, va = ag.time_step(ls, p, uu, vv, ua, va, W, A, dt, make, state, opts, viscosity=VISC)
    L2 = ag.centroid_height(p, N, N)
    gc.collect()
    held_plain = _open_contexts(gb) - before
    L2.backward()
    want = (float(L2), P.grad.numpy().copy(), U.grad.numpy().copy(), float(W.grad))
    ls.close()
    assert held_plain > held  # the plain graph keeps a context per velocity stage operation

    assert got[0] == want[0]
    for a, b in zip(got[1:], want[1:]):
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-14 * np.abs(b).max())

    # the water-density derivative against a central difference of the whole window, to 1e-4
    # relative as the other whole-time-step checks.  The step is 1e-5 rho: over four steps the
    # ENO3 stencil choices of the velocity advection switch within +-1e-3 rho of this state,
    # where the map has kinks (measured: the quotient is 6.26e-5 at h = 3e-3, 6.9155e-5 at
    # 3e-4 and 6.91581e-5 at 3e-5, against the adjoint's 6.91581e-5).
    def loss_at(w):
        with torch.no_grad():
            return float(ag.time_step_window_loss(gb, N, N, torch.from_numpy(case["phi"].copy()), torch.from_numpy(u0.copy()),
                                                  torch.from_numpy(v0.copy()), torch.tensor(w, dtype=torch.float64),
                                                  torch.tensor(1.0, dtype=torch.float64), dt, STEPS, EVERY, opts,
                                                  surface_tension=0.5, viscosity=VISC, p0=case["p"]))

    h = 3e-5
    fd = (loss_at(3.0 + h) - loss_at(3.0 - h)) / (2 * h)
    assert abs(got[3] - fd) <= 1e-4 * max(abs(fd), 1e-12), (got[3], fd)
