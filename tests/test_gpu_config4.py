"""The differentiation workload at 256^2: the rising bubble's centroid height after K whole
order-3 time steps (autograd.time_step_window_loss: reinitialisation off, viscosity on,
checkpoints every 10 steps; rho 1 : 1000, mu 0.01 : 1, sigma 0.0728, dt 1.5e-4 fixed, seeded
small initial velocities), its gradient in the initial level set and the water density from
the hand-written adjoints, against central differences (eps = 1e-6) along 16 seeded unit
directions, and against the CPU oracle's component-wise FP64 gradient on a sub-window.

The 10-step window is smooth at the differences' scale: all 16 directions agree to 8.1e-7
(measured on GB300), held here to 2e-6.  Over 50 steps the loss is no longer smooth at that
scale, for reasons that belong to the reference's discretisation, which the FP64 path
reproduces bit for bit:
  * the smeared Heaviside uses pi = 3.141592 (MACROS.h:5), so at the band edge |phi| = 1.5 dx
    it reaches 1 + 1.04e-7, not 1: each time a node crosses the edge the face densities and
    viscosities jump by 1e-7 relative.  Along 14 of the 16 directions one node crosses an edge
    within +-eps (three projections of one time step see it);
  * ENO3 stencil selection jumps where the competing second differences have opposite signs,
    and has kinks where they tie (the zero normal velocity on the walls ties them exactly).
A line scan along one direction shows both: jumps of about 1e-12 in the loss and one-sided
slopes that differ by 2% at the base point, with the adjoint on the right-hand slope.  A
build with pi exact removes the band-edge jumps but not the ENO3 ones (its differences
scatter as much).  Central differences over +-1e-6 then scatter by up to 4.1% around the
adjoint (median 9e-4); with the solves held to a fixed 25 iterations, or their tolerance moved
from 1e-12 to 1e-10, the differences do not change, so the solver is not the cause.  The
50-step check holds each direction to 6e-2 and the median to 3e-3, and the water-density
derivative to 1e-2 (measured 5.3e-3 at h = 1).

Sub-window against the oracle: the first 2 steps at 256^2, the GPU adjoint's gradient at four
interface nodes against the oracle's Richardson-extrapolated central differences (h = 1e-6,
5e-7) of the same window, to 1e-5 (the oracle's loss equals the GPU's to the solve tolerance);
and dL/d(rho_water) against the oracle's central difference on a 64^2, 4-step window, to 2e-5
(measured 1.5e-6; the oracle's loss equals the GPU's bit for bit there)."""
import importlib
import math

import numpy as np
import pytest

from tests.golden.cases import rising_bubble_case

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N, DT, EVERY = 256, 1.5e-4, 10
VISC = dict(water_viscosity=1.0, air_viscosity=0.01)
EPS = 1e-6


@pytest.fixture(scope="module")
def ag():
    return importlib.import_module("2d_engine_gb300.autograd")


@pytest.fixture(scope="module")
def case():
    return rising_bubble_case(N, N, seed=31)


def _opts(gb):
    # 1e-10: above the FP64 floor these solves reach (3e-11 relative residual at rho 1:1000)
    return gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-10, max_iterations=2000)


def _loss(gb, ag, case, steps, phi, water=1000.0, grad=False):
    P = torch.from_numpy(phi.copy()).requires_grad_(grad)
    W = torch.tensor(water, dtype=torch.float64, requires_grad=grad)
    A = torch.tensor(1.0, dtype=torch.float64)
    with torch.set_grad_enabled(grad):
        L = ag.time_step_window_loss(gb, N, N, P, torch.from_numpy(case["u"]), torch.from_numpy(case["v"]), W, A, DT, steps, EVERY,
                                     _opts(gb), viscosity=VISC, p0=case["p"])
    if not grad:
        return float(L)
    L.backward()
    return float(L.detach()), P.grad.numpy().copy(), float(W.grad)


def _directions(case):
    rng = np.random.default_rng(32)
    out = []
    for _ in range(16):
        d = np.zeros_like(case["phi"])
        d[2:2 + N, 2:2 + N] = rng.standard_normal((N, N))
        out.append(d / np.linalg.norm(d))
    return out


def _errors(gb, ag, case, steps):
    _, g, gw = _loss(gb, ag, case, steps, case["phi"], grad=True)
    rel = []
    for d in _directions(case):
        fd = (_loss(gb, ag, case, steps, case["phi"] + EPS * d) - _loss(gb, ag, case, steps, case["phi"] - EPS * d)) / (2 * EPS)
        rel.append(abs(float(np.sum(g * d)) - fd) / abs(fd))
    return np.array(rel), gw


def test_window_10_steps_16_directions(gb, ag, case):
    rel, _ = _errors(gb, ag, case, 10)
    assert rel.max() <= 2e-6, rel


def test_window_50_steps_16_directions(gb, ag, case):
    rel, gw = _errors(gb, ag, case, 50)
    assert rel.max() <= 6e-2 and np.median(rel) <= 3e-3, rel
    h = 1.0
    fd = (_loss(gb, ag, case, 50, case["phi"], 1000.0 + h) - _loss(gb, ag, case, 50, case["phi"], 1000.0 - h)) / (2 * h)
    assert abs(gw - fd) <= 1e-2 * abs(fd), (gw, fd)


def _centroid(phi):
    dx = 1.0 / (N - 1)
    eps = 1.5 * dx
    x = -phi[2:2 + N, 2:2 + N] / eps
    h = np.where(x < -1, 0.0, np.where(x > 1, 1.0, 0.5 + 0.5 * x + 0.5 / math.pi * np.sin(math.pi * x)))
    y = (np.arange(N) * dx)[:, None]
    return float((y * h).sum() / h.sum())


def test_subwindow_against_oracle_componentwise(gb, ag, case, oracle):
    steps = 2
    L, g, gw = _loss(gb, ag, case, steps, case["phi"], grad=True)
    gr = oracle.grid(N, N)
    fl = oracle.flow(viscosity=True, **VISC)
    ua0 = ag.advecting_copy(torch.from_numpy(case["u"])).numpy()
    va0 = ag.advecting_copy(torch.from_numpy(case["v"])).numpy()

    def oracle_loss(phi0, water=1000.0):
        pr = oracle.params(water_density=water, air_density=1.0, surface_tension=0.0728, reinit_iterations=0, pcg_tolerance=0.0,
                           pcg_max_iterations=100000, pcg_rel_residual=1e-12)
        phi, u, v = phi0.copy(), case["u"].copy(), case["v"].copy()
        ua, va, p, kap = ua0.copy(), va0.copy(), case["p"].copy(), np.zeros((N, N))
        for _ in range(steps):
            oracle.time_step(gr, pr, fl, phi, u, v, ua, va, p, kap, None, DT)
        return _centroid(phi)

    assert abs(oracle_loss(case["phi"]) - L) <= 1e-12 * abs(L)
    inner = np.abs(case["phi"][2:2 + N, 2:2 + N]) < 1.5 / (N - 1)
    cand = np.argwhere(inner)
    for j, i in cand[np.random.default_rng(5).choice(len(cand), 4, replace=False)]:
        e = np.zeros_like(case["phi"])
        e[2 + j, 2 + i] = 1.0
        # One node moved by 1e-6 leaves an O(h^2) term near 1e-5 in the plain quotient (measured:
        # 3.8e-5, 1.16e-5, 3.0e-6 at h = 2e-6, 1e-6, 5e-7, whatever the oracle's solve tolerance),
        # so the reference value is Richardson's extrapolation from h and h / 2.
        d1, d2 = ((oracle_loss(case["phi"] + h * e) - oracle_loss(case["phi"] - h * e)) / (2 * h) for h in (EPS, EPS / 2))
        fd = (4 * d2 - d1) / 3
        ad = float(g[2 + j, 2 + i])
        assert abs(ad - fd) <= 1e-5 * abs(fd), (i, j, ad, fd, d1, d2)


def test_density_derivative_against_oracle_64(gb, ag, oracle):
    """dL/d(rho_water) against the oracle's central difference (h = 1) on a 64^2, 4-step
    window (dt 6e-4).  At 256^2 over two steps the derivative is ~1e-13 and the oracle's
    quotient scatters by 0.5% between steps of 1, 10 and 20 (its solves' noise), so the
    density is checked where the window moves the bubble enough."""
    n, steps, dt = 64, 4, 6e-4
    c64 = rising_bubble_case(n, n, seed=31)
    P = torch.from_numpy(c64["phi"].copy())
    W = torch.tensor(1000.0, dtype=torch.float64, requires_grad=True)
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-13, max_iterations=20000)
    L = ag.time_step_window_loss(gb, n, n, P, torch.from_numpy(c64["u"]), torch.from_numpy(c64["v"]), W,
                                 torch.tensor(1.0, dtype=torch.float64), dt, steps, 2, opts, viscosity=VISC, p0=c64["p"])
    L.backward()
    gw = float(W.grad)
    gr = oracle.grid(n, n)
    fl = oracle.flow(viscosity=True, **VISC)
    ua0 = ag.advecting_copy(torch.from_numpy(c64["u"])).numpy()
    va0 = ag.advecting_copy(torch.from_numpy(c64["v"])).numpy()

    def oracle_loss(water):
        pr = oracle.params(water_density=water, air_density=1.0, surface_tension=0.0728, reinit_iterations=0, pcg_tolerance=0.0,
                           pcg_max_iterations=100000, pcg_rel_residual=1e-13)
        phi, u, v = c64["phi"].copy(), c64["u"].copy(), c64["v"].copy()
        ua, va, p, kap = ua0.copy(), va0.copy(), c64["p"].copy(), np.zeros((n, n))
        for _ in range(steps):
            oracle.time_step(gr, pr, fl, phi, u, v, ua, va, p, kap, None, dt)
        x = -phi[2:2 + n, 2:2 + n] / (1.5 / (n - 1))
        h = np.where(x < -1, 0.0, np.where(x > 1, 1.0, 0.5 + 0.5 * x + 0.5 / math.pi * np.sin(math.pi * x)))
        y = (np.arange(n) / (n - 1.0))[:, None]
        return float((y * h).sum() / h.sum())

    assert oracle_loss(1000.0) == float(L.detach())
    fd = (oracle_loss(1001.0) - oracle_loss(999.0)) / 2.0
    assert abs(gw - fd) <= 2e-5 * abs(fd), (gw, fd)
