"""Adjoints through the C ABI: the WENO5 advection adjoint and the projection
adjoint against central finite differences of the GPU forward maps, against an
FP64 reference gradient (central differences of the CPU oracle, component by
component), and a rising-bubble differentiation window (centroid height after K
level-set RK3 steps, reinitialisation off) through the torch.autograd wrappers
with checkpointed segments."""
import importlib

import numpy as np
import pytest

from conftest import load_golden
from tests.golden.cases import rising_bubble_case

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

EPS_FD = 1e-6
GRAD_TOL = 1e-5  # adjoint gradients against central differences (relative)


def central(f, x, d, eps=EPS_FD):
    """Central difference of f at x along d, with step eps and one Richardson step at
    eps/2.  Where the level set is locally linear the WENO5 smoothness indicators are
    near their 1e-6 floor and the weights vary on that scale, so the plain quotient at
    eps = 1e-6 carries O(eps^2) errors near 1e-5 relative; the extrapolation removes most
    of them.  The single-sweep checks below, whose difference quotients sum over every
    component of a random direction, step at 1e-7."""
    q = lambda h: (f(x + h * d) - f(x - h * d)) / (2 * h)
    return (4 * q(eps / 2) - q(eps)) / 3


def make_ctx(gb, g):
    return gb.Context(int(g["ni"]), int(g["nj"]), 0.0, 0.0, float(g["x_max"]), float(g["y_max"]))


def advect(gb, c, phi, ua, va, dt):
    c.set(gb.FIELD_PHI, phi)
    c.set(gb.FIELD_UA, ua)
    c.set(gb.FIELD_VA, va)
    c.levelset_advection(dt)
    return c.get(gb.FIELD_PHI)


@pytest.mark.parametrize("name", ["bubbles_17", "bubbles_33", "rising_bubble_40x24"])
def test_weno5_adjoint_matches_finite_differences(gb, name):
    g = load_golden(name)
    dt = float(g["dt"])
    c = make_ctx(gb, g)
    rng = np.random.default_rng(7)
    lam = rng.standard_normal(g["phi"].shape)
    phi, ua, va = g["phi"], g["ua"], g["va"]
    advect(gb, c, phi, ua, va, dt)
    c.set(gb.FIELD_PHI, phi)  # linearise at the input
    mu, mua, mva = c.weno5_adjoint(dt, lam)
    L = lambda p, a, b: float(np.sum(lam * advect(gb, c, p, a, b, dt)))
    nu = ua.size
    Lv = lambda w: L(phi, w[:nu].reshape(ua.shape), w[nu:].reshape(va.shape))
    for k in range(4):
        d = rng.standard_normal(phi.shape)
        fd = central(lambda p: L(p, ua, va), phi, d, eps=1e-7)
        ad = float(np.sum(mu * d))
        assert abs(ad - fd) <= GRAD_TOL * max(abs(fd), 1e-12), (k, ad, fd)
        dw = rng.standard_normal(nu + va.size)
        fd = central(Lv, np.concatenate([ua.ravel(), va.ravel()]), dw, eps=1e-7)
        ad = float(np.sum(mua.ravel() * dw[:nu]) + np.sum(mva.ravel() * dw[nu:]))
        assert abs(ad - fd) <= GRAD_TOL * max(abs(fd), 1e-12), (k, ad, fd)
    c.close()


def test_weno5_adjoint_matches_oracle_reference_gradient(gb, oracle):
    """Every component of d<lam, phi'>/dphi from central differences of the FP64 oracle."""
    g = load_golden("bubbles_17")
    ni, nj, dt = int(g["ni"]), int(g["nj"]), float(g["dt"])
    gr = oracle.grid(ni, nj, 0.0, 0.0, float(g["x_max"]), float(g["y_max"]))
    pr = oracle.params()
    lam = np.random.default_rng(8).standard_normal(g["phi"].shape)

    def L(p):
        q = p.copy()
        oracle.levelset_advection(gr, pr, q, g["ua"].copy(), g["va"].copy(), dt)
        return float(np.sum(lam * q))

    ref = np.zeros_like(lam)
    base = g["phi"].copy()
    for idx in np.ndindex(base.shape):
        e = np.zeros_like(base)
        e[idx] = 1.0
        ref[idx] = central(L, base, e)
    c = make_ctx(gb, g)
    c.set(gb.FIELD_PHI, base); c.set(gb.FIELD_UA, g["ua"]); c.set(gb.FIELD_VA, g["va"])
    mu, _, _ = c.weno5_adjoint(dt, lam, velocity=False)
    assert np.abs(mu - ref).max() <= 1e-6 * np.abs(ref).max()
    c.close()


@pytest.mark.parametrize("name", ["bubbles_17", "bubbles_33", "tall_24x40"])
def test_projection_adjoint_matches_finite_differences(gb, name):
    g = load_golden(name)
    dt = float(g["dt"])
    c = make_ctx(gb, g)
    # 1e-11: the FP64 MG-PCG's attainable relative residual on these systems lies near 2e-12
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-11, max_iterations=20000)
    c.set(gb.FIELD_PHI, g["phi"])
    rng = np.random.default_rng(9)
    lu, lv, lp = rng.standard_normal(g["u"].shape), rng.standard_normal(g["v"].shape), rng.standard_normal(g["p"].shape)
    lp[0, :] = lp[-1, :] = lp[:, 0] = lp[:, -1] = 0  # the pressure ghosts are not unknowns

    def L(u, v):
        c.set(gb.FIELD_U, u); c.set(gb.FIELD_V, v); c.set(gb.FIELD_P, g["p"])
        c.projection(dt, opts, allow_max_iters=True)
        return float(np.sum(lu * c.get(gb.FIELD_U)) + np.sum(lv * c.get(gb.FIELD_V)) + np.sum(lp * c.get(gb.FIELD_P)))

    L(g["u"], g["v"])
    mu, mv, st = c.projection_adjoint(dt, lu, lv, lp, opts)
    assert st.rel_residual <= 1e-11
    eps = 1e-3  # the map is affine in the velocity: only the solver tolerance limits the difference quotient
    for k in range(4):
        du, dv = rng.standard_normal(g["u"].shape), rng.standard_normal(g["v"].shape)
        fd = (L(g["u"] + eps * du, g["v"] + eps * dv) - L(g["u"] - eps * du, g["v"] - eps * dv)) / (2 * eps)
        ad = float(np.sum(mu * du) + np.sum(mv * dv))
        assert abs(ad - fd) <= GRAD_TOL * max(abs(fd), 1e-12), (k, ad, fd)
    c.close()


def window_case():
    c = rising_bubble_case(33, 33, seed=11)
    return c, 0.25 / 32


def test_window_gradient_against_finite_differences(gb):
    """Centroid height after 20 level-set RK3 steps, checkpoints every 10 steps: 16 seeded
    unit directions, central differences with eps = 1e-6 (Richardson-extrapolated)."""
    ag = importlib.import_module("2d_engine_gb300.autograd")
    case, dt = window_case()
    c = gb.Context(33, 33)
    ua, va = torch.from_numpy(case["ua"]), torch.from_numpy(case["va"])
    phi0 = torch.from_numpy(case["phi"].copy()).requires_grad_(True)
    loss = ag.window_loss(c, phi0, ua, va, dt, steps=20, checkpoint_every=10)
    loss.backward()
    grad = phi0.grad.numpy().copy()
    rng = np.random.default_rng(12)
    with torch.no_grad():
        f = lambda p: float(ag.window_loss(c, torch.from_numpy(p), ua, va, dt, steps=20))
        for k in range(16):
            d = rng.standard_normal(case["phi"].shape)
            d /= np.linalg.norm(d)
            fd = central(f, case["phi"], d)
            ad = float(np.sum(grad * d))
            assert abs(ad - fd) <= GRAD_TOL * max(abs(fd), 1e-3 * np.linalg.norm(grad)), (k, ad, fd)
    c.close()


def test_window_gradient_against_oracle_reference(gb, oracle):
    """The same window at 17^2 over 10 steps against the FP64 oracle's component-wise central differences."""
    ag = importlib.import_module("2d_engine_gb300.autograd")
    case = rising_bubble_case(17, 17, seed=13)
    dt, steps = 0.25 / 16, 10
    ni = nj = 17
    gr = oracle.grid(ni, nj)
    pr = oracle.params()
    it = (slice(2, 2 + nj), slice(2, 2 + ni))

    def loss_np(p0):
        p = p0.copy()
        for _ in range(steps):
            keep = p[it].copy()
            oracle.levelset_advection(gr, pr, p, case["ua"].copy(), case["va"].copy(), dt)
            oracle.levelset_advection(gr, pr, p, case["ua"].copy(), case["va"].copy(), dt)
            p[it] = 0.75 * keep + 0.25 * p[it]
            oracle.levelset_advection(gr, pr, p, case["ua"].copy(), case["va"].copy(), dt)
            p[it] = (1 / 3.0) * keep + (2 / 3.0) * p[it]
        return float(ag.centroid_height(torch.from_numpy(p), ni, nj))

    base = case["phi"].copy()
    ref = np.zeros_like(base)
    for idx in np.ndindex(base.shape):
        e = np.zeros_like(base)
        e[idx] = 1.0
        ref[idx] = central(loss_np, base, e)
    c = gb.Context(ni, nj)
    phi0 = torch.from_numpy(base.copy()).requires_grad_(True)
    ag.window_loss(c, phi0, torch.from_numpy(case["ua"]), torch.from_numpy(case["va"]), dt, steps=steps,
                   checkpoint_every=5).backward()
    got = phi0.grad.numpy()
    assert np.abs(got - ref).max() <= GRAD_TOL * np.abs(ref).max()
    c.close()


@pytest.mark.parametrize("name", ["bubbles_17", "bubbles_33", "tall_24x40"])
def test_projection_density_gradient(gb, name):
    """dL/d(water density) and dL/d(air density) of a projection loss: adjoint against central
    differences of the forward projection (the map is smooth in the densities)."""
    g = load_golden(name)
    dt = float(g["dt"])
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-11, max_iterations=20000)
    rng = np.random.default_rng(10)
    lu, lv, lp = rng.standard_normal(g["u"].shape), rng.standard_normal(g["v"].shape), rng.standard_normal(g["p"].shape)
    lp[0, :] = lp[-1, :] = lp[:, 0] = lp[:, -1] = 0

    def ctx(water, air):
        c = gb.Context(int(g["ni"]), int(g["nj"]), 0.0, 0.0, float(g["x_max"]), float(g["y_max"]), water_density=water,
                       air_density=air)
        for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p")):
            c.set(f, g[k])
        c.projection(dt, opts, allow_max_iters=True)
        return c

    def L(water, air):
        c = ctx(water, air)
        val = float(np.sum(lu * c.get(gb.FIELD_U)) + np.sum(lv * c.get(gb.FIELD_V)) + np.sum(lp * c.get(gb.FIELD_P)))
        c.close()
        return val

    c = ctx(1000.0, 1.0)
    c.projection_adjoint(dt, lu, lv, lp, opts)
    dw, da = c.projection_density_gradient(dt)
    c.close()
    for got, f, x in ((dw, lambda h: L(1000.0 + h, 1.0), 1000.0), (da, lambda h: L(1000.0, 1.0 + h), 1.0)):
        h = 1e-2 * x  # large enough that the solves' 1e-11 residual does not show in the quotient
        q = lambda s: (f(s) - f(-s)) / (2 * s)
        fd = (4 * q(h / 2) - q(h)) / 3  # central differences, one Richardson step
        assert abs(got - fd) <= GRAD_TOL * max(abs(fd), 1e-12), (got, fd)


def test_buoyant_window_density_gradient(gb):
    """Gradient of the bubble centroid after a buoyancy-driven projection and 10 level-set RK3
    steps with respect to both densities, through the projection and WENO5 adjoints (with
    checkpointed segments), against central differences of the whole window."""
    ag = importlib.import_module("2d_engine_gb300.autograd")
    case = rising_bubble_case(33, 33, seed=14)
    dt = 0.25 / 32
    u = case["u"].copy()
    v = case["v"].copy()
    v[2:-2, 2:-2] += dt * -9.8  # one gravity step on the y-faces (walls included, as ApplyGraivity)
    state = dict(phi=case["phi"], u=u, v=v, p=case["p"], x_max=1.0, y_max=1.0)

    def loss(w, a, grad=False):
        W = torch.tensor(w, dtype=torch.float64, requires_grad=grad)
        A = torch.tensor(a, dtype=torch.float64, requires_grad=grad)
        L, c = ag.buoyant_window_loss(gb, 33, 33, state, W, A, dt, steps=10, checkpoint_every=5)
        if grad:
            L.backward()
            out = (float(L), float(W.grad), float(A.grad))
        else:
            out = float(L)
        c.close()
        return out

    L0, gw, ga = loss(1000.0, 1.0, grad=True)
    for got, f, x in ((gw, lambda h: loss(1000.0 + h, 1.0), 1000.0), (ga, lambda h: loss(1000.0, 1.0 + h), 1.0)):
        h = 1e-2 * x
        q = lambda s: (f(s) - f(-s)) / (2 * s)
        fd = (4 * q(h / 2) - q(h)) / 3
        assert abs(got - fd) <= GRAD_TOL * max(abs(fd), 1e-3 * abs(L0)), (got, fd)


@pytest.mark.parametrize("name", ["bubbles_17", "bubbles_33", "tall_24x40"])
def test_projection_phi_gradient(gb, name):
    """dL/dphi of a projection loss (face weights, jump fluxes, curvature, velocity update's
    interface faces) against central differences of the forward projection along seeded smooth
    directions of the interior level set.  The steps (2% of the smallest |phi|) leave every
    node's phase unchanged, where the map is smooth; the solves go to 1e-13 so that their
    residual stays out of the quotients.  Densities 3:1 and sigma = 1: at 1000:1 the harmonic
    face weight varies on a scale of 1e-3 |phi| next to a water node at the interface, finer
    than a step the solves' residual allows (the adjoint's algebra is the same)."""
    g = load_golden(name)
    dt = float(g["dt"])
    ni, nj = int(g["ni"]), int(g["nj"])
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-13, max_iterations=20000)
    rng = np.random.default_rng(12)
    lu, lv, lp = rng.standard_normal(g["u"].shape), rng.standard_normal(g["v"].shape), rng.standard_normal(g["p"].shape)
    lp[0, :] = lp[-1, :] = lp[:, 0] = lp[:, -1] = 0

    def ctx(phi):
        c = gb.Context(ni, nj, 0.0, 0.0, float(g["x_max"]), float(g["y_max"]), water_density=3.0, air_density=1.0,
                       surface_tension=1.0)
        c.set(gb.FIELD_PHI, phi)
        for f, k in ((gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p")):
            c.set(f, g[k])
        c.projection(dt, opts, allow_max_iters=True)
        return c

    def L(phi):
        c = ctx(phi)
        val = float(np.sum(lu * c.get(gb.FIELD_U)) + np.sum(lv * c.get(gb.FIELD_V)) + np.sum(lp * c.get(gb.FIELD_P)))
        c.close()
        return val

    phi0 = g["phi"].copy()
    c = ctx(phi0)
    c.projection_adjoint(dt, lu, lv, lp, opts)
    grad = c.projection_phi_gradient(dt)
    c.close()
    inner = np.abs(phi0[2:2 + nj, 2:2 + ni])
    y, x = np.mgrid[0:nj, 0:ni]
    for k in range(3):
        a, b, ph = rng.uniform(1, 4), rng.uniform(1, 4), rng.uniform(0, 2 * np.pi)
        d = np.zeros_like(phi0)
        d[2:2 + nj, 2:2 + ni] = np.sin(a * np.pi * x / ni + ph) * np.cos(b * np.pi * y / nj)
        h = 2e-2 * float(inner.min())  # no node changes phase
        q = lambda s: (L(phi0 + s * d) - L(phi0 - s * d)) / (2 * s)
        fd = (4 * q(h / 2) - q(h)) / 3
        got = float(np.sum(grad * d))
        assert abs(got - fd) <= 1e-4 * max(abs(fd), 1e-9 * abs(L(phi0))), (k, got, fd)


def test_coupled_window_phi_gradient(gb):
    """The fully coupled window: the initial level set drives the projection (face weights,
    jump terms, curvature, velocity update) and is advected 6 level-set RK3 steps by the
    projected velocity; the centroid height's gradient in the initial level set, through both
    paths, against central differences of the whole window along seeded smooth directions
    (densities 3:1, sigma = 1; steps that keep every node's phase)."""
    ag = importlib.import_module("2d_engine_gb300.autograd")
    n = 33
    case = rising_bubble_case(n, n, seed=15)
    dt = 0.25 / 32
    u = case["u"].copy()
    v = case["v"].copy()
    v[2:-2, 2:-2] += dt * -9.8
    state = dict(u=u, v=v, p=case["p"], x_max=1.0, y_max=1.0, sigma=1.0)
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-13, max_iterations=20000)
    phi0 = case["phi"].copy()
    W, A = torch.tensor(3.0, dtype=torch.float64), torch.tensor(1.0, dtype=torch.float64)

    def loss(phi, grad=False):
        P = torch.from_numpy(phi.copy()).requires_grad_(grad)
        L, c = ag.coupled_window_loss(gb, n, n, state, P, W, A, dt, steps=6, checkpoint_every=3, opts=opts)
        if grad:
            L.backward()
            out = (float(L), P.grad.numpy().copy())
        else:
            out = float(L)
        c.close()
        return out

    L0, g = loss(phi0, grad=True)
    rng = np.random.default_rng(16)
    inner = np.abs(phi0[2:2 + n, 2:2 + n])
    y, x = np.mgrid[0:n, 0:n]
    for k in range(2):
        a, b, ph = rng.uniform(1, 3), rng.uniform(1, 3), rng.uniform(0, 2 * np.pi)
        d = np.zeros_like(phi0)
        d[2:2 + n, 2:2 + n] = np.sin(a * np.pi * x / n + ph) * np.cos(b * np.pi * y / n)
        h = 2e-2 * float(inner.min())
        q = lambda s: (loss(phi0 + s * d) - loss(phi0 - s * d)) / (2 * s)
        fd = (4 * q(h / 2) - q(h)) / 3
        got = float(np.sum(g * d))
        assert abs(got - fd) <= 1e-4 * max(abs(fd), 1e-9 * abs(L0)), (k, got, fd)


def test_velocity_advection_adjoint(gb):
    """VJP of the ENO3 velocity advection (both MAC components, advected values and advecting
    velocities) against central differences of the forward along random directions of U and V;
    the steps leave every ENO choice and upwind side unchanged, where the map is linear.  The
    velocity is generic (noise on every face, walls included): a wall column of exact zeros ties
    the ENO comparisons, where the map has a kink and the adjoint follows the forward's
    tie-break."""
    ag = importlib.import_module("2d_engine_gb300.autograd")
    n = 29
    case = rising_bubble_case(n, n, seed=17)
    rng = np.random.default_rng(18)
    u0 = case["u"] * 10.0 + 0.3 * rng.standard_normal(case["u"].shape)
    v0 = case["v"] * 10.0 + 0.3 * rng.standard_normal(case["v"].shape)
    dt = 0.5 / (n - 1)
    lu, lv = rng.standard_normal(u0.shape), rng.standard_normal(v0.shape)
    c = gb.Context(n, n, advection_precision=gb.PRECISION_FP64)

    def forward(u, v):
        c.set(gb.FIELD_U, u)
        c.set(gb.FIELD_V, v)
        c.velocity_advection(dt)
        return c.get(gb.FIELD_U), c.get(gb.FIELD_V)

    def L(u, v):
        uo, vo = forward(u, v)
        return float(np.sum(lu * uo) + np.sum(lv * vo))

    forward(u0, v0)
    mu_ua, mu_va = c.velocity_advection_adjoint(dt, lu, lv)
    gu = lu + ag.ghost_copy_transpose(mu_ua, n + 1, n)
    gv = lv + ag.ghost_copy_transpose(mu_va, n, n + 1)
    for k in range(3):
        du, dv = rng.standard_normal(u0.shape), rng.standard_normal(v0.shape)
        h = 1e-7
        fd = (L(u0 + h * du, v0 + h * dv) - L(u0 - h * du, v0 - h * dv)) / (2 * h)
        got = float(np.sum(gu * du) + np.sum(gv * dv))
        assert abs(got - fd) <= 1e-6 * max(abs(fd), 1.0), (k, got, fd)
    c.close()


def test_time_step_window_gradient(gb):
    """Two whole order-3 time steps (level-set RK3, then three velocity stages of ENO3 advection,
    gravity and walls, projection, with the RK3 blends; reinitialisation and viscosity off) as
    autograd operations: the forward equals gb2d_advance_time_step, and the centroid height's
    gradient in the initial level set and the initial x-velocity matches central differences of
    the whole window (densities 3:1, sigma = 1; generic velocities; steps that change no phase
    and no ENO choice)."""
    ag = importlib.import_module("2d_engine_gb300.autograd")
    n = 25
    case = rising_bubble_case(n, n, seed=19)
    rng = np.random.default_rng(20)
    dt = 0.2 / (n - 1)
    u0 = case["u"] * 5.0 + 0.1 * rng.standard_normal(case["u"].shape)
    v0 = case["v"] * 5.0 + 0.1 * rng.standard_normal(case["v"].shape)
    ua0, va0 = ag.advecting_copy(torch.from_numpy(u0)).numpy(), ag.advecting_copy(torch.from_numpy(v0)).numpy()
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-13, max_iterations=20000)
    kw = dict(surface_tension=1.0, advection_precision=gb.PRECISION_FP64)

    def make(w, a):
        return gb.Context(n, n, water_density=w, air_density=a, **kw)

    def window(phi, u, v, grad=False):
        P, U, V = (torch.from_numpy(x.copy()).requires_grad_(grad) for x in (phi, u, v))
        W, A = torch.tensor(3.0, dtype=torch.float64), torch.tensor(1.0, dtype=torch.float64)
        ls = gb.Context(n, n, **kw)
        state = {"p": case["p"].copy()}
        p, uu, vv, ua, va = P, U, V, torch.from_numpy(ua0), torch.from_numpy(va0)
        for _ in range(2):
            p, uu, vv, ua, va = ag.time_step(ls, p, uu, vv, ua, va, W, A, dt, make, state, opts)
        L = ag.centroid_height(p, n, n)
        out = (float(L), p.detach().numpy().copy(), uu.detach().numpy().copy(), vv.detach().numpy().copy())
        if grad:
            L.backward()
            out = out + (P.grad.numpy().copy(), U.grad.numpy().copy())
        ls.close()
        return out

    # the forward against the library's own time step (0 reinitialisation sweeps, no viscosity)
    c = gb.Context(n, n, water_density=3.0, air_density=1.0, reinit_iterations=0, **kw)
    for f, x in ((gb.FIELD_PHI, case["phi"]), (gb.FIELD_U, u0), (gb.FIELD_V, v0), (gb.FIELD_P, case["p"]), (gb.FIELD_UA, ua0),
                 (gb.FIELD_VA, va0)):
        c.set(f, x)
    for _ in range(2):
        c.advance_time_step(dt, opts)
    L0, phi_t, u_t, v_t, g_phi, g_u = window(case["phi"], u0, v0, grad=True)
    it = (slice(2, 2 + n), slice(2, 2 + n))
    assert np.abs(phi_t[it] - c.get(gb.FIELD_PHI)[it]).max() <= 1e-11
    assert np.abs(u_t[2:2 + n, 2:3 + n] - c.get(gb.FIELD_U)[2:2 + n, 2:3 + n]).max() <= 1e-9
    c.close()

    phi0 = case["phi"]
    inner = np.abs(phi0[it])
    y, x = np.mgrid[0:n, 0:n]
    d = np.zeros_like(phi0)
    d[it] = np.sin(2.3 * np.pi * x / n + 0.4) * np.cos(1.7 * np.pi * y / n)
    h = 2e-2 * float(inner.min())
    q = lambda s: (window(phi0 + s * d, u0, v0)[0] - window(phi0 - s * d, u0, v0)[0]) / (2 * s)
    fd = (4 * q(h / 2) - q(h)) / 3
    got = float(np.sum(g_phi * d))
    assert abs(got - fd) <= 1e-4 * max(abs(fd), 1e-9), ("phi", got, fd)
    du = rng.standard_normal(u0.shape)
    h = 1e-6
    q = lambda s: (window(phi0, u0 + s * du, v0)[0] - window(phi0, u0 - s * du, v0)[0]) / (2 * s)
    fd = (4 * q(h / 2) - q(h)) / 3
    got = float(np.sum(g_u * du))
    assert abs(got - fd) <= 1e-4 * max(abs(fd), 1e-9), ("u", got, fd)


def test_reinitialization_sweep_adjoint(gb):
    """One reinitialisation sweep with S held: its VJP in phi and in S against central
    differences along random directions (an off-centre bubble, so every Godunov case and both
    WENO sides occur)."""
    n = 40
    case = rising_bubble_case(n, n, seed=21)
    c = gb.Context(n, n, advection_precision=gb.PRECISION_FP64)
    rng = np.random.default_rng(22)
    phi = case["phi"]
    p = phi[2:2 + n, 2:2 + n]
    dx = 1.0 / (n - 1)
    sign = p / np.sqrt(p * p + dx * dx)
    lam = rng.standard_normal(phi.shape)
    mu, ms = c.reinit_sweep_adjoint(phi, sign, lam)
    for k in range(4):
        d = rng.standard_normal(phi.shape)
        fd = central(lambda x: float(np.sum(lam * c.reinit_sweep(x, sign))), phi, d, eps=1e-7)
        ad = float(np.sum(mu * d))
        assert abs(ad - fd) <= GRAD_TOL * max(abs(fd), 1e-3 * np.linalg.norm(mu)), (k, ad, fd)
        # Between sign changes of S the sweep is linear in S (the Godunov choices depend on S's
        # sign only), so a wide step has no truncation error and keeps rounding (the step moves
        # the output by dtau * h * step) well below the tolerance.
        e = rng.standard_normal(sign.shape)
        fd = central(lambda x: float(np.sum(lam * c.reinit_sweep(phi, x))), sign, e, eps=1e-5)
        ad = float(np.sum(ms * e))
        assert abs(ad - fd) <= GRAD_TOL * max(abs(fd), 1e-3 * np.linalg.norm(ms)), (k, ad, fd)
    c.close()


def test_levelset_rk3_with_reinitialization_gradient(gb):
    """Centroid height after two whole level-set updates (advection TVD-RK3 plus the
    reinitialisation TVD-RK3, 3 sweeps per Reinitialization): the autograd forward equals
    gb2d_levelset_rk3, and the gradient in the starting level set matches central
    differences."""
    ag = importlib.import_module("2d_engine_gb300.autograd")
    case, dt = window_case()
    c = gb.Context(33, 33, reinit_iterations=3)
    ua, va = torch.from_numpy(case["ua"]), torch.from_numpy(case["va"])
    c.set(gb.FIELD_PHI, case["phi"])
    c.set(gb.FIELD_UA, case["ua"])
    c.set(gb.FIELD_VA, case["va"])
    c.levelset_rk3(dt)
    want = c.get(gb.FIELD_PHI)
    with torch.no_grad():
        got = ag.levelset_rk3(c, torch.from_numpy(case["phi"].copy()), ua, va, dt).numpy()
    np.testing.assert_allclose(got[2:-2, 2:-2], want[2:-2, 2:-2], rtol=0, atol=1e-13)

    def loss(p):
        for _ in range(2):
            p = ag.levelset_rk3(c, p, ua, va, dt)
        return ag.centroid_height(p, 33, 33)

    phi0 = torch.from_numpy(case["phi"].copy()).requires_grad_(True)
    loss(phi0).backward()
    grad = phi0.grad.numpy().copy()
    rng = np.random.default_rng(23)
    with torch.no_grad():
        f = lambda p: float(loss(torch.from_numpy(p)))
        for k in range(6):
            d = rng.standard_normal(case["phi"].shape)
            d /= np.linalg.norm(d)
            fd = central(f, case["phi"], d)
            ad = float(np.sum(grad * d))
            assert abs(ad - fd) <= GRAD_TOL * max(abs(fd), 1e-3 * np.linalg.norm(grad)), (k, ad, fd)
    c.close()


def test_viscosity_adjoint(gb):
    """The sourcing's explicit viscosity (viscosities 1 : 0.01, densities 3 : 1): its VJP in U,
    V, the level set (interior and ghost-1 ring) and the two densities against central
    differences of the GPU forward."""
    n = 30
    case = rising_bubble_case(n, n, seed=24)
    rng = np.random.default_rng(25)
    dt = 0.2 / (n - 1)
    u0 = case["u"] + 0.3 * rng.standard_normal(case["u"].shape)
    v0 = case["v"] + 0.3 * rng.standard_normal(case["v"].shape)

    def fwd(phi, u, v, w=3.0, a=1.0):
        c = gb.Context(n, n, water_density=w, air_density=a)
        c.set_flow_params(water_viscosity=1.0, air_viscosity=0.01, viscosity=True)
        for f, x in ((gb.FIELD_PHI, phi), (gb.FIELD_U, u), (gb.FIELD_V, v)):
            c.set(f, x)
        c.sourcing(dt)
        out = c.get(gb.FIELD_U), c.get(gb.FIELD_V)
        c.close()
        return out

    lu, lv = rng.standard_normal(u0.shape), rng.standard_normal(v0.shape)
    L = lambda out: float(np.sum(lu * out[0]) + np.sum(lv * out[1]))
    c = gb.Context(n, n, water_density=3.0, air_density=1.0)
    c.set_flow_params(water_viscosity=1.0, air_viscosity=0.01, viscosity=True)
    for f, x in ((gb.FIELD_PHI, case["phi"]), (gb.FIELD_U, u0), (gb.FIELD_V, v0)):
        c.set(f, x)
    mu, mv, mp, (dw, da) = c.viscosity_adjoint(dt, lu, lv)
    c.close()
    phi = case["phi"]
    for k in range(3):
        du, dv = rng.standard_normal(u0.shape), rng.standard_normal(v0.shape)
        fd = central(lambda t: L(fwd(phi, u0 + t * du, v0 + t * dv)), 0.0, 1.0, eps=1e-3)  # affine in U, V
        ad = float(np.sum(mu * du) + np.sum(mv * dv))
        assert abs(ad - fd) <= 1e-9 * max(abs(fd), 1.0), ("uv", k, ad, fd)
        dp = rng.standard_normal(phi.shape)
        fd = central(lambda t: L(fwd(phi + t * dp, u0, v0)), 0.0, 1.0, eps=1e-5)
        ad = float(np.sum(mp * dp))
        assert abs(ad - fd) <= GRAD_TOL * max(abs(fd), 1e-3 * np.linalg.norm(mp)), ("phi", k, ad, fd)
    fd = central(lambda t: L(fwd(phi, u0, v0, w=3.0 + t)), 0.0, 1.0, eps=1e-4)
    assert abs(dw - fd) <= GRAD_TOL * abs(fd), ("water", dw, fd)
    fd = central(lambda t: L(fwd(phi, u0, v0, a=1.0 + t)), 0.0, 1.0, eps=1e-4)
    assert abs(da - fd) <= GRAD_TOL * abs(fd), ("air", da, fd)


def test_time_step_with_reinitialization_and_viscosity(gb):
    """One whole order-3 time step with the reinitialisation (2 sweeps per Reinitialization) and
    the explicit viscosity on, as autograd operations: the forward equals gb2d_advance_time_step,
    and the centroid height's gradients in the initial level set, the initial x-velocity and the
    water density match central differences of the step."""
    ag = importlib.import_module("2d_engine_gb300.autograd")
    n = 25
    case = rising_bubble_case(n, n, seed=26)
    rng = np.random.default_rng(27)
    dt = 0.2 / (n - 1)
    u0 = case["u"] * 5.0 + 0.1 * rng.standard_normal(case["u"].shape)
    v0 = case["v"] * 5.0 + 0.1 * rng.standard_normal(case["v"].shape)
    ua0, va0 = ag.advecting_copy(torch.from_numpy(u0)).numpy(), ag.advecting_copy(torch.from_numpy(v0)).numpy()
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-13, max_iterations=20000)
    kw = dict(surface_tension=1.0, advection_precision=gb.PRECISION_FP64, reinit_iterations=2)
    flow = dict(water_viscosity=0.5, air_viscosity=0.05)

    def make(w, a):
        return gb.Context(n, n, water_density=w, air_density=a, **kw)

    def step(phi, u, v, w=3.0, grad=False):
        P, U = (torch.from_numpy(x.copy()).requires_grad_(grad) for x in (phi, u))
        W, A = torch.tensor(w, dtype=torch.float64, requires_grad=grad), torch.tensor(1.0, dtype=torch.float64)
        ls = gb.Context(n, n, **kw)
        state = {"p": case["p"].copy()}
        p, uu, vv, _, _ = ag.time_step(ls, P, U, torch.from_numpy(v), torch.from_numpy(ua0), torch.from_numpy(va0), W, A, dt, make,
                                       state, opts, reinit=True, viscosity=flow)
        L = ag.centroid_height(p, n, n) + 0.01 * (uu[2:2 + n, 2:3 + n] ** 2).sum()
        out = (float(L), p.detach().numpy().copy(), uu.detach().numpy().copy())
        if grad:
            L.backward()
            out = out + (P.grad.numpy().copy(), U.grad.numpy().copy(), float(W.grad))
        ls.close()
        return out

    c = make(3.0, 1.0)
    c.set_flow_params(viscosity=True, **flow)
    for f, x in ((gb.FIELD_PHI, case["phi"]), (gb.FIELD_U, u0), (gb.FIELD_V, v0), (gb.FIELD_P, case["p"]), (gb.FIELD_UA, ua0),
                 (gb.FIELD_VA, va0)):
        c.set(f, x)
    c.advance_time_step(dt, opts)
    _, phi_t, u_t, g_phi, g_u, g_w = step(case["phi"], u0, v0, grad=True)
    it = (slice(2, 2 + n), slice(2, 2 + n))
    assert np.abs(phi_t[it] - c.get(gb.FIELD_PHI)[it]).max() <= 1e-11
    assert np.abs(u_t[2:2 + n, 2:3 + n] - c.get(gb.FIELD_U)[2:2 + n, 2:3 + n]).max() <= 1e-9
    c.close()

    phi0 = case["phi"]
    y, x = np.mgrid[0:n, 0:n]
    d = np.zeros_like(phi0)
    d[it] = np.sin(2.3 * np.pi * x / n + 0.4) * np.cos(1.7 * np.pi * y / n)
    h = 2e-2 * float(np.abs(phi0[it]).min())
    q = lambda s: (step(phi0 + s * d, u0, v0)[0] - step(phi0 - s * d, u0, v0)[0]) / (2 * s)
    fd = (4 * q(h / 2) - q(h)) / 3
    got = float(np.sum(g_phi * d))
    assert abs(got - fd) <= 1e-4 * max(abs(fd), 1e-9), ("phi", got, fd)
    du = rng.standard_normal(u0.shape)
    q = lambda s: (step(phi0, u0 + s * du, v0)[0] - step(phi0, u0 - s * du, v0)[0]) / (2 * s)
    fd = (4 * q(5e-7) - q(1e-6)) / 3
    got = float(np.sum(g_u * du))
    assert abs(got - fd) <= 1e-4 * max(abs(fd), 1e-9), ("u", got, fd)
    q = lambda s: (step(phi0, u0, v0, w=3.0 + s)[0] - step(phi0, u0, v0, w=3.0 - s)[0]) / (2 * s)
    fd = (4 * q(5e-4) - q(1e-3)) / 3
    assert abs(g_w - fd) <= 1e-4 * max(abs(fd), 1e-9), ("water", g_w, fd)
