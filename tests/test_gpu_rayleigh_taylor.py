"""Rayleigh-Taylor instability: y = 1 + 0.05 cos(2 pi x) on [0,1] x [0,2], heavy fluid
(density 3) above light (1), viscosity 1e-3 in both, no surface tension, gravity -9.8.
With as many nodes in y as in x, dy = 2 dx: the reference's jump operator then puts
only 1/dx^2 terms on its diagonal (POISSON_SOLVER.cpp:872), which both sides mirror.
The GPU FP64 path follows the CPU oracle frame by frame (CFL time steps), and the mixed
path stays close to it."""
import numpy as np
import pytest

from tests.golden.cases import rayleigh_taylor_level_set

pytestmark = pytest.mark.gpu
N = 64
FRAMES = 6
PHYS = dict(water_density=3.0, air_density=1.0, surface_tension=0.0)
FLOW = dict(water_viscosity=1e-3, air_viscosity=1e-3, gravity=(0.0, -9.8))


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_frames(oracle):
    gr = oracle.grid(N, N, 0.0, 0.0, 1.0, 2.0)
    pr = oracle.params(pcg_tolerance=1e-14, pcg_max_iterations=200000, **PHYS)
    fl = oracle.flow(viscosity=True, **FLOW)
    phi = rayleigh_taylor_level_set(N, N)
    u, v = np.zeros((N + 4, N + 5)), np.zeros((N + 5, N + 4))
    ua, va = np.zeros((N + 6, N + 7)), np.zeros((N + 7, N + 6))
    p, k = np.zeros((N + 2, N + 2)), np.zeros((N, N))
    dts = []
    for _ in range(FRAMES):
        oracle.curvature(gr, phi, k)
        dt, _ = oracle.cfl_time_step(gr, pr, fl, u, v, k, 0.5)
        dts.append(dt)
        oracle.time_step(gr, pr, fl, phi, u, v, ua, va, p, k, None, dt)
    return np.array(dts), dict(phi=phi, u=u, v=v, p=p)


def gpu_frames(gb, precision):
    c = gb.Context(N, N, 0.0, 0.0, 1.0, 2.0, advection_precision=precision, **PHYS)
    c.set_flow_params(viscosity=True, cfl_number=0.5, **FLOW)
    c.set(gb.FIELD_PHI, rayleigh_taylor_level_set(N, N))
    opts = gb.solve_opts(precision=precision, tolerance=1e-10, max_iterations=20000)
    dts, dt = [], 0.0
    for _ in range(FRAMES):
        dt, st = c.advance_frame(cfl=1.0, prev_dt=dt, opts=opts)
        assert st.rel_residual <= 1e-10
        dts.append(dt)
    out = {k: c.get(f) for k, f in (("phi", gb.FIELD_PHI), ("u", gb.FIELD_U), ("v", gb.FIELD_V), ("p", gb.FIELD_P))}
    c.close()
    return np.array(dts), out


def test_rayleigh_taylor_fp64_follows_oracle(gb, oracle):
    want_dt, want = oracle_frames(oracle)
    dts, got = gpu_frames(gb, gb.PRECISION_FP64)
    assert dts[0] == want_dt[0]
    assert np.abs(dts / want_dt - 1).max() <= 1e-9
    for k in ("phi", "u", "v", "p"):
        assert rel_l2(got[k], want[k]) <= 1e-8, (k, rel_l2(got[k], want[k]))


def test_rayleigh_taylor_mixed_close_to_oracle(gb, oracle):
    want_dt, want = oracle_frames(oracle)
    dts, got = gpu_frames(gb, gb.PRECISION_MIXED)
    inner = (slice(2, 2 + N), slice(2, 2 + N))
    assert rel_l2(got["phi"][inner], want["phi"][inner]) <= 1e-5
    for k in ("u", "v"):
        assert rel_l2(got[k], want[k]) <= 1e-3, k
