"""GPU parity of the SolveForRK stages around the projection and of the whole
order-3 time step, through the C ABI, against the reference's own outputs
(golden fixtures from tests/golden/make_golden.py).

Gravity, density and the wall conditions are bit-exact.  The viscosity's smeared
Heaviside calls sin(), which CUDA and the host libm may round differently in the
last ulp, so viscous faces are held to 1e-13 relative.  Stages that contain a
projection inherit its solver difference (MG-preconditioned CG against the
reference's IC(0)-PCG) and are held to relative-L2 bounds."""
import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu
FLOW_NAMES = [n for n in golden_names() if "step0_u" in load_golden(n)]
FLOW = dict(water_viscosity=1.0, air_viscosity=0.01, gravity=(0.0, -9.8))
SOLVE_TOL = 1e-11
P_TOL = 1e-10        # one projection, FP64 (as the projection parity tests)
STEP_TOL = 1e-9      # three projections in a row, FP64


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_ctx(gb, g, visc, **kw):
    c = gb.Context(int(g["ni"]), int(g["nj"]), 0.0, 0.0, float(g["x_max"]), float(g["y_max"]), **kw)
    c.set_flow_params(viscosity=visc, **FLOW)
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_UA, "ua"), (gb.FIELD_VA, "va"),
                 (gb.FIELD_P, "p")):
        c.set(f, g[k])
    return c


def near(got, want, rtol=1e-13):
    np.testing.assert_allclose(got, want, rtol=rtol, atol=rtol * np.abs(want).max())


@pytest.mark.parametrize("name", FLOW_NAMES)
@pytest.mark.parametrize("visc", [0, 1])
def test_gravity_sourcing_boundary(gb, name, visc):
    g = load_golden(name)
    c = make_ctx(gb, g, visc)
    dt = float(g["dt"])
    c.apply_gravity(dt)
    np.testing.assert_array_equal(c.get(gb.FIELD_U), g["grav_u"])
    np.testing.assert_array_equal(c.get(gb.FIELD_V), g["grav_v"])
    c.sourcing(dt)
    np.testing.assert_array_equal(c.get(gb.FIELD_DENSITY), g[f"src{visc}_density"])
    if visc:
        near(c.get(gb.FIELD_U), g["src1_u"])
        near(c.get(gb.FIELD_V), g["src1_v"])
        assert np.abs(g["src1_u"] - g["grav_u"]).max() > 0  # the viscous term acts
    else:
        np.testing.assert_array_equal(c.get(gb.FIELD_U), g["src0_u"])
        np.testing.assert_array_equal(c.get(gb.FIELD_V), g["src0_v"])
    c.velocity_boundary()
    check = near if visc else np.testing.assert_array_equal
    check(c.get(gb.FIELD_U), g[f"bc{visc}_u"])
    check(c.get(gb.FIELD_V), g[f"bc{visc}_v"])
    c.close()


@pytest.mark.parametrize("name", FLOW_NAMES)
def test_solve_for_rk(gb, name):
    g = load_golden(name)
    c = make_ctx(gb, g, 1)
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=SOLVE_TOL, max_iterations=20000)
    st = c.solve_for_rk(float(g["dt"]), opts)
    assert st.rel_residual <= SOLVE_TOL
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_UA, "ua"), (gb.FIELD_VA, "va"), (gb.FIELD_KAPPA, "kappa")):
        np.testing.assert_array_equal(c.get(f), g["rk_" + k])
    for f, k in ((gb.FIELD_P, "p"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v")):
        assert rel_l2(c.get(f), g["rk_" + k]) <= P_TOL, k
    c.close()


@pytest.mark.parametrize("name", FLOW_NAMES)
def test_solve_for_rk_fused_equals_stages(gb, name):
    """The fused gravity/sourcing/wall pass gives the same bits as the three separate calls."""
    g = load_golden(name)
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=SOLVE_TOL, max_iterations=20000)
    dt = float(g["dt"])
    a = make_ctx(gb, g, 1)
    a.solve_for_rk(dt, opts)
    b = make_ctx(gb, g, 1)
    b.velocity_advection(dt)
    b.apply_gravity(dt)
    b.sourcing(dt)
    b.velocity_boundary()
    b.projection(dt, opts)
    for f in (gb.FIELD_U, gb.FIELD_V, gb.FIELD_P, gb.FIELD_DENSITY, gb.FIELD_UA, gb.FIELD_VA):
        np.testing.assert_array_equal(a.get(f), b.get(f))
    a.close()
    b.close()


@pytest.mark.parametrize("name", FLOW_NAMES)
@pytest.mark.parametrize("visc", [0, 1])
def test_time_step(gb, name, visc):
    g = load_golden(name)
    c = make_ctx(gb, g, visc)
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=SOLVE_TOL, max_iterations=20000)
    st = c.advance_time_step(float(g["dt"]), opts)
    assert st.rel_residual <= SOLVE_TOL and st.iterations >= 3
    # the level set moves before the velocity stages and is bit-exact
    np.testing.assert_array_equal(c.get(gb.FIELD_PHI), g[f"step{visc}_phi"])
    np.testing.assert_array_equal(c.get(gb.FIELD_DENSITY), g[f"step{visc}_density"])
    for f, k in ((gb.FIELD_P, "p"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_UA, "ua"), (gb.FIELD_VA, "va")):
        assert rel_l2(c.get(f), g[f"step{visc}_{k}"]) <= STEP_TOL, k
    c.close()


@pytest.mark.parametrize("name", FLOW_NAMES)
def test_time_step_mixed_close_to_reference(gb, name):
    """FP32 level-set fluxes and the FP32 preconditioner: same step to the mixed path's tolerances."""
    g = load_golden(name)
    c = make_ctx(gb, g, 1, advection_precision=gb.PRECISION_MIXED)
    st = c.advance_time_step(float(g["dt"]), gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=1e-10))
    assert st.rel_residual <= 1e-10
    ni, nj = int(g["ni"]), int(g["nj"])
    inner = (slice(2, 2 + nj), slice(2, 2 + ni))
    assert rel_l2(c.get(gb.FIELD_PHI)[inner], g["step1_phi"][inner]) <= 1e-5
    for f, k in ((gb.FIELD_U, "u"), (gb.FIELD_V, "v")):
        assert rel_l2(c.get(f), g[f"step1_{k}"]) <= 1e-4, k
    c.close()


@pytest.mark.parametrize("name", FLOW_NAMES)
def test_cfl_time_step(gb, name):
    g = load_golden(name)
    c = make_ctx(gb, g, 0)
    c.curvature()
    dt, rates = c.cfl_time_step()
    assert dt == float(g["cfl_dt"])
    assert all(r > 0 for r in rates)
    c.close()


@pytest.mark.parametrize("name", FLOW_NAMES)
def test_advance_frame_matches_oracle(gb, oracle, name):
    """SIMULATION_WORLD::AdvanceOneFrame: curvature, CFL time step, one order-3 step."""
    g = load_golden(name)
    ni, nj = int(g["ni"]), int(g["nj"])
    c = make_ctx(gb, g, 1)
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=SOLVE_TOL, max_iterations=20000)
    dt, st = c.advance_frame(cfl=1.0, prev_dt=0.0, opts=opts)
    gr = oracle.grid(ni, nj, 0.0, 0.0, float(g["x_max"]), float(g["y_max"]))
    pr = oracle.params(pcg_tolerance=float(g["pcg_tolerance"]), pcg_max_iterations=200000)
    fl = oracle.flow(viscosity=True, **FLOW)
    phi, u, v, ua, va, p = (g[k].copy() for k in ("phi", "u", "v", "ua", "va", "p"))
    k = np.zeros((nj, ni))
    oracle.curvature(gr, phi, k)
    want_dt, _ = oracle.cfl_time_step(gr, pr, fl, u, v, k, 0.5)
    assert dt == want_dt * 1.0
    oracle.time_step(gr, pr, fl, phi, u, v, ua, va, p, k, None, dt)
    np.testing.assert_array_equal(c.get(gb.FIELD_PHI), phi)
    for f, want in ((gb.FIELD_P, p), (gb.FIELD_U, u), (gb.FIELD_V, v)):
        assert rel_l2(c.get(f), want) <= STEP_TOL
    c.close()


@pytest.mark.parametrize("name", FLOW_NAMES)
def test_mixed_velocity_advection_and_viscosity_close_to_fp64(gb, name):
    """The FP32 ENO3 and viscous fluxes of the mixed path against the reference's FP64 results."""
    g = load_golden(name)
    dt = float(g["dt"])
    c = make_ctx(gb, g, 1, advection_precision=gb.PRECISION_MIXED)
    c.velocity_advection(dt)
    for f, k in ((gb.FIELD_U, "va_u"), (gb.FIELD_V, "va_v")):
        d = c.get(f) - g[k]
        assert np.abs(d).max() <= 1e-6 * np.abs(g[k]).max(), k
    c.close()
    c = make_ctx(gb, g, 1, advection_precision=gb.PRECISION_MIXED)
    c.apply_gravity(dt)
    c.sourcing(dt)
    for f, k, k0 in ((gb.FIELD_U, "src1_u", "grav_u"), (gb.FIELD_V, "src1_v", "grav_v")):
        # Error relative to the size of the viscous update itself.  Inside the smearing
        # band an FP32 phi (relative error 2^-23) moves H by up to ~1e-7, the face density
        # rho_a + (rho_w - rho_a) H by ~1e-4 for a density ratio of 1000, which is a 1e-4
        # relative change of dt / rho where rho is near rho_a.
        d = c.get(f) - g[k]
        assert np.abs(d).max() <= 1e-4 * np.abs(g[k] - g[k0]).max() + 1e-15 * np.abs(g[k]).max(), k
    c.close()
