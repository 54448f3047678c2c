"""The CPU oracle reproduces the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the headless reference build) bit for bit."""
import numpy as np
import pytest

from conftest import golden_names, load_golden

NAMES = golden_names()


def setup(oracle, g):
    ni, nj = int(g["ni"]), int(g["nj"])
    return oracle.grid(ni, nj, 0.0, 0.0, float(g["x_max"]), float(g["y_max"])), ni, nj


@pytest.mark.parametrize("name", NAMES)
def test_levelset_advection_and_reinit(oracle, name):
    g = load_golden(name)
    gr, ni, nj = setup(oracle, g)
    pr = oracle.params()
    phi = g["phi"].copy()
    oracle.levelset_advection(gr, pr, phi, g["ua"].copy(), g["va"].copy(), float(g["dt"]))
    np.testing.assert_array_equal(phi, g["la_phi"])
    oracle.reinitialization(gr, pr, phi)
    np.testing.assert_array_equal(phi, g["reinit_phi"])


@pytest.mark.parametrize("name", NAMES)
def test_levelset_rk3(oracle, name):
    g = load_golden(name)
    gr, ni, nj = setup(oracle, g)
    phi = g["phi"].copy()
    oracle.levelset_rk3(gr, oracle.params(), phi, g["ua"].copy(), g["va"].copy(), float(g["dt"]))
    np.testing.assert_array_equal(phi, g["rk3_phi"])


@pytest.mark.parametrize("name", NAMES)
def test_velocity_advection(oracle, name):
    g = load_golden(name)
    gr, ni, nj = setup(oracle, g)
    u, v, ua, va = g["u"].copy(), g["v"].copy(), g["ua"].copy(), g["va"].copy()
    oracle.velocity_advection(gr, oracle.params(), u, v, ua, va, float(g["dt"]))
    for got, key in ((u, "va_u"), (v, "va_v"), (ua, "va_ua"), (va, "va_va")):
        np.testing.assert_array_equal(got, g[key])


@pytest.mark.parametrize("name", NAMES)
def test_curvature(oracle, name):
    g = load_golden(name)
    gr, ni, nj = setup(oracle, g)
    phi = g["phi"].copy()
    k = np.zeros((nj, ni))
    oracle.curvature(gr, phi, k)
    np.testing.assert_array_equal(k, g["curv_kappa"])
    np.testing.assert_array_equal(phi, g["curv_phi"])


@pytest.mark.parametrize("name", NAMES)
def test_poisson_system(oracle, name):
    g = load_golden(name)
    gr, ni, nj = setup(oracle, g)
    pr = oracle.params()
    phi = g["phi"].copy()
    k = np.zeros((nj, ni))
    oracle.curvature(gr, phi, k)
    bx, by, dg, rhs = oracle.poisson_assemble(gr, pr, phi, g["u"], g["v"], k, float(g["dt"]))
    np.testing.assert_array_equal(rhs.ravel(), g["sys_b"])
    np.testing.assert_array_equal(dg.ravel(), g["sys_diag"])
    ax = oracle.poisson_apply(gr, bx, by, dg, g["sys_x"].reshape(nj, ni))
    np.testing.assert_array_equal(ax.ravel(), g["sys_ax"])


@pytest.mark.parametrize("name", NAMES)
def test_projection(oracle, name):
    g = load_golden(name)
    gr, ni, nj = setup(oracle, g)
    pr = oracle.params(pcg_tolerance=float(g["pcg_tolerance"]), pcg_max_iterations=200000)
    phi, u, v, p = g["phi"].copy(), g["u"].copy(), g["v"].copy(), g["p"].copy()
    k = np.zeros((nj, ni))
    st = oracle.projection(gr, pr, phi, u, v, p, k, float(g["dt"]))
    assert st.iterations == int(g["proj_iterations"])
    np.testing.assert_array_equal(p, g["proj_p"])
    np.testing.assert_array_equal(phi, g["proj_phi"])
    np.testing.assert_array_equal(k, g["proj_kappa"])
    # Interface faces use sin() in the smeared Heaviside: libm may differ by an ulp across hosts.
    for got, key in ((u, "proj_u"), (v, "proj_v")):
        np.testing.assert_allclose(got, g[key], rtol=1e-14, atol=1e-14 * np.abs(g[key]).max())
