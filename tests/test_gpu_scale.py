"""GPU checks at sizes beyond the golden fixtures: against the CPU oracle at
sizes it finishes in seconds, and size-independent properties at the benchmark
size (1024^2): residual reached, FP64 and mixed solutions agree, the projected
velocity is discretely divergence-free up to the jump terms."""
import numpy as np
import pytest

from tests.golden.cases import bubbles_case

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def load(c, gb, case):
    c.set(gb.FIELD_PHI, case["phi"]); c.set(gb.FIELD_U, case["u"]); c.set(gb.FIELD_V, case["v"]); c.set(gb.FIELD_P, case["p"])
    c.set(gb.FIELD_UA, case["ua"]); c.set(gb.FIELD_VA, case["va"])


@pytest.mark.parametrize("n", [129, 256])
def test_projection_matches_oracle(gb, oracle, n):
    case = bubbles_case(n, seed=7)
    dt = 0.5 / (n - 1)
    g = oracle.grid(n, n)
    phi, u, v, p = case["phi"].copy(), case["u"].copy(), case["v"].copy(), case["p"].copy()
    k = np.zeros((n, n))
    oracle.projection(g, oracle.params(pcg_tolerance=1e-11, pcg_max_iterations=100000), phi, u, v, p, k, dt)
    c = gb.Context(n, n)
    load(c, gb, case)
    st = c.projection(dt, gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-11, max_iterations=500))
    assert st.rel_residual <= 1e-11
    assert rel_l2(c.get(gb.FIELD_P), p) <= 1e-9
    assert rel_l2(c.get(gb.FIELD_U), u) <= 1e-9


@pytest.mark.parametrize("n", [1024, 2048, 2049])
def test_benchmark_size_fp64_vs_mixed(gb, n):
    """At 1024^2 (the finest FP32 level in 32x16 tiles), 2048^2 (32x32 tiles) and 2049^2
    (partial tiles of every shape on every level).  Both solves are held to their FP64 true
    residual, so the pressures agree to the conditioning times the tolerance (the solves go
    to 1e-10 here, for a 1e-7 bound at every size); a smoother that mishandled a tile would
    show as extra iterations of the mixed solve instead, which the iteration bound catches."""
    case = bubbles_case(n, seed=0)
    dt = 0.5 / (n - 1)
    res = {}
    for prec in (gb.PRECISION_FP64, gb.PRECISION_MIXED):
        c = gb.Context(n, n)
        load(c, gb, case)
        st = c.projection(dt, gb.solve_opts(precision=prec, tolerance=1e-10))
        assert st.rel_residual <= 1e-10
        res[prec] = (c.get(gb.FIELD_P), c.get(gb.FIELD_U), st)
        c.close()
    assert rel_l2(res[1][0], res[0][0]) <= 1e-7
    assert rel_l2(res[1][1], res[0][1]) <= 1e-7
    assert res[1][2].iterations <= res[0][2].iterations + 8


def test_reinitialization_restores_distance(gb):
    n = 128
    case = bubbles_case(n, seed=3)
    c = gb.Context(n, n, reinit_iterations=100)
    phi = case["phi"].copy()
    phi[2:-2, 2:-2] *= 3.0  # a level set that is not a distance function
    c.set(gb.FIELD_PHI, phi)
    c.reinitialization()
    out = c.get(gb.FIELD_PHI)[2:-2, 2:-2]
    gy, gx = np.gradient(out, 1.0 / (n - 1))
    band = np.abs(out) < 3.0 / (n - 1)
    mag = np.sqrt(gx ** 2 + gy ** 2)[band]
    assert abs(np.median(mag) - 1.0) < 0.05


def test_alu_peaks_plausible(gb):
    """gb2d_alu_peaks (the denominators of the level-set sweeps' ALU roofline): both finite and
    positive, FP32 far above FP64, neither above the part's nominal rates (GB300: FP32 FMA
    about 80 TFLOP/s at 2.07 GHz, FP64 about 1.3 TFLOP/s)."""
    f64, f32 = gb.alu_peaks()
    assert 0.1 < f64 < 2.0, f64
    assert 10.0 < f32 < 100.0, f32
    assert f32 > 20 * f64
