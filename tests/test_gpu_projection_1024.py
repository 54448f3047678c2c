"""The benchmark projection at 1024^2 (8 seeded circles, rho 1:1000, sigma 0.0728, dt = 0.5
dx, zero initial pressure) against the reference's own projection of the same inputs
(tests/golden/projection_1024.npz: PROJECTION_2D::Solve with PCG-IC(0), its pressure
bit-identical to the oracle's, stored every 4th node).

At this size FP64 itself sets a floor.  The reference's solve reaches a true residual of
4.0e-11 and stops improving; solving again from its own result moves p by 1.1e-10
relative (resolve_rel_l2_p in the fixture).  The error of a solve is about 70x its
relative residual, most of it in the pressure's near-constant mode, which only the corner
pin fixes and which the velocity update does not see.  So the FP64 bound here is stated
on u and v (the benchmark spec's 1e-10), with p bounded by a few times the reference's own
noise floor; the mixed path is held to 1e-8 against the reference at the tolerance where
it reaches that (3e-10), and at the benchmark's tolerance (1e-8) its velocities are
within 3e-8 while p carries the near-constant mode at a few 1e-7.

Measured on GB300: FP64 to 5e-11 (20 iterations): p 2.3e-10 (1.3e-10 against the
re-solve), u 2.6e-11, v 2.5e-11; mixed to 3e-10 (24 iterations): p 0.9-1.6e-9, u 2e-10,
v 1.4e-10; mixed to 1e-8 (16 iterations): p 1.2-3.8e-7, u 1.1e-8, v 1.3e-8."""
import numpy as np
import pytest

from conftest import GOLDEN
from tests.golden.cases import bubbles_case

N = 1024


@pytest.fixture(scope="module")
def ref():
    with np.load(f"{GOLDEN}/projection_1024.npz") as z:
        return {k: z[k] for k in z.files}


def project(gb, precision, tol):
    case = bubbles_case(N, seed=0)
    c = gb.Context(N, N)
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p")):
        c.set(f, case[k])
    st = c.projection(0.5 / (N - 1), gb.solve_opts(precision=precision, tolerance=tol, max_iterations=400))
    out = {k: c.get(f) for k, f in (("p", gb.FIELD_P), ("u", gb.FIELD_U), ("v", gb.FIELD_V))}
    c.close()
    return out, st


def errors(out, ref):
    s = int(ref["stride"])
    return {k: float(np.linalg.norm(out[k][1::s, 1::s] - ref[k]) / np.linalg.norm(ref[k])) for k in ("p", "u", "v")}


def test_reference_fixture_records_its_noise_floor(ref):
    assert int(ref["iterations"]) == 4348
    assert ref["true_residual"] < 1e-10 and ref["true_residual_resolve"] < 1e-10
    assert 5e-11 < float(ref["resolve_rel_l2_p"]) < 5e-10
    # the sampled nodes see the same difference as the whole field
    s = float(np.linalg.norm(ref["p_resolve"] - ref["p"]) / np.linalg.norm(ref["p"]))
    assert abs(s / float(ref["resolve_rel_l2_p"]) - 1) < 0.1


@pytest.mark.gpu
def test_fp64_matches_reference_at_1024(gb, ref):
    out, st = project(gb, gb.PRECISION_FP64, 5e-11)
    assert st.rel_residual <= 5e-11
    e = errors(out, ref)
    assert e["u"] <= 1e-10 and e["v"] <= 1e-10, e
    assert e["p"] <= 5 * float(ref["resolve_rel_l2_p"]), e


@pytest.mark.gpu
def test_mixed_within_1e8_of_reference_at_1024(gb, ref):
    out, st = project(gb, gb.PRECISION_MIXED, 3e-10)
    assert st.rel_residual <= 3e-10
    e = errors(out, ref)
    assert max(e.values()) <= 1e-8, e


@pytest.mark.gpu
def test_mixed_at_benchmark_tolerance(gb, ref):
    out, st = project(gb, gb.PRECISION_MIXED, 1e-8)
    assert st.rel_residual <= 1e-8
    e = errors(out, ref)
    assert e["u"] <= 3e-8 and e["v"] <= 3e-8, e
    assert e["p"] <= 1e-6, e
