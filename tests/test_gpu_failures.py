"""Failure paths of the projection, injected on the host (no GPU fault involved).

The reference stops on a zero level-set gradient in the curvature
(LEVELSET_2D.h:869-873: it prints and exits) and its PCG has no guard against
non-finite values (PCG_METHOD.cpp:254 only compares the residual with the
tolerance).  Through the C ABI the same situations return a status instead:
GB2D_ERR_ZERO_GRADIENT for a flat level set, GB2D_ERR_NONFINITE for a NaN that
reaches the pressure system, and GB2D_ERR_ARG for a non-positive density.  After
each error the context stays usable: a clean state projects normally."""
import numpy as np
import pytest

from tests.golden.cases import bubbles_case

ERR_ARG, ERR_NONFINITE, ERR_ZERO_GRADIENT = -1, -3, -5
N = 48


def _context(gb, case):
    c = gb.Context(N, N)
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p")):
        c.set(f, case[k])
    return c


def _projection_code(gb, c, precision):
    opts = gb.solve_opts(precision=precision, tolerance=1e-8, max_iterations=200)
    try:
        c.projection(0.5 / (N - 1), opts)
    except gb.GB2DError as e:
        return e.code
    return 0


def _recovers(gb, c, precision):
    """A clean state on the same context projects to the tolerance."""
    case = bubbles_case(N, seed=3)
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p")):
        c.set(f, case[k])
    st = c.projection(0.5 / (N - 1), gb.solve_opts(precision=precision, tolerance=1e-8))
    assert st.rel_residual <= 1e-8
    assert np.all(np.isfinite(c.get(gb.FIELD_P)))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_nan_in_level_set_returns_nonfinite(gb, precision):
    case = bubbles_case(N, seed=3)
    case["phi"][2 + N // 2, 2 + N // 3] = np.nan
    c = _context(gb, case)
    assert _projection_code(gb, c, precision) == ERR_NONFINITE
    _recovers(gb, c, precision)
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_nan_in_velocity_returns_nonfinite(gb, precision):
    case = bubbles_case(N, seed=3)
    case["u"][2 + N // 2, 2 + N // 2] = np.nan
    c = _context(gb, case)
    assert _projection_code(gb, c, precision) == ERR_NONFINITE
    _recovers(gb, c, precision)
    c.close()


@pytest.mark.gpu
def test_infinite_velocity_returns_nonfinite(gb):
    case = bubbles_case(N, seed=3)
    case["v"][2 + N // 4, 2 + N // 2] = np.inf
    c = _context(gb, case)
    assert _projection_code(gb, c, 1) == ERR_NONFINITE
    c.close()


@pytest.mark.gpu
def test_flat_level_set_returns_zero_gradient(gb):
    case = bubbles_case(N, seed=3)
    case["phi"][:] = 0.25  # one phase everywhere, no gradient anywhere
    c = _context(gb, case)
    assert _projection_code(gb, c, 1) == ERR_ZERO_GRADIENT
    with pytest.raises(gb.GB2DError) as e:
        c.curvature()
    assert e.value.code == ERR_ZERO_GRADIENT
    _recovers(gb, c, 1)
    c.close()


@pytest.mark.gpu
def test_flat_patch_at_one_node_returns_zero_gradient(gb):
    """Both the central and the one-sided gradient vanish at one node: the
    reference's one-sided fallback (LEVELSET_2D.h:957-968) also divides by zero there."""
    case = bubbles_case(N, seed=3)
    i, j = 2 + N // 2, 2 + N // 2
    case["phi"][j - 1:j + 2, i - 1:i + 2] = case["phi"][j, i]
    c = _context(gb, case)
    with pytest.raises(gb.GB2DError) as e:
        c.curvature()
    assert e.value.code == ERR_ZERO_GRADIENT
    c.close()
