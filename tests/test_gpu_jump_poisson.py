"""Known-answer jump-condition Poisson problems of the reference's POISSON_EQUATION_TEST
(tests 3, 5 and 8 on [-1,1]^2, 61 x 61 nodes, Dirichlet boundaries) through
gb2d_jump_poisson_solve: normals bit-exact, the solution against the reference's own,
and, for tests 3 and 5, the discretisation error against the exact solutions equal to
the reference's.  Test 8 (a five-petal interface r = 0.5 + 0.2 sin 5 theta, coefficient
1 inside and 0.1 outside, both jumps; POISSON_EQUATION_TEST.h:441-456, 566-583, 635-652)
states no exact solution the test checks (the reference reports an error for tests 0
and 3 only, :296-306): it is pinned on the reference's own solution."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu
NAMES = ["poisson_test3_61", "poisson_test5_61", "poisson_test8_61"]


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def solve(gb, g, precision, tol):
    n = int(g["n"])
    c = gb.Context(n, n, -1.0, -1.0, 1.0, 1.0)
    bc = np.where(g["bc"] >= 0, 0, g["bc"]).astype(np.int32)
    out = c.jump_poisson_solve(g["beta"], bc, g["rhs"], g["levelset"], g["jc_on_solution"], g["jc_on_derivative"],
                               g["pressure_in"], opts=gb.solve_opts(precision=precision, tolerance=tol, max_iterations=20000))
    c.close()
    return out


def exact(g):
    n = int(g["n"])
    x = np.linspace(-1.0, 1.0, n)
    X, Y = np.meshgrid(x, x)
    if int(g["test_number"]) == 3:
        return g["true_solution"][1:-1, 1:-1]
    r = np.sqrt(X ** 2 + Y ** 2)
    return np.where(r <= 0.5, 1.0, 1.0 + np.log(2 * np.maximum(r, 1e-300)))


def l2_error(g, sol):
    dx = 2.0 / (int(g["n"]) - 1)
    return float(np.sqrt(np.sum((sol[1:-1, 1:-1] - exact(g)) ** 2) * dx * dx))


@pytest.mark.parametrize("name", NAMES)
def test_fp64_matches_reference(gb, name):
    g = load_golden(name)
    sol, nx, ny, st = solve(gb, g, gb.PRECISION_FP64, 1e-12)
    assert st.rel_residual <= 1e-12
    np.testing.assert_array_equal(nx[1:-1, 1:-1], g["normal_x"][1:-1, 1:-1])
    np.testing.assert_array_equal(ny[1:-1, 1:-1], g["normal_y"][1:-1, 1:-1])
    assert rel_l2(sol, g["solution"]) <= 1e-10
    if int(g["test_number"]) == 8:
        return
    # the known answer: the same discretisation error as the reference's solution
    e_ref, e = l2_error(g, g["solution"]), l2_error(g, sol)
    assert abs(e - e_ref) <= 1e-6 * e_ref
    if int(g["test_number"]) == 3:
        assert abs(e_ref - float(g["l2_norm"])) <= 1e-9 * float(g["l2_norm"])
    assert e < 2e-2


@pytest.mark.parametrize("name", NAMES)
def test_mixed_close_to_reference(gb, name):
    g = load_golden(name)
    sol, _, _, st = solve(gb, g, gb.PRECISION_MIXED, 1e-10)
    assert st.rel_residual <= 1e-10
    assert rel_l2(sol, g["solution"]) <= 1e-8
