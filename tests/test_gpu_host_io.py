"""gb2d_projection_host (the projection with its state copied in from and out to host
arrays in one call, the copies overlapping the assembly and the velocity update) gives
exactly what gb2d_set_field + gb2d_projection + gb2d_get_field give."""
import numpy as np
import pytest

from tests.golden.cases import bubbles_case

pytestmark = pytest.mark.gpu


def load(c, gb, case):
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p")):
        c.set(f, case[k])


@pytest.mark.parametrize("n,precision", [(128, "mixed"), (257, "fp64"), (1024, "mixed")])
def test_host_projection_matches_separate_calls(gb, n, precision):
    case = bubbles_case(n, seed=3)
    dt = 0.5 / (n - 1)
    prec = gb.PRECISION_MIXED if precision == "mixed" else gb.PRECISION_FP64
    opts = gb.solve_opts(precision=prec, tolerance=1e-10, max_iterations=2000)
    a = gb.Context(n, n)
    load(a, gb, case)
    sa = a.projection(dt, opts)
    want = {k: a.get(f) for k, f in (("p", gb.FIELD_P), ("u", gb.FIELD_U), ("v", gb.FIELD_V))}
    b = gb.Context(n, n)
    outs = {k: np.full(want[k].shape, np.nan) for k in want}
    sb = b.projection_host(dt, opts, phi=case["phi"], u=case["u"], v=case["v"], p=case["p"], p_out=outs["p"], u_out=outs["u"],
                           v_out=outs["v"])
    assert sb.iterations == sa.iterations
    assert sb.rel_residual == sa.rel_residual
    assert (sb.max_velocity_x, sb.max_velocity_y) == (sa.max_velocity_x, sa.max_velocity_y)
    for k in want:
        assert np.array_equal(outs[k], want[k]), k
        assert np.array_equal(b.get({"p": gb.FIELD_P, "u": gb.FIELD_U, "v": gb.FIELD_V}[k]), want[k]), k
    a.close()
    b.close()


def test_host_projection_null_buffers(gb):
    """Null inputs keep the context's fields; null outputs are not copied."""
    n = 96
    case = bubbles_case(n, seed=5)
    dt = 0.5 / (n - 1)
    opts = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=1e-10, max_iterations=2000)
    a = gb.Context(n, n)
    load(a, gb, case)
    a.projection(dt, opts)
    b = gb.Context(n, n)
    b.set(gb.FIELD_PHI, case["phi"])
    b.set(gb.FIELD_V, case["v"])
    u_out = np.zeros_like(case["u"])
    b.projection_host(dt, opts, u=case["u"], p=case["p"], u_out=u_out)
    assert np.array_equal(u_out, a.get(gb.FIELD_U))
    assert np.array_equal(b.get(gb.FIELD_P), a.get(gb.FIELD_P))
    assert np.array_equal(b.get(gb.FIELD_V), a.get(gb.FIELD_V))
    a.close()
    b.close()
