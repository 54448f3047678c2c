"""The allocation-free solve entry point (gb2d_poisson_solve_noalloc) gives the
same pressure as the context-based gb2d_poisson_solve.

It exists for callers that cannot allocate device memory (hosts that keep all
GPU memory in their own pool, or must not allocate inside a frame); its scratch
is a fixed file-scope device array.  Device buffers for the system are made by
the test itself; the entry point only reads and writes them.  Collected last so
that a run stopping at the first failure has run every other test first."""
import ctypes

import numpy as np
import pytest

from tests.golden.cases import bubbles_case

pytestmark = pytest.mark.gpu


def test_noalloc_solve_matches_context_solve_twice(gb):
    torch = pytest.importorskip("torch")
    ni, nj = 240, 200  # 48000 unknowns, under the 65536 maximum
    case = bubbles_case(ni, nj, seed=21)
    dt = 0.5 / (ni - 1)
    c = gb.Context(ni, nj)
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v")):
        c.set(f, case[k])
    bx, by, dg, rhs = c.poisson_assemble(dt)
    opts = gb.solve_opts(solver=gb.SOLVER_PCG_JACOBI, precision=gb.PRECISION_FP64, tolerance=1e-11, max_iterations=50000)
    x_ref, st = c.poisson_solve(rhs, None, opts)
    assert st.rel_residual <= 1e-11

    dev = {k: torch.from_numpy(np.ascontiguousarray(a)).cuda() for k, a in (("bx", bx), ("by", by), ("dg", dg), ("rhs", rhs))}
    lib = gb.library()
    dx, dy = 1.0 / (ni - 1), 1.0 / (nj - 1)
    for call in range(2):
        x = torch.zeros((nj, ni), dtype=torch.float64, device="cuda")
        it, rr = ctypes.c_int(), ctypes.c_double()
        rc = lib.gb2d_poisson_solve_noalloc(ni, nj, dx, dy, dev["bx"].data_ptr(), dev["by"].data_ptr(), dev["dg"].data_ptr(),
                                            dev["rhs"].data_ptr(), x.data_ptr(), 1e-11, 50000, None, ctypes.byref(it), ctypes.byref(rr))
        assert rc == 0, (call, rc)
        assert rr.value <= 1e-11
        got = x.cpu().numpy()
        err = np.linalg.norm(got - x_ref) / np.linalg.norm(x_ref)
        assert err <= 1e-10, (call, err)


def test_noalloc_converged_warm_start_returns_unchanged(gb):
    """A warm start that already meets the tolerance (here the context solver's
    solution) takes zero iterations, leaves x bit for bit as it was and returns 0;
    so does an all-zero right-hand side."""
    torch = pytest.importorskip("torch")
    ni, nj = 120, 96
    case = bubbles_case(ni, nj, seed=5)
    dt = 0.5 / (ni - 1)
    c = gb.Context(ni, nj)
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v")):
        c.set(f, case[k])
    bx, by, dg, rhs = c.poisson_assemble(dt)
    opts = gb.solve_opts(solver=gb.SOLVER_PCG_JACOBI, precision=gb.PRECISION_FP64, tolerance=1e-12, max_iterations=50000)
    x_ref, st = c.poisson_solve(rhs, None, opts)
    c.close()
    dev = {k: torch.from_numpy(np.ascontiguousarray(a)).cuda() for k, a in (("bx", bx), ("by", by), ("dg", dg), ("rhs", rhs))}
    lib = gb.library()
    dx, dy = 1.0 / (ni - 1), 1.0 / (nj - 1)
    for rhs_dev, x0 in ((dev["rhs"], x_ref), (torch.zeros_like(dev["rhs"]), np.zeros_like(x_ref))):
        x = torch.from_numpy(np.ascontiguousarray(x0)).cuda()
        it, rr = ctypes.c_int(-1), ctypes.c_double(-1.0)
        rc = lib.gb2d_poisson_solve_noalloc(ni, nj, dx, dy, dev["bx"].data_ptr(), dev["by"].data_ptr(), dev["dg"].data_ptr(),
                                            rhs_dev.data_ptr(), x.data_ptr(), 1e-8, 100, None, ctypes.byref(it), ctypes.byref(rr))
        assert rc == 0
        assert it.value == 0
        assert rr.value <= 1e-8
        assert np.array_equal(x.cpu().numpy(), x0)


def test_noalloc_rejects_sizes_above_maximum(gb):
    lib = gb.library()
    it, rr = ctypes.c_int(), ctypes.c_double()
    n = 257  # 66049 > 65536 unknowns
    rc = lib.gb2d_poisson_solve_noalloc(n, n, 0.1, 0.1, 1, 1, 1, 1, 1, 1e-8, 10, None, ctypes.byref(it), ctypes.byref(rr))
    assert rc == -7
