"""Host-side pieces of the autograd wrappers (no GPU): the ghost-1 extrapolation that the
viscous stages of a time step read, against the oracle's ghost extrapolation, and the split
gravity / walls stage around the viscosity, against the fused one."""
import ctypes
import importlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_extrapolate_ghost1_matches_oracle(oracle, gb):
    ag = importlib.import_module("2d_engine_gb300.autograd")
    rng = np.random.default_rng(41)
    for ni, nj in ((7, 5), (16, 16), (33, 20)):
        phi = rng.standard_normal((nj + 4, ni + 4))
        ref = phi.copy()
        L = oracle.lib()
        L.or_fill_ghost_extrapolate.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.or_fill_ghost_extrapolate(ref.ctypes.data, 2, ni, nj)
        got = ag.extrapolate_ghost1(torch.from_numpy(phi)).numpy()
        rows, cols = slice(2, 2 + nj), slice(2, 2 + ni)
        for sl in ((rows, 1), (rows, 2 + ni), (1, cols), (2 + nj, cols)):
            np.testing.assert_array_equal(got[sl], ref[sl])
        # the interior, the ghost-2 ring and the corners are left as they were
        keep = np.ones_like(phi, dtype=bool)
        for sl in ((rows, 1), (rows, 2 + ni), (1, cols), (2 + nj, cols)):
            keep[sl] = False
        np.testing.assert_array_equal(got[keep], phi[keep])


def test_split_gravity_walls_equals_fused(gb):
    ag = importlib.import_module("2d_engine_gb300.autograd")
    rng = np.random.default_rng(42)
    ni, nj = 12, 9
    u = torch.from_numpy(rng.standard_normal((nj + 4, ni + 5)))
    v = torch.from_numpy(rng.standard_normal((nj + 5, ni + 4)))
    dt, g = 0.013, (0.3, -9.8)
    fu, fv = ag.gravity_walls(u, v, dt, g)
    su, sv = ag.gravity_walls(*ag.gravity_walls(u, v, dt, g, walls=False), dt, (0.0, 0.0), gravity_on=False)
    assert torch.equal(fu, su) and torch.equal(fv, sv)
