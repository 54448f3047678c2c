"""ctypes binding of the CPU oracle (oracle/_build/liboracle2d.so).

TEST INFRASTRUCTURE ONLY: the checker the GPU path is compared with.  Imported
by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the
product package.

All arrays follow the reference's ghost-inclusive ARRAY_2D layout
(ARRAY_2D.h:140-146) as numpy arrays of shape (rows = j, cols = i):
    phi (nj+4, ni+4)   u (nj+4, ni+5)   v (nj+5, ni+4)   density (nj+4, ni+4)
    ua  (nj+6, ni+7)   va (nj+7, ni+6)  p (nj+2, ni+2)   kappa (nj, ni)
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle2d.so")
_lib = None


class Grid(ctypes.Structure):
    _fields_ = [("ni", ctypes.c_int), ("nj", ctypes.c_int),
                ("x_min", ctypes.c_double), ("y_min", ctypes.c_double),
                ("x_max", ctypes.c_double), ("y_max", ctypes.c_double)]


class Params(ctypes.Structure):
    _fields_ = [("water_density", ctypes.c_double), ("air_density", ctypes.c_double),
                ("surface_tension", ctypes.c_double), ("weno_epsilon", ctypes.c_double),
                ("reinit_iterations", ctypes.c_int), ("reinit_scaling", ctypes.c_int),
                ("pcg_tolerance", ctypes.c_double), ("pcg_max_iterations", ctypes.c_int),
                ("pcg_rel_residual", ctypes.c_double)]


class Flow(ctypes.Structure):
    _fields_ = [("water_viscosity", ctypes.c_double), ("air_viscosity", ctypes.c_double),
                ("gravity_x", ctypes.c_double), ("gravity_y", ctypes.c_double), ("viscosity", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("residual", ctypes.c_double),
                ("max_velocity_x", ctypes.c_double), ("max_velocity_y", ctypes.c_double)]


def build():
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        G, R, S = ctypes.POINTER(Grid), ctypes.POINTER(Params), ctypes.POINTER(Stats)
        d = ctypes.c_double
        L.or_levelset_advection.argtypes = [G, R, P, P, P, d]
        L.or_reinitialization.argtypes = [G, R, P]
        L.or_levelset_rk3.argtypes = [G, R, P, P, P, d]
        L.or_velocity_advection.argtypes = [G, R, P, P, P, P, d]
        L.or_curvature.argtypes = [G, P, P]
        L.or_projection.argtypes = [G, R, P, P, P, P, P, d, S]
        L.or_poisson_assemble.argtypes = [G, R, P, P, P, P, d, P, P, P, P]
        L.or_poisson_apply.argtypes = [G, P, P, P, P, P]
        L.or_pcg_ic0.argtypes = [G, R, P, P, P, P, P, S]
        L.or_projection_begin.argtypes = [G, R, P, P, P, P, P, d, ctypes.POINTER(ctypes.c_void_p)]
        L.or_projection_iterate.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.or_projection_finish.argtypes = [ctypes.c_void_p, S]
        L.or_projection_free.argtypes = [ctypes.c_void_p]
        L.or_projection_free.restype = None
        L.or_fill_ghost_extrapolate.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        W = ctypes.POINTER(Flow)
        L.or_cfl_time_step.argtypes = [G, R, W, P, P, P, d, P]
        L.or_normals.argtypes = [G, P, P, P]
        L.or_fast_sweeping.argtypes = [G, P, ctypes.c_int]
        L.or_fast_sweeping.restype = ctypes.c_int
        L.or_jump_poisson_assemble.argtypes = [G, P, P, P, P, P, P, P, P, P, P, P, P, P]
        L.or_jump_poisson_assemble.restype = ctypes.c_int
        L.or_cfl_time_step.restype = d
        L.or_apply_gravity.argtypes = [G, W, P, P, d]
        L.or_sourcing.argtypes = [G, R, W, P, P, P, P, d]
        L.or_velocity_bc.argtypes = [G, P, P]
        L.or_solve_for_rk.argtypes = [G, R, W, P, P, P, P, P, P, P, P, d, S]
        L.or_time_step.argtypes = [G, R, W, P, P, P, P, P, P, P, P, d, S]
        for f in ("or_levelset_advection", "or_reinitialization", "or_levelset_rk3", "or_velocity_advection",
                  "or_curvature", "or_projection", "or_poisson_assemble", "or_pcg_ic0", "or_apply_gravity",
                  "or_projection_begin", "or_projection_iterate", "or_projection_finish",
                  "or_sourcing", "or_solve_for_rk", "or_time_step"):
            getattr(L, f).restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def grid(ni, nj, x_min=0.0, y_min=0.0, x_max=1.0, y_max=1.0):
    return Grid(ni, nj, x_min, y_min, x_max, y_max)


def params(water_density=1000.0, air_density=1.0, surface_tension=0.0728, weno_epsilon=1e-6,
           reinit_iterations=25, reinit_scaling=5, pcg_tolerance=1e-12, pcg_max_iterations=100000,
           pcg_rel_residual=0.0):
    return Params(water_density, air_density, surface_tension, weno_epsilon,
                  reinit_iterations, reinit_scaling, pcg_tolerance, pcg_max_iterations, pcg_rel_residual)


def levelset_advection(g, pr, phi, ua, va, dt):
    _check(lib().or_levelset_advection(ctypes.byref(g), ctypes.byref(pr), _p(phi), _p(ua), _p(va), dt), "levelset_advection")


def reinitialization(g, pr, phi):
    _check(lib().or_reinitialization(ctypes.byref(g), ctypes.byref(pr), _p(phi)), "reinitialization")


def levelset_rk3(g, pr, phi, ua, va, dt):
    _check(lib().or_levelset_rk3(ctypes.byref(g), ctypes.byref(pr), _p(phi), _p(ua), _p(va), dt), "levelset_rk3")


def velocity_advection(g, pr, u, v, ua, va, dt):
    _check(lib().or_velocity_advection(ctypes.byref(g), ctypes.byref(pr), _p(u), _p(v), _p(ua), _p(va), dt), "velocity_advection")


def curvature(g, phi, kappa):
    _check(lib().or_curvature(ctypes.byref(g), _p(phi), _p(kappa)), "curvature")


def projection(g, pr, phi, u, v, p, kappa, dt):
    st = Stats()
    _check(lib().or_projection(ctypes.byref(g), ctypes.byref(pr), _p(phi), _p(u), _p(v), _p(p), _p(kappa), dt, ctypes.byref(st)), "projection")
    return st


class ProjectionRun:
    """or_projection split into slices: begin (curvature, assembly, IC(0) factor) at
    construction, iterate(count) runs at most `count` PCG iterations and returns how many
    ran, finish() runs the rest and the velocity update.  The arrays are updated in place
    and must stay alive until finish()."""

    def __init__(self, g, pr, phi, u, v, p, kappa, dt):
        self._keep = (g, pr, phi, u, v, p, kappa)
        h = ctypes.c_void_p()
        _check(lib().or_projection_begin(ctypes.byref(g), ctypes.byref(pr), _p(phi), _p(u), _p(v), _p(p), _p(kappa), dt,
                                         ctypes.byref(h)), "projection_begin")
        self.h = h
        self.done = False

    def iterate(self, count):
        d = ctypes.c_int(0)
        k = lib().or_projection_iterate(self.h, count, ctypes.byref(d))
        if k < 0:
            raise RuntimeError(f"oracle projection_iterate failed with status {k}")
        self.done = bool(d.value)
        return k

    def finish(self):
        st = Stats()
        _check(lib().or_projection_finish(self.h, ctypes.byref(st)), "projection_finish")
        self.close()
        return st

    def close(self):
        if self.h:
            lib().or_projection_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_assemble(g, pr, phi, u, v, kappa, dt):
    ni, nj = g.ni, g.nj
    bx = np.zeros((nj, ni + 1)); by = np.zeros((nj + 1, ni)); dg = np.zeros((nj, ni)); rhs = np.zeros((nj, ni))
    _check(lib().or_poisson_assemble(ctypes.byref(g), ctypes.byref(pr), _p(phi), _p(u), _p(v), _p(kappa), dt,
                                     _p(bx), _p(by), _p(dg), _p(rhs)), "poisson_assemble")
    return bx, by, dg, rhs


def poisson_apply(g, bx, by, dg, x):
    y = np.zeros_like(x)
    lib().or_poisson_apply(ctypes.byref(g), _p(bx), _p(by), _p(dg), _p(x), _p(y))
    return y


def pcg_ic0(g, pr, bx, by, dg, rhs, x):
    st = Stats()
    _check(lib().or_pcg_ic0(ctypes.byref(g), ctypes.byref(pr), _p(bx), _p(by), _p(dg), _p(rhs), _p(x), ctypes.byref(st)), "pcg_ic0")
    return st


def flow(water_viscosity=1.0, air_viscosity=0.01, gravity=(0.0, -9.8), viscosity=False):
    return Flow(water_viscosity, air_viscosity, gravity[0], gravity[1], int(bool(viscosity)))


def _opt(a):
    return None if a is None else _p(a)


def apply_gravity(g, fl, u, v, dt):
    _check(lib().or_apply_gravity(ctypes.byref(g), ctypes.byref(fl), _p(u), _p(v), dt), "apply_gravity")


def sourcing(g, pr, fl, phi, u, v, density, dt):
    _check(lib().or_sourcing(ctypes.byref(g), ctypes.byref(pr), ctypes.byref(fl), _p(phi), _p(u), _p(v), _opt(density), dt),
           "sourcing")


def velocity_bc(g, u, v):
    lib().or_velocity_bc(ctypes.byref(g), _p(u), _p(v))


def solve_for_rk(g, pr, fl, phi, u, v, ua, va, p, kappa, density, dt):
    st = Stats()
    _check(lib().or_solve_for_rk(ctypes.byref(g), ctypes.byref(pr), ctypes.byref(fl), _p(phi), _p(u), _p(v), _p(ua), _p(va),
                                 _p(p), _p(kappa), _opt(density), dt, ctypes.byref(st)), "solve_for_rk")
    return st


def time_step(g, pr, fl, phi, u, v, ua, va, p, kappa, density, dt):
    st = Stats()
    _check(lib().or_time_step(ctypes.byref(g), ctypes.byref(pr), ctypes.byref(fl), _p(phi), _p(u), _p(v), _p(ua), _p(va),
                              _p(p), _p(kappa), _opt(density), dt, ctypes.byref(st)), "time_step")
    return st


def cfl_time_step(g, pr, fl, u, v, kappa, cfl_number=0.5):
    """CFLOneTimeStep: (dt, (c_f, g_f, v_f, s_f))."""
    rates = np.zeros(4)
    dt = lib().or_cfl_time_step(ctypes.byref(g), ctypes.byref(pr), ctypes.byref(fl), _p(u), _p(v), _p(kappa), cfl_number,
                                _p(rates))
    return dt, tuple(rates)


def normals(g, phi):
    """ComputeNormals: fills phi's ghosts (copy) and returns (nx, ny) with ghost 1."""
    nx, ny = np.zeros((g.nj + 2, g.ni + 2)), np.zeros((g.nj + 2, g.ni + 2))
    lib().or_normals(ctypes.byref(g), _p(phi), _p(nx), _p(ny))
    return nx, ny


def jump_poisson_assemble(g, pressure, density, bc, div, phi, nx, ny, jc_solution, jc_derivative):
    ni, nj = g.ni, g.nj
    bc = np.ascontiguousarray(bc, dtype=np.int32)
    bx = np.zeros((nj, ni + 1)); by = np.zeros((nj + 1, ni)); dg = np.zeros((nj, ni)); rhs = np.zeros((nj, ni))
    _check(lib().or_jump_poisson_assemble(ctypes.byref(g), _p(pressure), _p(density), bc.ctypes.data, _p(div), _p(phi), _p(nx),
                                          _p(ny), _p(jc_solution), _p(jc_derivative), _p(bx), _p(by), _p(dg), _p(rhs)),
           "jump_poisson_assemble")
    return bx, by, dg, rhs


def fast_sweeping(g, phi, sweeps=4):
    _check(lib().or_fast_sweeping(ctypes.byref(g), _p(phi), sweeps), "fast_sweeping")
