"""ctypes binding of the headless reference build (oracle/_ref/libref2d.so).

Test infrastructure: only tests/golden/make_golden.py (and checks run where the
reference sources are present) use it.  The library exists only where
`make -C oracle/ref` could read the reference sources.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "..", "_ref", "libref2d.so")

PHI, U, V, UA, VA, P, KAPPA, RHO, JC, DIV, SIGN, SCRATCH, DENSITY, U_RK3, V_RK3 = range(15)


def available():
    return os.path.exists(LIB_PATH)


class RefSim:
    """One EULERIAN_FLUID_SOLVER_2D instance of the reference (air/water bubble setup)."""

    def __init__(self, ni, nj, x_min=0.0, y_min=0.0, x_max=1.0, y_max=1.0, water_density=1000.0, air_density=1.0,
                 water_viscosity=1.0, air_viscosity=0.01, surface_tension=0.0728, gravity=(0.0, -9.8),
                 pcg_tolerance=1e-12, pcg_max_iterations=100000, reinit_iterations=25, reinit_scaling=5,
                 cfl_number=0.5, weno_epsilon=1e-6):
        L = ctypes.CDLL(LIB_PATH)
        vp, d, i = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
        L.ref_create.restype = vp
        L.ref_create.argtypes = [i, i, d, d, d, d, ctypes.POINTER(d)]
        L.ref_destroy.argtypes = [vp]
        for f in ("ref_levelset_advection", "ref_reinitialization", "ref_velocity_advection", "ref_projection", "ref_step",
                  "ref_apply_gravity", "ref_sourcing", "ref_solve_for_rk"):
            getattr(L, f).argtypes = [vp, d]
        L.ref_curvature.argtypes = [vp]
        L.ref_velocity_bc.argtypes = [vp]
        L.ref_fast_sweeping.argtypes = [vp, i]
        L.ref_configure_viscosity.argtypes = [vp, i]
        L.ref_cfl_dt.argtypes = [vp]
        L.ref_cfl_dt.restype = d
        L.ref_field_shape.argtypes = [vp, i] + [ctypes.POINTER(i)] * 4
        L.ref_get_field.argtypes = [vp, i, vp]
        L.ref_set_field.argtypes = [vp, i, vp]
        L.ref_pcg_info.argtypes = [vp, ctypes.POINTER(i), ctypes.POINTER(d)]
        L.ref_poisson_system.argtypes = [vp, ctypes.POINTER(i), ctypes.POINTER(i)] + [vp] * 5
        self.L = L
        prm = (d * 13)(water_density, air_density, water_viscosity, air_viscosity, surface_tension,
                       gravity[0], gravity[1], pcg_tolerance, pcg_max_iterations, reinit_iterations,
                       reinit_scaling, cfl_number, weno_epsilon)
        self.h = L.ref_create(ni, nj, x_min, y_min, x_max, y_max, prm)
        self.ni, self.nj = ni, nj

    def close(self):
        if self.h:
            self.L.ref_destroy(self.h)
            self.h = None

    def shape(self, fid):
        a = [ctypes.c_int() for _ in range(4)]
        self.L.ref_field_shape(self.h, fid, *[ctypes.byref(x) for x in a])
        i0, j0, ir, jr = (x.value for x in a)
        return (jr, ir)

    def get(self, fid):
        a = np.zeros(self.shape(fid))
        self.L.ref_get_field(self.h, fid, a.ctypes.data)
        return a

    def set(self, fid, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.shape == self.shape(fid), (a.shape, self.shape(fid))
        self.L.ref_set_field(self.h, fid, a.ctypes.data)

    def levelset_advection(self, dt):
        self.L.ref_levelset_advection(self.h, dt)

    def reinitialization(self, dt=0.0):
        self.L.ref_reinitialization(self.h, dt)

    def velocity_advection(self, dt):
        self.L.ref_velocity_advection(self.h, dt)

    def projection(self, dt):
        self.L.ref_projection(self.h, dt)

    def curvature(self):
        self.L.ref_curvature(self.h)

    def step(self, dt):
        self.L.ref_step(self.h, dt)

    def fast_sweeping(self, sweeps=4):
        self.L.ref_fast_sweeping(self.h, sweeps)

    def apply_gravity(self, dt):
        self.L.ref_apply_gravity(self.h, dt)

    def sourcing(self, dt):
        self.L.ref_sourcing(self.h, dt)

    def velocity_bc(self):
        self.L.ref_velocity_bc(self.h)

    def solve_for_rk(self, dt):
        self.L.ref_solve_for_rk(self.h, dt)

    def configure_viscosity(self, enable):
        """1: apply the delta-function explicit viscosity (the configuration the reference's
        air/water setup skips); 0: the reference's as-shipped air/water behaviour (none)."""
        self.L.ref_configure_viscosity(self.h, int(enable))

    def cfl_dt(self):
        return self.L.ref_cfl_dt(self.h)

    def pcg_info(self):
        it, r = ctypes.c_int(), ctypes.c_double()
        self.L.ref_pcg_info(self.h, ctypes.byref(it), ctypes.byref(r))
        return it.value, r.value

    def poisson_system(self):
        n, nnz = ctypes.c_int(), ctypes.c_int()
        self.L.ref_poisson_system(self.h, ctypes.byref(n), ctypes.byref(nnz), None, None, None, None, None)
        rp = np.zeros(n.value + 1, dtype=np.int32); col = np.zeros(nnz.value, dtype=np.int32)
        val = np.zeros(nnz.value); b = np.zeros(n.value); x = np.zeros(n.value)
        self.L.ref_poisson_system(self.h, ctypes.byref(n), ctypes.byref(nnz), rp.ctypes.data, col.ctypes.data,
                                  val.ctypes.data, b.ctypes.data, x.ctypes.data)
        return rp, col, val, b, x


class RefPoissonTest:
    """POISSON_EQUATION_TEST of the reference (tests 3, 5 and 8: jump-condition Poisson on
    [-1,1]^2 with n x n nodes, Dirichlet boundaries, PCG)."""

    FIELDS = dict(solution=0, true_solution=1, beta=2, rhs=3, jc_on_solution=4, jc_on_derivative=5, bc=6, levelset=7,
                  normal_x=8, normal_y=9)

    def __init__(self, test_number, n, tolerance=1e-13, max_iteration=200000):
        L = ctypes.CDLL(LIB_PATH)
        vp, d, i = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
        L.ref_poisson_create.restype = vp
        L.ref_poisson_create.argtypes = [i, i, d, i]
        L.ref_poisson_destroy.argtypes = [vp]
        L.ref_poisson_solve.restype = d
        L.ref_poisson_solve.argtypes = [vp]
        L.ref_poisson_field.argtypes = [vp, i, ctypes.POINTER(i), ctypes.POINTER(i), vp]
        L.ref_poisson_test_system.argtypes = [vp, ctypes.POINTER(i), ctypes.POINTER(i), vp, vp, vp, vp, ctypes.POINTER(i)]
        self.L = L
        self.h = L.ref_poisson_create(test_number, n, tolerance, max_iteration)
        if not self.h:
            raise ValueError("test number must be 3, 5 or 8")

    def solve(self):
        return self.L.ref_poisson_solve(self.h)

    def get(self, name):
        ir, jr = ctypes.c_int(), ctypes.c_int()
        self.L.ref_poisson_field(self.h, self.FIELDS[name], ctypes.byref(ir), ctypes.byref(jr), None)
        a = np.zeros((jr.value, ir.value))
        self.L.ref_poisson_field(self.h, self.FIELDS[name], ctypes.byref(ir), ctypes.byref(jr), a.ctypes.data)
        return a

    def system(self):
        n, nnz, it = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.L.ref_poisson_test_system(self.h, ctypes.byref(n), ctypes.byref(nnz), None, None, None, None, ctypes.byref(it))
        rp = np.zeros(n.value + 1, dtype=np.int32); col = np.zeros(nnz.value, dtype=np.int32)
        val = np.zeros(nnz.value); b = np.zeros(n.value)
        self.L.ref_poisson_test_system(self.h, ctypes.byref(n), ctypes.byref(nnz), rp.ctypes.data, col.ctypes.data,
                                       val.ctypes.data, b.ctypes.data, ctypes.byref(it))
        return rp, col, val, b, it.value

    def close(self):
        if self.h:
            self.L.ref_poisson_destroy(self.h)
            self.h = None
