"""Python binding of the gb2d C ABI (include/gb2d.h) for sm_103a GPUs.

The product is the CUDA library 2d_engine_gb300/_build/libgb2d.so; this module
loads it with ctypes and mirrors the step interface of the reference solver's
EULERIAN_FLUID_SOLVER_2D (Levelset_Advection, Reinitialization,
Velocity_Advection, Projection, SolveForRK and its gravity / sourcing / wall
stages, AdvanceOneTimeStepThread).  There is no CPU fallback: if the library is
missing or no GPU is visible, the calls raise.

Arrays are numpy float64 in the reference's ghost-inclusive ARRAY_2D layout,
shape (rows = j, cols = i):  phi (nj+4, ni+4), u (nj+4, ni+5), v (nj+5, ni+4),
ua (nj+6, ni+7), va (nj+7, ni+6), p (nj+2, ni+2), kappa (nj, ni), density (nj+4, ni+4).
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libgb2d.so")

FIELD_PHI, FIELD_U, FIELD_V, FIELD_UA, FIELD_VA, FIELD_P, FIELD_KAPPA, FIELD_DENSITY = range(8)
PRECISION_FP64, PRECISION_MIXED = 0, 1
SOLVER_MGPCG, SOLVER_PCG_JACOBI = 0, 1

ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "non-finite value", -4: "iteration cap reached",
          -5: "zero level-set gradient", -6: "no CUDA device", -7: "size above the fixed maximum"}
NOALLOC_MAX_CELLS = 65536


class GridT(ctypes.Structure):
    _fields_ = [("ni", ctypes.c_int), ("nj", ctypes.c_int), ("x_min", ctypes.c_double), ("y_min", ctypes.c_double),
                ("x_max", ctypes.c_double), ("y_max", ctypes.c_double)]


class ParamsT(ctypes.Structure):
    _fields_ = [("water_density", ctypes.c_double), ("air_density", ctypes.c_double), ("surface_tension", ctypes.c_double),
                ("weno_epsilon", ctypes.c_double), ("reinit_iterations", ctypes.c_int), ("reinit_scaling", ctypes.c_int),
                ("advection_precision", ctypes.c_int)]


class FlowParamsT(ctypes.Structure):
    _fields_ = [("water_viscosity", ctypes.c_double), ("air_viscosity", ctypes.c_double), ("gravity_x", ctypes.c_double),
                ("gravity_y", ctypes.c_double), ("cfl_number", ctypes.c_double), ("viscosity", ctypes.c_int)]


class SolveOptsT(ctypes.Structure):
    _fields_ = [("solver", ctypes.c_int), ("precision", ctypes.c_int), ("tolerance", ctypes.c_double),
                ("max_iterations", ctypes.c_int), ("mg_smooth", ctypes.c_int)]


class SolveStatsT(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("outer_iterations", ctypes.c_int), ("rel_residual", ctypes.c_double),
                ("max_velocity_x", ctypes.c_double), ("max_velocity_y", ctypes.c_double)]


class BatchStatsT(ctypes.Structure):
    _fields_ = [("frames", ctypes.c_int), ("instances", ctypes.c_int), ("cg_iterations", ctypes.c_longlong),
                ("max_rel_residual", ctypes.c_double), ("wall_ms", ctypes.c_double), ("cell_frames_per_s", ctypes.c_double)]


class GB2DError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gb2d error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


_lib = None


def library():
    """Load libgb2d.so (built by __graft_entry__.build() / 2d_engine_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA library first (python 2d_engine_gb300/build.py)")
    L = ctypes.CDLL(LIB_PATH)
    vp, d, i = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
    G, P, O, S = ctypes.POINTER(GridT), ctypes.POINTER(ParamsT), ctypes.POINTER(SolveOptsT), ctypes.POINTER(SolveStatsT)
    sig = {
        "gb2d_create": [G, P, ctypes.POINTER(vp)],
        "gb2d_destroy": [vp],
        "gb2d_field_extent": [G, i, ctypes.POINTER(i), ctypes.POINTER(i)],
        "gb2d_set_field": [vp, i, vp],
        "gb2d_get_field": [vp, i, vp],
        "gb2d_field_device_ptr": [vp, i, ctypes.POINTER(vp)],
        "gb2d_synchronize": [vp],
        "gb2d_levelset_advection": [vp, d],
        "gb2d_reinitialization": [vp],
        "gb2d_levelset_rk3": [vp, d],
        "gb2d_fast_sweeping": [vp, i],
        "gb2d_velocity_advection": [vp, d],
        "gb2d_curvature": [vp],
        "gb2d_projection": [vp, d, O, S],
        "gb2d_set_flow_params": [vp, ctypes.POINTER(FlowParamsT)],
        "gb2d_apply_gravity": [vp, d],
        "gb2d_sourcing": [vp, d],
        "gb2d_velocity_boundary": [vp],
        "gb2d_solve_for_rk": [vp, d, O, S],
        "gb2d_advance_time_step": [vp, d, O, S],
        "gb2d_cfl_time_step": [vp, ctypes.POINTER(d), vp],
        "gb2d_advance_frame": [vp, d, ctypes.POINTER(d), O, S],
        "gb2d_weno5_adjoint": [vp, d, vp, vp, vp, vp],
        "gb2d_projection_adjoint": [vp, d, vp, vp, vp, vp, vp, O, S],
        "gb2d_batch_create": [i, G, P, ctypes.POINTER(FlowParamsT), i, ctypes.POINTER(vp)],
        "gb2d_batch_destroy": [vp],
        "gb2d_batch_size": [vp, ctypes.POINTER(i), ctypes.POINTER(i)],
        "gb2d_batch_context": [vp, i, ctypes.POINTER(vp)],
        "gb2d_batch_autotune": [vp, d, O, vp],
        "gb2d_batch_advance": [vp, i, d, vp, O, ctypes.POINTER(BatchStatsT)],
        "gb2d_batch_run_graph": [vp, i, d, vp, O, ctypes.POINTER(BatchStatsT)],
        "gb2d_batch_schedule": [vp, i, ctypes.POINTER(i), ctypes.POINTER(i)],
        "gb2d_jump_poisson_solve": [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, O, S],
        "gb2d_projection_density_gradient": [vp, d, ctypes.POINTER(d), ctypes.POINTER(d)],
        "gb2d_projection_phi_gradient": [vp, d, vp],
        "gb2d_velocity_advection_adjoint": [vp, d, vp, vp, vp, vp],
        "gb2d_reinit_sweep_apply": [vp, vp, vp, vp],
        "gb2d_reinit_sweep_adjoint": [vp, vp, vp, vp, vp, vp],
        "gb2d_viscosity_adjoint": [vp, d, vp, vp, vp, vp, vp, vp],
        "gb2d_projection_host": [vp, d, O, vp, vp, vp, vp, vp, vp, vp, S],
        "gb2d_poisson_assemble": [vp, d, vp, vp, vp, vp],
        "gb2d_poisson_apply": [vp, vp, vp],
        "gb2d_poisson_solve": [vp, vp, vp, O, S],
        "gb2d_set_stream": [vp, vp],
        "gb2d_set_tile_plan": [vp, i],
        "gb2d_probe_enable": [vp, i],
        "gb2d_probe_read": [vp, ctypes.POINTER(i), ctypes.POINTER(d), ctypes.POINTER(d)],
        "gb2d_kernel_launches": [ctypes.POINTER(ctypes.c_ulonglong)],
        "gb2d_alu_peaks": [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
        "gb2d_solver_layout": [vp, i, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i)],
        "gb2d_preconditioner_apply": [vp, i, i, vp, vp],
        "gb2d_check_exact_division": [ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong)],
        "gb2d_checkpoint_save": [vp],
        "gb2d_checkpoint_restore": [vp],
        "gb2d_poisson_solve_noalloc": [i, i, d, d, vp, vp, vp, vp, vp, d, i, vp, ctypes.POINTER(i), ctypes.POINTER(d)],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = i
    L.gb2d_last_error.argtypes = [vp]
    L.gb2d_last_error.restype = ctypes.c_char_p
    L.gb2d_batch_last_error.argtypes = [vp]
    L.gb2d_batch_last_error.restype = ctypes.c_char_p
    _lib = L
    return L


def kernel_launches():
    """Kernels launched by libgb2d.so in this process so far."""
    n = ctypes.c_ulonglong()
    library().gb2d_kernel_launches(ctypes.byref(n))
    return n.value


def alu_peaks():
    """(FP64, FP32) FMA peaks of the current device in TFLOP/s, measured (gb2d_alu_peaks)."""
    a, b = ctypes.c_double(), ctypes.c_double()
    rc = library().gb2d_alu_peaks(ctypes.byref(a), ctypes.byref(b))
    if rc:
        raise RuntimeError(f"gb2d_alu_peaks failed ({rc})")
    return a.value, b.value


def check_exact_division(n, seed=1):
    """Mismatches of the FP64 division by 3 and 6 of the WENO5 kernels against IEEE division on 2n inputs."""
    m = ctypes.c_ulonglong()
    rc = library().gb2d_check_exact_division(n, seed, ctypes.byref(m))
    if rc != 0:
        raise GB2DError(rc, "gb2d_check_exact_division failed")
    return m.value


def _ptr(a):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("arrays must be C-contiguous float64")
    return a.ctypes.data


def solve_opts(solver=SOLVER_MGPCG, precision=PRECISION_FP64, tolerance=1e-8, max_iterations=10000, mg_smooth=2):
    return SolveOptsT(solver, precision, tolerance, max_iterations, mg_smooth)


class Context:
    """One simulation state on the GPU (a gb2d_ctx)."""

    def __init__(self, ni, nj, x_min=0.0, y_min=0.0, x_max=1.0, y_max=1.0, water_density=1000.0, air_density=1.0,
                 surface_tension=0.0728, weno_epsilon=1e-6, reinit_iterations=25, reinit_scaling=5,
                 advection_precision=PRECISION_FP64):
        self.L = library()
        self.grid = GridT(ni, nj, x_min, y_min, x_max, y_max)
        self.params = ParamsT(water_density, air_density, surface_tension, weno_epsilon, reinit_iterations,
                              reinit_scaling, advection_precision)
        h = ctypes.c_void_p()
        rc = self.L.gb2d_create(ctypes.byref(self.grid), ctypes.byref(self.params), ctypes.byref(h))
        if rc != 0:
            raise GB2DError(rc, "gb2d_create failed")
        self.h = h
        self.ni, self.nj = ni, nj

    def close(self):
        if getattr(self, "h", None):
            self.L.gb2d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise GB2DError(rc, self.L.gb2d_last_error(self.h).decode(errors="replace"))
        return rc

    def shape(self, field):
        ir, jr = ctypes.c_int(), ctypes.c_int()
        self._check(self.L.gb2d_field_extent(ctypes.byref(self.grid), field, ctypes.byref(ir), ctypes.byref(jr)))
        return (jr.value, ir.value)

    def set(self, field, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.shape != self.shape(field):
            raise ValueError(f"field {field}: expected shape {self.shape(field)}, got {a.shape}")
        self._check(self.L.gb2d_set_field(self.h, field, _ptr(a)))

    def get(self, field, out=None):
        out = np.empty(self.shape(field)) if out is None else out
        self._check(self.L.gb2d_get_field(self.h, field, _ptr(out)))
        return out

    def synchronize(self):
        self._check(self.L.gb2d_synchronize(self.h))

    def set_stream(self, stream_handle):
        """Use a caller's CUDA stream (integer cudaStream_t, e.g. torch.cuda.Stream().cuda_stream); None = own."""
        self._check(self.L.gb2d_set_stream(self.h, ctypes.c_void_p(stream_handle) if stream_handle else None))

    def set_tile_plan(self, plan):
        """Tile shape of the solver's smoothing levels: -1 the per-level rule, 0-3 one shape for all."""
        self._check(self.L.gb2d_set_tile_plan(self.h, plan))

    def device_ptr(self, field):
        p = ctypes.c_void_p()
        self._check(self.L.gb2d_field_device_ptr(self.h, field, ctypes.byref(p)))
        return p.value

    def checkpoint_save(self):
        self._check(self.L.gb2d_checkpoint_save(self.h))

    def checkpoint_restore(self):
        self._check(self.L.gb2d_checkpoint_restore(self.h))

    def probe(self, enable):
        self._check(self.L.gb2d_probe_enable(self.h, 1 if enable else 0))

    def solver_layout(self, precision):
        """(levels, first cluster-tail level or -1, cluster CTAs) of one precision's hierarchy."""
        lv, top, ctas = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self.L.gb2d_solver_layout(self.h, precision, ctypes.byref(lv), ctypes.byref(top), ctypes.byref(ctas)))
        return lv.value, top.value, ctas.value

    def preconditioner_apply(self, r, precision=PRECISION_MIXED, mg_smooth=2):
        """One V-cycle z = M r of the preconditioner of the last assembled system (r, z: (nj, ni))."""
        r = np.ascontiguousarray(r, dtype=np.float64)
        if r.shape != (self.nj, self.ni):
            raise ValueError(f"r: expected shape {(self.nj, self.ni)}, got {r.shape}")
        z = np.empty_like(r)
        self._check(self.L.gb2d_preconditioner_apply(self.h, precision, mg_smooth, _ptr(r), _ptr(z)))
        return z

    def probe_read(self):
        n, ms, by = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        self._check(self.L.gb2d_probe_read(self.h, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(by)))
        return n.value, ms.value, by.value

    # Step interface of EULERIAN_FLUID_SOLVER_2D
    def levelset_advection(self, dt):
        self._check(self.L.gb2d_levelset_advection(self.h, dt))

    def reinitialization(self):
        self._check(self.L.gb2d_reinitialization(self.h))

    def fast_sweeping(self, sweeps=4):
        """LEVELSET_2D::FastSweepingMethodOriginal(sweeps)."""
        self._check(self.L.gb2d_fast_sweeping(self.h, sweeps))

    def levelset_rk3(self, dt):
        self._check(self.L.gb2d_levelset_rk3(self.h, dt))

    def velocity_advection(self, dt):
        self._check(self.L.gb2d_velocity_advection(self.h, dt))

    def curvature(self):
        self._check(self.L.gb2d_curvature(self.h))

    def projection(self, dt, opts=None, allow_max_iters=False):
        opts = opts or solve_opts()
        st = SolveStatsT()
        rc = self.L.gb2d_projection(self.h, dt, ctypes.byref(opts), ctypes.byref(st))
        if rc != 0 and not (allow_max_iters and rc == -4):
            self._check(rc)
        return st

    def projection_host(self, dt, opts=None, phi=None, u=None, v=None, p=None, p_out=None, u_out=None, v_out=None,
                        allow_max_iters=False):
        """gb2d_projection_host: the projection with its inputs copied in from, and its outputs
        copied out to, host arrays (float64, C-contiguous, the field shapes; None = skip),
        the copies overlapping the assembly and the velocity update."""
        opts = opts or solve_opts()
        st = SolveStatsT()
        ins = []
        for f, a in ((FIELD_PHI, phi), (FIELD_U, u), (FIELD_V, v), (FIELD_P, p)):
            if a is not None:
                a = np.ascontiguousarray(a, dtype=np.float64)
                if a.shape != self.shape(f):
                    raise ValueError(f"field {f}: expected shape {self.shape(f)}, got {a.shape}")
            ins.append(a)
        for f, a in ((FIELD_P, p_out), (FIELD_U, u_out), (FIELD_V, v_out)):
            if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous or a.shape != self.shape(f)):
                raise ValueError(f"field {f}: output must be float64, C-contiguous, shape {self.shape(f)}")
        ptr = lambda a: _ptr(a) if a is not None else None
        rc = self.L.gb2d_projection_host(self.h, dt, ctypes.byref(opts), *[ptr(a) for a in ins], ptr(p_out), ptr(u_out), ptr(v_out),
                                         ctypes.byref(st))
        if rc != 0 and not (allow_max_iters and rc == -4):
            self._check(rc)
        return st

    def set_flow_params(self, water_viscosity=1.0, air_viscosity=0.0, gravity=(0.0, -9.8), viscosity=False, cfl_number=0.5):
        """Constants of SolveForRK's gravity and sourcing stages and of CFLOneTimeStep; viscosity=False is
        the reference's air/water behaviour (no viscous term), True applies VISCOSITY_2D::ApplyViscosity's
        explicit term."""
        f = FlowParamsT(water_viscosity, air_viscosity, gravity[0], gravity[1], cfl_number, int(bool(viscosity)))
        self._check(self.L.gb2d_set_flow_params(self.h, ctypes.byref(f)))

    def cfl_time_step(self):
        """CFLOneTimeStep from the current U, V and KAPPA: (dt, (c_f, g_f, v_f, s_f))."""
        dt = ctypes.c_double()
        rates = np.zeros(4)
        self._check(self.L.gb2d_cfl_time_step(self.h, ctypes.byref(dt), _ptr(rates)))
        return dt.value, tuple(float(r) for r in rates)

    def advance_frame(self, cfl=1.0, prev_dt=0.0, opts=None, allow_max_iters=False):
        """SIMULATION_WORLD::AdvanceOneFrame: curvature, CFL time step * cfl, one time step. Returns (dt, stats)."""
        opts = opts or solve_opts()
        st = SolveStatsT()
        dt = ctypes.c_double(prev_dt)
        rc = self.L.gb2d_advance_frame(self.h, cfl, ctypes.byref(dt), ctypes.byref(opts), ctypes.byref(st))
        if rc != 0 and not (allow_max_iters and rc == -4):
            self._check(rc)
        return dt.value, st

    def apply_gravity(self, dt):
        self._check(self.L.gb2d_apply_gravity(self.h, dt))

    def sourcing(self, dt):
        self._check(self.L.gb2d_sourcing(self.h, dt))

    def velocity_boundary(self):
        self._check(self.L.gb2d_velocity_boundary(self.h))

    def solve_for_rk(self, dt, opts=None, allow_max_iters=False):
        opts = opts or solve_opts()
        st = SolveStatsT()
        rc = self.L.gb2d_solve_for_rk(self.h, dt, ctypes.byref(opts), ctypes.byref(st))
        if rc != 0 and not (allow_max_iters and rc == -4):
            self._check(rc)
        return st

    def advance_time_step(self, dt, opts=None, allow_max_iters=False):
        """AdvanceOneTimeStepThread (order 3): level-set + reinit RK3, then velocity RK3 over three SolveForRK."""
        opts = opts or solve_opts()
        st = SolveStatsT()
        rc = self.L.gb2d_advance_time_step(self.h, dt, ctypes.byref(opts), ctypes.byref(st))
        if rc != 0 and not (allow_max_iters and rc == -4):
            self._check(rc)
        return st

    # Adjoints (vector-Jacobian products)
    def weno5_adjoint(self, dt, lam_phi, velocity=True):
        """VJP of one levelset_advection at the current PHI, UA, VA: (mu_phi, mu_ua, mu_va)."""
        lam = np.ascontiguousarray(lam_phi, dtype=np.float64)
        mu = np.empty(self.shape(FIELD_PHI))
        mua = np.empty(self.shape(FIELD_UA)) if velocity else None
        mva = np.empty(self.shape(FIELD_VA)) if velocity else None
        self._check(self.L.gb2d_weno5_adjoint(self.h, dt, _ptr(lam), _ptr(mu), _ptr(mua) if velocity else None,
                                              _ptr(mva) if velocity else None))
        return mu, mua, mva

    def projection_adjoint(self, dt, lam_u, lam_v, lam_p=None, opts=None, allow_max_iters=False):
        """VJP of the last projection with respect to its intermediate velocity: (mu_u, mu_v, stats)."""
        lu = np.ascontiguousarray(lam_u, dtype=np.float64)
        lv = np.ascontiguousarray(lam_v, dtype=np.float64)
        lp = None if lam_p is None else np.ascontiguousarray(lam_p, dtype=np.float64)
        mu, mv = np.empty(self.shape(FIELD_U)), np.empty(self.shape(FIELD_V))
        opts = opts or solve_opts(tolerance=1e-12)
        st = SolveStatsT()
        rc = self.L.gb2d_projection_adjoint(self.h, dt, _ptr(lu), _ptr(lv), None if lp is None else _ptr(lp), _ptr(mu), _ptr(mv),
                                            ctypes.byref(opts), ctypes.byref(st))
        if rc != 0 and not (allow_max_iters and rc == -4):
            self._check(rc)
        return mu, mv, st

    def jump_poisson_solve(self, density, bc, div, levelset, jc_solution, jc_derivative, pressure, opts=None,
                           allow_max_iters=False):
        """General jump-condition Poisson problem (POISSON_SOLVER::Solve with jumps): returns
        (solution, normal_x, normal_y, stats); pressure carries the Dirichlet values and warm start."""
        f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        d, dv, ls, js, jd = f(density), f(div), f(levelset), f(jc_solution), f(jc_derivative)
        bci = np.ascontiguousarray(bc, dtype=np.int32)
        p = f(pressure).copy()
        nx, ny = np.zeros_like(p), np.zeros_like(p)
        opts = opts or solve_opts(tolerance=1e-10)
        st = SolveStatsT()
        rc = self.L.gb2d_jump_poisson_solve(self.h, _ptr(d), bci.ctypes.data, _ptr(dv), _ptr(ls), _ptr(js), _ptr(jd), _ptr(p),
                                            _ptr(nx), _ptr(ny), ctypes.byref(opts), ctypes.byref(st))
        if rc != 0 and not (allow_max_iters and rc == -4):
            self._check(rc)
        return p, nx, ny, st

    def projection_density_gradient(self, dt):
        """(dL/d water_density, dL/d air_density) of the loss of the last projection_adjoint call."""
        w, a = ctypes.c_double(), ctypes.c_double()
        self._check(self.L.gb2d_projection_density_gradient(self.h, dt, ctypes.byref(w), ctypes.byref(a)))
        return w.value, a.value

    def velocity_advection_adjoint(self, dt, lam_u, lam_v):
        """VJP of the last velocity_advection: (mu_ua, mu_va), the cotangents of the advecting
        copies UA, VA (gb2d_velocity_advection_adjoint)."""
        lam_u = np.ascontiguousarray(lam_u, dtype=np.float64)
        lam_v = np.ascontiguousarray(lam_v, dtype=np.float64)
        mu_ua, mu_va = np.zeros(self.shape(FIELD_UA)), np.zeros(self.shape(FIELD_VA))
        self._check(self.L.gb2d_velocity_advection_adjoint(self.h, dt, _ptr(lam_u), _ptr(lam_v), _ptr(mu_ua), _ptr(mu_va)))
        return mu_ua, mu_va

    def reinit_sweep(self, phi, sign):
        """One reinitialisation sweep of phi with S = sign (gb2d_reinit_sweep_apply)."""
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        sign = np.ascontiguousarray(sign, dtype=np.float64)
        out = np.empty(self.shape(FIELD_PHI))
        self._check(self.L.gb2d_reinit_sweep_apply(self.h, _ptr(phi), _ptr(sign), _ptr(out)))
        return out

    def reinit_sweep_adjoint(self, phi, sign, lam):
        """VJP of reinit_sweep at (phi, sign): (mu_phi, mu_sign) (gb2d_reinit_sweep_adjoint)."""
        phi, sign, lam = (np.ascontiguousarray(x, dtype=np.float64) for x in (phi, sign, lam))
        mu, ms = np.empty(self.shape(FIELD_PHI)), np.empty((self.nj, self.ni))
        self._check(self.L.gb2d_reinit_sweep_adjoint(self.h, _ptr(phi), _ptr(sign), _ptr(lam), _ptr(mu), _ptr(ms)))
        return mu, ms

    def viscosity_adjoint(self, dt, lam_u, lam_v):
        """VJP of the sourcing's viscosity at the context's PHI, U, V:
        (mu_u, mu_v, mu_phi, (dL/d water_density, dL/d air_density))."""
        lu, lv = (np.ascontiguousarray(x, dtype=np.float64) for x in (lam_u, lam_v))
        mu, mv, mp = np.empty(self.shape(FIELD_U)), np.empty(self.shape(FIELD_V)), np.empty(self.shape(FIELD_PHI))
        dd = np.empty(2)
        self._check(self.L.gb2d_viscosity_adjoint(self.h, dt, _ptr(lu), _ptr(lv), _ptr(mu), _ptr(mv), _ptr(mp), _ptr(dd)))
        return mu, mv, mp, (float(dd[0]), float(dd[1]))

    def projection_phi_gradient(self, dt):
        """dL/dphi (PHI's shape) of the loss of the last projection_adjoint (gb2d_projection_phi_gradient)."""
        out = np.zeros(self.shape(FIELD_PHI))
        self._check(self.L.gb2d_projection_phi_gradient(self.h, dt, _ptr(out)))
        return out

    # Pressure system (a10/a15)

    def poisson_assemble(self, dt):
        ni, nj = self.ni, self.nj
        bx, by = np.zeros((nj, ni + 1)), np.zeros((nj + 1, ni))
        dg, rhs = np.zeros((nj, ni)), np.zeros((nj, ni))
        self._check(self.L.gb2d_poisson_assemble(self.h, dt, _ptr(bx), _ptr(by), _ptr(dg), _ptr(rhs)))
        return bx, by, dg, rhs

    def poisson_apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self._check(self.L.gb2d_poisson_apply(self.h, _ptr(x), _ptr(y)))
        return y

    def poisson_solve(self, rhs, x0=None, opts=None, allow_max_iters=False):
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        x = np.zeros_like(rhs) if x0 is None else np.ascontiguousarray(x0, dtype=np.float64).copy()
        opts = opts or solve_opts()
        st = SolveStatsT()
        rc = self.L.gb2d_poisson_solve(self.h, _ptr(rhs), _ptr(x), ctypes.byref(opts), ctypes.byref(st))
        if rc != 0 and not (allow_max_iters and rc == -4):
            self._check(rc)
        return x, st


class _View(Context):
    """A context owned by a Batch (not destroyed by Python)."""

    def __init__(self, L, h, ni, nj, grid):
        self.L, self.h, self.ni, self.nj, self.grid = L, h, ni, nj, grid

    def close(self):
        self.h = None


class Batch:
    """Independent simulations of uneven sizes advanced together (gb2d_batch_*)."""

    def __init__(self, sizes, params=None, flows=None, workers=0):
        """sizes: list of (ni, nj, x_max, y_max) on [0, x_max] x [0, y_max]; params / flows: per-instance
        dicts for Context's keyword arguments / set_flow_params (or one dict for all)."""
        self.L = library()
        n = len(sizes)
        G = (GridT * n)(*[GridT(ni, nj, 0.0, 0.0, xm, ym) for ni, nj, xm, ym in sizes])

        def each(x, k):
            return (x[k] if isinstance(x, (list, tuple)) else x) or {}

        P = (ParamsT * n)()
        F = (FlowParamsT * n)()
        for k in range(n):
            p = dict(water_density=1000.0, air_density=1.0, surface_tension=0.0728, weno_epsilon=1e-6,
                     reinit_iterations=25, reinit_scaling=5, advection_precision=PRECISION_MIXED)
            p.update(each(params, k))
            P[k] = ParamsT(p["water_density"], p["air_density"], p["surface_tension"], p["weno_epsilon"],
                           p["reinit_iterations"], p["reinit_scaling"], p["advection_precision"])
            f = dict(water_viscosity=1.0, air_viscosity=0.0, gravity=(0.0, -9.8), cfl_number=0.5, viscosity=False)
            f.update(each(flows, k))
            F[k] = FlowParamsT(f["water_viscosity"], f["air_viscosity"], f["gravity"][0], f["gravity"][1], f["cfl_number"],
                               int(bool(f["viscosity"])))
        h = ctypes.c_void_p()
        rc = self.L.gb2d_batch_create(n, G, P, F, workers, ctypes.byref(h))
        if rc != 0:
            raise GB2DError(rc, "gb2d_batch_create failed")
        self.h, self.n, self.sizes, self.grids = h, n, sizes, G
        nn, w = ctypes.c_int(), ctypes.c_int()
        self.L.gb2d_batch_size(self.h, ctypes.byref(nn), ctypes.byref(w))
        self.workers = w.value

    def _check(self, rc):
        if rc != 0:
            raise GB2DError(rc, self.L.gb2d_batch_last_error(self.h).decode(errors="replace"))

    def context(self, k):
        c = ctypes.c_void_p()
        self._check(self.L.gb2d_batch_context(self.h, k, ctypes.byref(c)))
        ni, nj = self.sizes[k][0], self.sizes[k][1]
        return _View(self.L, c, ni, nj, self.grids[k])

    def autotune(self, cfl=1.0, opts=None):
        opts = opts or solve_opts(precision=PRECISION_MIXED)
        out = (ctypes.c_int * self.n)()
        self._check(self.L.gb2d_batch_autotune(self.h, cfl, ctypes.byref(opts), out))
        return list(out)

    def advance(self, frames, cfl=1.0, dts=None, opts=None, allow_max_iters=False):
        opts = opts or solve_opts(precision=PRECISION_MIXED)
        dts = np.zeros(self.n) if dts is None else np.ascontiguousarray(dts, dtype=np.float64)
        st = BatchStatsT()
        rc = self.L.gb2d_batch_advance(self.h, frames, cfl, _ptr(dts), ctypes.byref(opts), ctypes.byref(st))
        if rc != 0 and not (allow_max_iters and rc == -4):
            self._check(rc)
        return dts, st

    def run_graph(self, frames, cfl=1.0, dts=None, opts=None, allow_max_iters=False):
        """advance() as one graph launch (gb2d_batch_run_graph)."""
        opts = opts or solve_opts(precision=PRECISION_MIXED)
        dts = np.zeros(self.n) if dts is None else np.ascontiguousarray(dts, dtype=np.float64)
        st = BatchStatsT()
        rc = self.L.gb2d_batch_run_graph(self.h, frames, cfl, _ptr(dts), ctypes.byref(opts), ctypes.byref(st))
        if rc != 0 and not (allow_max_iters and rc == -4):
            self._check(rc)
        return dts, st

    def schedule(self, k):
        """(sweeps, tile plan) of instance k (gb2d_batch_schedule)."""
        sw, tp = ctypes.c_int(), ctypes.c_int()
        self._check(self.L.gb2d_batch_schedule(self.h, k, ctypes.byref(sw), ctypes.byref(tp)))
        return sw.value, tp.value

    def close(self):
        if getattr(self, "h", None):
            self.L.gb2d_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
