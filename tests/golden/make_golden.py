"""Generate the golden fixtures in tests/golden/*.npz from the reference itself.

Runs the headless build of the reference solver (oracle/_ref/libref2d.so, made by
`make -C oracle/ref` from the reference sources) on the seeded inputs of
tests/golden/cases.py and stores inputs and outputs:

  levelset_advection  one Levelset_Advection (WENO5 + ghost extrapolation)
  reinitialization    one Reinitialization (25 WENO5-Godunov sweeps)
  levelset_rk3        TVD-RK3 of Levelset_Advection then of Reinitialization,
                      composed here exactly as EULERIAN_FLUID_SOLVER_2D.h:1694-1741
  velocity_advection  one Velocity_Advection (ENO3 on both MAC components)
  curvature           ComputeCurvaturesThread
  projection          PROJECTION_2D::Solve(dt) with PCG-IC(0) at a tight tolerance,
                      plus the assembled CSR system and A*x for a seeded x
  gravity / sourcing / velocity_bc
                      ApplyGraivity, Sourcing (DetermineDensity and, with the
                      viscosity solver configured, ApplyViscosity) and
                      SetupBoundaryConditionForVelocity applied in turn
  solve_for_rk        one SolveForRK stage (viscosity configured)
  time_step           AdvanceOneTimeStepThread (order 3), without viscosity (the
                      reference's air/water setup) and with it configured
  cfl                 CFLOneTimeStep after ComputeCurvaturesThread
  fast sweeping       FastSweepingMethodOriginal with 1 and 4 sweeps
and, in rising_bubble_128_frames.npz, 100 frames of the 128^2 rising bubble
(SIMULATION_WORLD::AdvanceOneFrame: curvature, CFL time step, time step); in
poisson_test{3,5,8}_61.npz, POISSON_EQUATION_TEST's jump-condition problems 3, 5 and 8.

Usage:  python tests/golden/make_golden.py [name ...]   (needs the reference sources)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))

import refsim as R  # noqa: E402
from tests.golden.cases import bubbles_case, rising_bubble_case  # noqa: E402

PHYS = dict(water_density=1000.0, air_density=1.0, surface_tension=0.0728)
FLOW = dict(water_viscosity=1.0, air_viscosity=0.01, gravity=(0.0, -9.8))


def csr_apply(rp, col, val, x):
    y = np.zeros(len(rp) - 1)
    for row in range(len(rp) - 1):
        acc = 0.0
        for k in range(rp[row], rp[row + 1]):
            acc += val[k] * x[col[k]]
        y[row] = acc
    return y


def make_case(name, c, dt, pcg_tolerance, flow=True):
    ni, nj, xm, ym = c["ni"], c["nj"], c["x_max"], c["y_max"]
    out = {k: np.asarray(c[k]) for k in ("phi", "u", "v", "ua", "va", "p")}
    out.update(ni=ni, nj=nj, x_max=xm, y_max=ym, dt=dt, pcg_tolerance=pcg_tolerance)
    mk = lambda **kw: R.RefSim(ni, nj, 0.0, 0.0, xm, ym, **PHYS, **kw)

    s = mk()
    s.set(R.PHI, c["phi"]); s.set(R.UA, c["ua"]); s.set(R.VA, c["va"])
    s.levelset_advection(dt)
    out["la_phi"] = s.get(R.PHI)
    s.reinitialization(dt)
    out["reinit_phi"] = s.get(R.PHI)
    s.close()

    for sweeps in (1, 4):
        s = mk()
        s.set(R.PHI, c["phi"])
        s.fast_sweeping(sweeps)
        out[f"fsm{sweeps}_phi"] = s.get(R.PHI)
        s.close()

    s = mk()
    s.set(R.PHI, c["phi"]); s.set(R.UA, c["ua"]); s.set(R.VA, c["va"])
    interior = (slice(2, 2 + nj), slice(2, 2 + ni))
    t = s.get(R.PHI)[interior].copy()
    s.levelset_advection(dt); s.levelset_advection(dt)
    a = s.get(R.PHI); a[interior] = 0.75 * t + 0.25 * a[interior]; s.set(R.PHI, a)
    s.levelset_advection(dt)
    a = s.get(R.PHI); a[interior] = (1 / 3.0) * t + (2 / 3.0) * a[interior]; s.set(R.PHI, a)
    t = s.get(R.PHI)[interior].copy()
    s.reinitialization(dt); s.reinitialization(dt)
    a = s.get(R.PHI); a[interior] = 0.75 * t + 0.25 * a[interior]; s.set(R.PHI, a)
    s.reinitialization(dt)
    a = s.get(R.PHI); a[interior] = (1 / 3.0) * t + (2 / 3.0) * a[interior]; s.set(R.PHI, a)
    out["rk3_phi"] = s.get(R.PHI)
    s.close()

    s = mk()
    s.set(R.U, c["u"]); s.set(R.V, c["v"]); s.set(R.UA, c["ua"]); s.set(R.VA, c["va"])
    s.velocity_advection(dt)
    out["va_u"], out["va_v"], out["va_ua"], out["va_va"] = s.get(R.U), s.get(R.V), s.get(R.UA), s.get(R.VA)
    s.close()

    s = mk()
    s.set(R.PHI, c["phi"]); s.curvature()
    out["curv_kappa"], out["curv_phi"] = s.get(R.KAPPA), s.get(R.PHI)
    s.close()
    if flow:
        s = R.RefSim(ni, nj, 0.0, 0.0, xm, ym, **PHYS, **FLOW)
        s.set(R.PHI, c["phi"]); s.set(R.U, c["u"]); s.set(R.V, c["v"]); s.curvature()
        out["cfl_dt"] = s.cfl_dt()
        s.close()

    s = mk(pcg_tolerance=pcg_tolerance, pcg_max_iterations=200000)
    s.set(R.PHI, c["phi"]); s.set(R.U, c["u"]); s.set(R.V, c["v"]); s.set(R.P, c["p"])
    s.projection(dt)
    out["proj_p"], out["proj_u"], out["proj_v"] = s.get(R.P), s.get(R.U), s.get(R.V)
    out["proj_phi"], out["proj_kappa"] = s.get(R.PHI), s.get(R.KAPPA)
    it, res = s.pcg_info()
    out["proj_iterations"], out["proj_residual"] = it, res
    rp, col, val, b, x = s.poisson_system()
    out["sys_b"] = b
    xr = np.random.default_rng(12345).standard_normal(ni * nj)
    out["sys_x"] = xr
    out["sys_ax"] = csr_apply(rp, col, val, xr)
    out["sys_diag"] = np.array([val[rp[r + 1] - 1] for r in range(ni * nj)])
    s.close()
    if flow:
        make_flow(out, c, dt, pcg_tolerance)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB, PCG {it} iterations, residual {res:.3e}")


def make_flow(out, c, dt, pcg_tolerance):
    """The SolveForRK stages around the projection and the whole order-3 time step."""
    ni, nj, xm, ym = c["ni"], c["nj"], c["x_max"], c["y_max"]
    mk = lambda: R.RefSim(ni, nj, 0.0, 0.0, xm, ym, **PHYS, **FLOW, pcg_tolerance=pcg_tolerance, pcg_max_iterations=200000)

    def load(s):
        for f, k in ((R.PHI, "phi"), (R.U, "u"), (R.V, "v"), (R.UA, "ua"), (R.VA, "va"), (R.P, "p")):
            s.set(f, c[k])

    # gravity -> sourcing (with and without viscosity) -> wall conditions, from the same start
    for visc in (0, 1):
        s = mk(); s.configure_viscosity(visc); load(s)
        s.apply_gravity(dt)
        out["grav_u"], out["grav_v"] = s.get(R.U), s.get(R.V)
        s.sourcing(dt)
        out[f"src{visc}_u"], out[f"src{visc}_v"], out[f"src{visc}_density"] = s.get(R.U), s.get(R.V), s.get(R.DENSITY)
        s.velocity_bc()
        out[f"bc{visc}_u"], out[f"bc{visc}_v"] = s.get(R.U), s.get(R.V)
        s.close()
    s = mk(); s.configure_viscosity(1); load(s)
    s.solve_for_rk(dt)
    for f, k in ((R.PHI, "phi"), (R.U, "u"), (R.V, "v"), (R.UA, "ua"), (R.VA, "va"), (R.P, "p"), (R.KAPPA, "kappa")):
        out["rk_" + k] = s.get(f)
    s.close()
    for visc in (0, 1):
        s = mk(); s.configure_viscosity(visc); load(s)
        s.step(dt)
        for f, k in ((R.PHI, "phi"), (R.U, "u"), (R.V, "v"), (R.UA, "ua"), (R.VA, "va"), (R.P, "p"),
                     (R.DENSITY, "density")):
            out[f"step{visc}_{k}"] = s.get(f)
        s.close()


def make_rising_bubble_run(name, n=128, steps=100, keep=(10,)):
    """The rising bubble on [0,1]^2 run by the reference itself, frame by frame as
    SIMULATION_WORLD::AdvanceOneFrame does (curvature, dt = CFLOneTimeStep() * CFL with
    CFL = 1, AdvanceOneTimeStepThread): bubble of radius 0.15 at (0.5, 0.3), rho 1 / 1000,
    sigma 0.0728, gravity -9.8, cfl_number 0.5, reinitialisation every step.  The initial
    level set is built as SIMULATION_WORLD.h:408-415 builds its bubbles: interior values,
    ghosts copied from the second interior line, corners left at the solver's init."""
    s = R.RefSim(n, n, 0.0, 0.0, 1.0, 1.0, **PHYS, **FLOW, pcg_tolerance=1e-13, pcg_max_iterations=200000, cfl_number=0.5)
    phi = s.get(R.PHI)
    x = np.arange(n) / (n - 1.0)
    X, Y = np.meshgrid(x, x)
    phi[2:2 + n, 2:2 + n] = np.sqrt((X - 0.5) ** 2 + (Y - 0.3) ** 2) - 0.15
    phi[2:2 + n, 0:2] = phi[2:2 + n, 3:4]            # FillGhostCellsFrom: second interior line
    phi[2:2 + n, 2 + n:] = phi[2:2 + n, n:n + 1]
    phi[0:2, 2:2 + n] = phi[3:4, 2:2 + n]
    phi[2 + n:, 2:2 + n] = phi[n:n + 1, 2:2 + n]
    s.set(R.PHI, phi)
    out = dict(phi0=phi.copy(), n=n, steps=steps, pcg_tolerance=1e-13)
    dts = []
    for k in range(1, steps + 1):
        s.curvature()
        dt = s.cfl_dt() * 1.0
        dts.append(dt)
        s.step(dt)
        if k in keep or k == steps:
            for f, key in ((R.PHI, "phi"), (R.U, "u"), (R.V, "v"), (R.P, "p")):
                out[f"{key}{k}"] = s.get(f)
    out["dts"] = np.array(dts)
    s.close()
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB, dt {dts[0]:.3e} .. {dts[-1]:.3e}")


def make_poisson_test(name, test_number, n):
    """POISSON_EQUATION_TEST of the reference (test 3: circle of radius 0.25 at (0.5, 0.5),
    beta 0.5 / 1, both jumps; test 5: circle of radius 0.5, flux jump 2) on [-1,1]^2 with
    n x n nodes and Dirichlet boundaries: inputs as the solver sees them, its system (b,
    A x for a seeded x), the solution and, for test 3, its L2 error against the exact one."""
    p = R.RefPoissonTest(test_number, n)
    l2 = p.solve()
    out = {k: p.get(k) for k in R.RefPoissonTest.FIELDS}
    rp, col, val, b, its = p.system()
    x = np.random.default_rng(777).standard_normal(len(b))
    out.update(n=n, test_number=test_number, l2_norm=l2, iterations=its, sys_b=b, sys_x=x, sys_ax=csr_apply(rp, col, val, x))
    # the solver's input pressure: Dirichlet values on the non-unknown nodes, zero elsewhere
    out["pressure_in"] = np.where(out["bc"] >= 0, 0.0, out["solution"])
    p.close()
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB, CG {its} iterations, L2 error {l2:.3e}")


FIXTURES = {
    "bubbles_17": lambda: make_case("bubbles_17", bubbles_case(17, seed=1), 0.5 / 16, 1e-13),
    "bubbles_33": lambda: make_case("bubbles_33", bubbles_case(33, seed=2), 0.5 / 32, 1e-13),
    "rising_bubble_40x24": lambda: make_case("rising_bubble_40x24", rising_bubble_case(40, 24, seed=3), 0.01, 1e-13),
    "tall_24x40": lambda: make_case("tall_24x40", bubbles_case(24, 40, seed=4, x_max=1.0, y_max=2.0), 0.02, 1e-13),
    "bubbles_65": lambda: make_case("bubbles_65", bubbles_case(65, seed=5), 0.5 / 64, 1e-12, flow=False),
    "rising_bubble_128_frames": lambda: make_rising_bubble_run("rising_bubble_128_frames"),
    "poisson_test3_61": lambda: make_poisson_test("poisson_test3_61", 3, 61),
    "poisson_test5_61": lambda: make_poisson_test("poisson_test5_61", 5, 61),
    "poisson_test8_61": lambda: make_poisson_test("poisson_test8_61", 8, 61),
}


def main():
    """python tests/golden/make_golden.py [name ...]: the named fixtures, or all of them."""
    if not R.available():
        sys.exit("oracle/_ref/libref2d.so missing: run `make -C oracle/ref` where the reference sources are present")
    for name in sys.argv[1:] or list(FIXTURES):
        FIXTURES[name]()


if __name__ == "__main__":
    main()
