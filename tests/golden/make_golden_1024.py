"""Generate tests/golden/projection_1024.npz: the reference's own projection of the
1024^2 benchmark workload (the standalone-projection case of tests/golden/cases.py with
seed 0: 8 circles, rho 1:1000, sigma 0.0728, dt = 0.5 dx, zero initial pressure).

The reference (oracle/_ref/libref2d.so, built from its sources by oracle/ref/Makefile)
runs PROJECTION_2D::Solve with PCG-IC(0).  Its stop test is absolute (r.z below the
square of its tolerance, PCG_METHOD.cpp:254), so the iteration count is taken from the
oracle, which reproduces the reference's iterates bit for bit: the oracle stops where
its recursive residual reaches 1e-14 of ||b|| (4348 iterations), and the reference is
run for exactly that many (tolerance 0, max_iteration = count - 1); the two pressures
are checked to be bit-identical here.  The same projection is then repeated from the
reference's own pressure as warm start (PROJECTION_2D.h:974 takes the previous p), again
for the oracle's count (2449).  Both pressures have a true residual ||b - A p|| / ||b||
of about 4e-11, the floor of FP64 arithmetic on this system, and they differ by about
1.1e-10 relative: the reference's own noise floor at this size.

Stored (the fields are subsampled to keep the fixture small; the relative L2 over the
sampled nodes estimates the one over all nodes): p (first solve), p_resolve (second
solve), u, v after the first solve, every 4th node from node 1 in each direction (p:
256 x 256 samples), with 12 low mantissa bits dropped (relative change < 4e-13); the
full-field norms and the iteration counts and true residuals.

Usage:  python tests/golden/make_golden_1024.py   (needs the reference sources; ~10 min)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle2d  # noqa: E402
import refsim as R  # noqa: E402
from tests.golden.cases import bubbles_case  # noqa: E402

N = 1024
STRIDE = 4
DROP_BITS = 12


def sample(a):
    """Every STRIDE-th entry of a ghost-inclusive array in both directions, from index 1."""
    return np.ascontiguousarray(a[1::STRIDE, 1::STRIDE])


def drop_bits(a):
    u = np.ascontiguousarray(a).view(np.uint64).copy()
    u &= ~np.uint64((1 << DROP_BITS) - 1)
    return u.view(np.float64)


def true_residual(case, p, dt):
    g = oracle2d.grid(N, N)
    phi, kap = case["phi"].copy(), np.zeros((N, N))
    oracle2d.curvature(g, phi, kap)
    bx, by, dg, rhs = oracle2d.poisson_assemble(g, oracle2d.params(), phi, case["u"], case["v"], kap, dt)
    r = rhs - oracle2d.poisson_apply(g, bx, by, dg, np.ascontiguousarray(p[1:-1, 1:-1]))
    return float(np.linalg.norm(r) / np.linalg.norm(rhs))


def main():
    if not R.available():
        sys.exit("oracle/_ref/libref2d.so missing: run `make -C oracle/ref` where the reference sources are present")
    oracle2d.build()
    case = bubbles_case(N, seed=0)
    dt = 0.5 / (N - 1)
    g = oracle2d.grid(N, N)
    pr = oracle2d.params(pcg_tolerance=0.0, pcg_max_iterations=20000, pcg_rel_residual=1e-14)
    phi, u, v, p = case["phi"].copy(), case["u"].copy(), case["v"].copy(), case["p"].copy()
    st1 = oracle2d.projection(g, pr, phi, u, v, p, np.zeros((N, N)), dt)
    p_or1 = p.copy()
    st2 = oracle2d.projection(g, pr, phi, case["u"].copy(), case["v"].copy(), p, np.zeros((N, N)), dt)
    p_or2 = p.copy()

    def ref_solve(p0, iterations):
        s = R.RefSim(N, N, 0.0, 0.0, 1.0, 1.0, water_density=1000.0, air_density=1.0, surface_tension=0.0728,
                     pcg_tolerance=0.0, pcg_max_iterations=iterations - 1)
        s.set(R.PHI, case["phi"]); s.set(R.U, case["u"]); s.set(R.V, case["v"]); s.set(R.P, p0)
        s.projection(dt)
        out = s.get(R.P), s.get(R.U), s.get(R.V), s.pcg_info()[0]
        s.close()
        return out

    p1, u1, v1, it1 = ref_solve(case["p"], st1.iterations)
    p2, _, _, it2 = ref_solve(p1, st2.iterations)
    assert it1 == st1.iterations and it2 == st2.iterations
    assert np.array_equal(p1, p_or1) and np.array_equal(p2, p_or2), "oracle and reference differ at 1024^2"
    out = dict(n=N, stride=STRIDE, dt=dt, seed=0, iterations=it1, iterations_resolve=it2,
               true_residual=true_residual(case, p1, dt), true_residual_resolve=true_residual(case, p2, dt),
               p=drop_bits(sample(p1)), p_resolve=drop_bits(sample(p2)), u=drop_bits(sample(u1)), v=drop_bits(sample(v1)),
               norm_p=float(np.linalg.norm(p1[1:-1, 1:-1])), norm_u=float(np.linalg.norm(u1)), norm_v=float(np.linalg.norm(v1)),
               resolve_rel_l2_p=float(np.linalg.norm(p2 - p1) / np.linalg.norm(p1)))
    path = os.path.join(HERE, "projection_1024.npz")
    np.savez_compressed(path, **out)
    print(f"projection_1024: {os.path.getsize(path) / 1024:.0f} KiB, PCG {it1} + {it2} iterations, true residuals "
          f"{out['true_residual']:.2e} / {out['true_residual_resolve']:.2e}, re-solve moves p by {out['resolve_rel_l2_p']:.2e}")


if __name__ == "__main__":
    main()
