"""Child process of tests/test_gpu_stream.py: one preconditioner V-cycle z = M r per
case, written to an .npz.  The smoothing kernels are chosen by the GB2D_SMOOTHER and
GB2D_CLUSTER_TAIL environment variables, which the library reads once per process.

  python -m tests.vcycle_child OUT.npz"""
import importlib
import sys

import numpy as np

from tests.golden.cases import bubbles_case

# (ni, nj): even and odd row lengths, partial strips and segments, one 1024^2 case.  On
# [0,1]^2 every case has dy >= dx: with dy < dx the reference's dx-only diagonal
# (POISSON_SOLVER.cpp:872) falls below the y-face conductances and the system is
# indefinite, which a V-cycle with a dense coarse inverse does not survive.
CASES = [(300, 200), (301, 257), (515, 513), (1024, 1024)]


def main(out):
    gb = importlib.import_module("2d_engine_gb300")
    res = {}
    for ni, nj in CASES:
        case = bubbles_case(ni, nj, seed=ni + nj)
        c = gb.Context(ni, nj)
        for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v")):
            c.set(f, case[k])
        _, _, _, rhs = c.poisson_assemble(0.5 / (ni - 1))
        r = rhs + np.random.default_rng(ni * nj).standard_normal(rhs.shape) * np.abs(rhs).max() * 1e-3
        for prec in (gb.PRECISION_FP64, gb.PRECISION_MIXED):
            for nu in (1, 2, 3):
                res[f"{ni}x{nj}_p{prec}_nu{nu}"] = c.preconditioner_apply(r, prec, nu)
        res[f"{ni}x{nj}_layout"] = np.array(c.solver_layout(gb.PRECISION_MIXED) + c.solver_layout(gb.PRECISION_FP64))
        c.close()
    np.savez(out, **res)


if __name__ == "__main__":
    main(sys.argv[1])
