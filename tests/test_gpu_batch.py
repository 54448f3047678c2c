"""Batches of independent rising bubbles of uneven sizes (gb2d_batch_*): the instances
advanced together by worker threads give the same bits as the same instances advanced
one by one, and the autotuner's choices are valid sweep counts."""
import numpy as np
import pytest

from tests.golden.cases import bubble_level_set

pytestmark = pytest.mark.gpu

SIZES = [(32, 32), (48, 48), (64, 64), (40, 56), (64, 96), (33, 33)]


def setup():
    rng = np.random.default_rng(21)
    sizes, phis, params = [], [], []
    for ni, nj in SIZES:
        y_max = (nj - 1) / (ni - 1)
        sizes.append((ni, nj, 1.0, y_max))
        phis.append(bubble_level_set(ni, nj, y_max, 0.5, rng.uniform(0.2, 0.4), rng.uniform(0.1, 0.2)))
        params.append(dict(water_density=float(np.exp(rng.uniform(np.log(10), np.log(1000))))))
    return sizes, phis, params


def test_batch_equals_instances_one_by_one(gb):
    sizes, phis, params = setup()
    flows = dict(water_viscosity=1.0, air_viscosity=0.01, viscosity=True)
    b = gb.Batch(sizes, params=params, flows=flows, workers=3)
    for k in range(len(sizes)):
        b.context(k).set(gb.FIELD_PHI, phis[k])
    opts = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=1e-8)
    smooth = b.autotune(cfl=1.0, opts=opts)
    assert all(s in (1, 2, 3) for s in smooth)
    dts, st = b.advance(3, cfl=1.0, opts=opts)
    assert st.frames == 3 and st.instances == len(sizes) and st.max_rel_residual <= 1e-8 and st.cell_frames_per_s > 0
    for k, (ni, nj, xm, ym) in enumerate(sizes):
        p = dict(advection_precision=gb.PRECISION_MIXED, water_density=params[k]["water_density"])
        c = gb.Context(ni, nj, 0.0, 0.0, xm, ym, **p)
        c.set_flow_params(**flows)
        c.set(gb.FIELD_PHI, phis[k])
        dt = 0.0
        o = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=1e-8, mg_smooth=smooth[k])
        for _ in range(3):
            dt, _ = c.advance_frame(cfl=1.0, prev_dt=dt, opts=o)
        assert dt == dts[k]
        v = b.context(k)
        for f in (gb.FIELD_PHI, gb.FIELD_U, gb.FIELD_V, gb.FIELD_P):
            np.testing.assert_array_equal(v.get(f), c.get(f))
        c.close()
    b.close()
