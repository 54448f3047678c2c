"""Batches of independent rising bubbles of uneven sizes (gb2d_batch_*): the instances
advanced together by worker threads give the same bits as the same instances advanced
one by one, and the autotuner's choices are valid sweep counts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(32, 32), (48, 48), (64, 64), (40, 56), (64, 96), (33, 33)]


def bubble_phi(ni, nj, y_max, cy, r):
    """Signed distance to a circle at (0.5, cy) on [0,1] x [0,y_max] with dx = dy, ghosts copied
    from the second interior line and corners at dx, as the .sim driver builds it."""
    dx = 1.0 / (ni - 1)
    phi = np.full((nj + 4, ni + 4), dx)
    x = np.arange(ni) * dx
    y = np.arange(nj) * (y_max / (nj - 1))
    X, Y = np.meshgrid(x, y)
    phi[2:2 + nj, 2:2 + ni] = np.sqrt((X - 0.5) ** 2 + (Y - cy) ** 2) - r
    phi[2:2 + nj, 0:2] = phi[2:2 + nj, 3:4]
    phi[2:2 + nj, 2 + ni:] = phi[2:2 + nj, ni:ni + 1]
    phi[0:2, 2:2 + ni] = phi[3:4, 2:2 + ni]
    phi[2 + nj:, 2:2 + ni] = phi[nj:nj + 1, 2:2 + ni]
    return phi


def setup():
    rng = np.random.default_rng(21)
    sizes, phis, params = [], [], []
    for ni, nj in SIZES:
        y_max = (nj - 1) / (ni - 1)
        sizes.append((ni, nj, 1.0, y_max))
        phis.append(bubble_phi(ni, nj, y_max, rng.uniform(0.2, 0.4), rng.uniform(0.1, 0.2)))
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
