"""Batches of independent rising bubbles of uneven sizes (gb2d_batch_*): the instances
advanced together by worker threads give the same bits as the same instances advanced
one by one under the same tuned schedules, the whole run as one graph launch
(gb2d_batch_run_graph) gives the same bits again, and the autotuner's choices are valid
schedules."""
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
    plans = [b.schedule(k)[1] for k in range(len(sizes))]
    assert [b.schedule(k)[0] for k in range(len(sizes))] == smooth and all(p in (-1, 0, 1, 2) for p in plans)
    dts, st = b.advance(3, cfl=1.0, opts=opts)
    assert st.frames == 3 and st.instances == len(sizes) and st.max_rel_residual <= 1e-8 and st.cell_frames_per_s > 0
    for k, (ni, nj, xm, ym) in enumerate(sizes):
        p = dict(advection_precision=gb.PRECISION_MIXED, water_density=params[k]["water_density"])
        c = gb.Context(ni, nj, 0.0, 0.0, xm, ym, **p)
        c.set_flow_params(**flows)
        c.set_tile_plan(plans[k])
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


def _batch(gb, sizes, phis, params, flows):
    b = gb.Batch(sizes, params=params, flows=flows, workers=3)
    for k in range(len(sizes)):
        b.context(k).set(gb.FIELD_PHI, phis[k])
    return b


def test_graph_run_equals_host_driven_batch(gb):
    """One graph launch per run (the frames of every instance, each CG solve a device loop)
    against worker threads driving the same frames: same fields, time steps and CG
    iterations, bit for bit; a second run continues from the first run's state."""
    sizes, phis, params = setup()
    flows = dict(water_viscosity=1.0, air_viscosity=0.01, viscosity=True)
    opts = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=1e-8)
    host, graph = _batch(gb, sizes, phis, params, flows), _batch(gb, sizes, phis, params, flows)
    dts_h, st_h = host.advance(3, cfl=1.0, opts=opts)
    dts_g, st_g = graph.run_graph(3, cfl=1.0, opts=opts)
    np.testing.assert_array_equal(dts_g, dts_h)
    assert st_g.cg_iterations == st_h.cg_iterations and st_g.max_rel_residual == st_h.max_rel_residual
    assert st_g.frames == 3 and st_g.max_rel_residual <= 1e-8 and st_g.wall_ms > 0
    dts_h, st_h = host.advance(2, cfl=1.0, dts=dts_h, opts=opts)
    dts_g, st_g = graph.run_graph(2, cfl=1.0, dts=dts_g, opts=opts)
    np.testing.assert_array_equal(dts_g, dts_h)
    assert st_g.cg_iterations == st_h.cg_iterations
    for k in range(len(sizes)):
        for f in (gb.FIELD_PHI, gb.FIELD_U, gb.FIELD_V, gb.FIELD_UA, gb.FIELD_VA, gb.FIELD_P):
            np.testing.assert_array_equal(graph.context(k).get(f), host.context(k).get(f))
    host.close()
    graph.close()


def test_graph_run_fp64_under_tuned_schedules(gb):
    """The FP64 solver path in the graph under the autotuned sweeps and tile plans: from the
    same checkpointed states, the host-driven frames and the graph run agree bit for bit."""
    sizes, phis, params = setup()
    sizes, phis, params = sizes[:3], phis[:3], params[:3]
    flows = dict(water_viscosity=1.0, air_viscosity=0.01, viscosity=True)
    opts = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-10)
    b = _batch(gb, sizes, phis, params, flows)
    b.autotune(cfl=1.0, opts=opts)
    fields = (gb.FIELD_PHI, gb.FIELD_U, gb.FIELD_V, gb.FIELD_P)
    for k in range(len(sizes)):
        b.context(k).checkpoint_save()
    dts_h, st_h = b.advance(2, cfl=1.0, opts=opts)
    want = [[b.context(k).get(f) for f in fields] for k in range(len(sizes))]
    for k in range(len(sizes)):
        b.context(k).checkpoint_restore()
    dts_g, st_g = b.run_graph(2, cfl=1.0, opts=opts)
    np.testing.assert_array_equal(dts_g, dts_h)
    assert st_g.cg_iterations == st_h.cg_iterations and st_g.max_rel_residual <= 1e-10
    for k in range(len(sizes)):
        for f, w in zip(fields, want[k]):
            np.testing.assert_array_equal(b.context(k).get(f), w)
    b.close()


def test_graph_run_reports_nonfinite_instance(gb):
    """A NaN put into one instance's level set on the host: the graph run still finishes (each
    solve's loop sees the non-finite residual and stops), the other instances advance as in a
    host-driven run, and the call returns GB2D_ERR_NONFINITE naming the instance."""
    sizes, phis, params = setup()
    sizes, phis, params = sizes[:3], phis[:3], params[:3]
    flows = dict(water_viscosity=1.0, air_viscosity=0.01, viscosity=True)
    opts = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=1e-8)
    host, graph = _batch(gb, sizes, phis, params, flows), _batch(gb, sizes, phis, params, flows)
    bad = phis[1].copy()
    bad[2 + sizes[1][1] // 2, 2 + sizes[1][0] // 2] = np.nan
    graph.context(1).set(gb.FIELD_PHI, bad)
    with pytest.raises(gb.GB2DError) as e:
        graph.run_graph(2, cfl=1.0, opts=opts)
    assert e.value.code == -3 and "instance 1" in str(e.value)
    host.advance(2, cfl=1.0, opts=opts)
    for k in (0, 2):
        for f in (gb.FIELD_PHI, gb.FIELD_U, gb.FIELD_V, gb.FIELD_P):
            np.testing.assert_array_equal(graph.context(k).get(f), host.context(k).get(f))
    host.close()
    graph.close()
