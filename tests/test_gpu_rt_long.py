"""The long Rayleigh-Taylor configuration: interface y = 1 + 0.05 cos(2 pi x) on [0,1] x [0,2]
with as many nodes in y as in x (dy = 2 dx, so the reference's dx-only diagonal applies),
heavy fluid (density 3) above light (1), viscosity 1e-3, no surface tension, gravity -9.8,
500 frames of the mixed-precision path (FP32 WENO5 / reinitialisation / ENO3 fluxes,
FP32 V-cycles, CFL time steps).

Every 50 frames the mixed state is restarted for one frame (curvature, CFL time step,
order-3 time step) on the FP64 path and, at 512^2, by the CPU oracle, and the three
results of that frame are compared: the FP64 path reproduces the oracle (the level set
bit for bit, the solved fields to the solve tolerance) and the mixed frame stays within
its FP32-flux error of both.  At 2048^2 (the benchmark's size) the oracle would take
minutes per frame; there the mixed frames are compared with the FP64 path, which the
512^2 run pins to the oracle along the same trajectory kind.

Measured on GB300 (max over the 10 checkpoints): 512^2 FP64 vs oracle: phi 0, u 1.6e-10,
v 2.3e-13, p 3.8e-11, dt identical; mixed vs oracle: phi 1.1e-9, u 1.6e-8, v 1.4e-10,
p 6.1e-9.  2048^2 mixed vs FP64: phi 3.9e-10, u 1.9e-8, v 7.2e-11, p 3.9e-9.  The bounds
below are about 5x those."""
import numpy as np
import pytest

from tests.golden.cases import rayleigh_taylor_level_set

pytestmark = pytest.mark.gpu
PHYS = dict(water_density=3.0, air_density=1.0, surface_tension=0.0)
FLOW = dict(water_viscosity=1e-3, air_viscosity=1e-3, gravity=(0.0, -9.8))
FRAMES, EVERY = 500, 50


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def fields(gb):
    return (("phi", gb.FIELD_PHI), ("u", gb.FIELD_U), ("v", gb.FIELD_V), ("ua", gb.FIELD_UA), ("va", gb.FIELD_VA),
            ("p", gb.FIELD_P))


def oracle_frame(oracle, n, state):
    gr = oracle.grid(n, n, 0.0, 0.0, 1.0, 2.0)
    pr = oracle.params(pcg_tolerance=0.0, pcg_max_iterations=200000, pcg_rel_residual=1e-12, **PHYS)
    fl = oracle.flow(viscosity=True, **FLOW)
    s = {k: a.copy() for k, a in state.items()}
    kap = np.zeros((n, n))
    oracle.curvature(gr, s["phi"], kap)
    dt, _ = oracle.cfl_time_step(gr, pr, fl, s["u"], s["v"], kap, 0.5)
    oracle.time_step(gr, pr, fl, s["phi"], s["u"], s["v"], s["ua"], s["va"], s["p"], kap, None, dt)
    return dt, s


def run(gb, n, oracle=None):
    """500 mixed frames; at every 50th the restarts.  Returns one record per checkpoint."""
    mk = lambda prec: gb.Context(n, n, 0.0, 0.0, 1.0, 2.0, advection_precision=prec, **PHYS)
    cm, c64 = mk(gb.PRECISION_MIXED), mk(gb.PRECISION_FP64)
    for c in (cm, c64):
        c.set_flow_params(viscosity=True, cfl_number=0.5, **FLOW)
    cm.set(gb.FIELD_PHI, rayleigh_taylor_level_set(n, n))
    om = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=1e-8)
    o64 = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-10, max_iterations=2000)
    inner = (slice(2, 2 + n), slice(2, 2 + n))
    dt, out = 0.0, []
    for f in range(1, FRAMES + 1):
        if f % EVERY:
            dt, _ = cm.advance_frame(cfl=1.0, prev_dt=dt, opts=om)
            continue
        state = {k: cm.get(fid) for k, fid in fields(gb)}
        for k, fid in fields(gb):
            c64.set(fid, state[k])
        dtm, _ = cm.advance_frame(cfl=1.0, prev_dt=dt, opts=om)
        dt64, st = c64.advance_frame(cfl=1.0, prev_dt=dt, opts=o64)
        assert st.rel_residual <= 1e-10
        rec = {"frame": f, "dt_mixed_vs_fp64": abs(dtm / dt64 - 1)}
        got = {k: (cm.get(fid), c64.get(fid)) for k, fid in fields(gb) if k in ("phi", "u", "v", "p")}
        for k, (a, b) in got.items():
            sl = inner if k == "phi" else (slice(None), slice(None))
            assert np.all(np.isfinite(a[sl])), (f, k)
            rec["mixed_vs_fp64_" + k] = rel_l2(a[sl], b[sl])
        if oracle is not None:
            dto, s = oracle_frame(oracle, n, state)
            rec["dt_fp64_vs_oracle"] = abs(dt64 / dto - 1)
            for k, (a, b) in got.items():
                sl = inner if k == "phi" else (slice(None), slice(None))
                rec["fp64_vs_oracle_" + k] = rel_l2(b[sl], s[k][sl])
                rec["mixed_vs_oracle_" + k] = rel_l2(a[sl], s[k][sl])
        out.append(rec)
        dt = dtm
    cm.close()
    c64.close()
    return out


def test_rayleigh_taylor_512_500_frames_against_oracle(gb, oracle):
    recs = run(gb, 512, oracle)
    assert len(recs) == FRAMES // EVERY
    worst = {k: max(r[k] for r in recs) for k in recs[0] if k != "frame"}
    assert worst["dt_fp64_vs_oracle"] <= 1e-12
    assert worst["fp64_vs_oracle_phi"] <= 1e-12
    for k in ("u", "v", "p"):
        assert worst["fp64_vs_oracle_" + k] <= 1e-9, (k, worst)
    assert worst["mixed_vs_oracle_phi"] <= 1e-8, worst
    for k in ("u", "v", "p"):
        assert worst["mixed_vs_oracle_" + k] <= 1e-7, (k, worst)


def test_rayleigh_taylor_2048_500_frames_against_fp64(gb):
    recs = run(gb, 2048)
    worst = {k: max(r[k] for r in recs) for k in recs[0] if k != "frame"}
    assert worst["mixed_vs_fp64_phi"] <= 1e-8, worst
    for k in ("u", "v", "p"):
        assert worst["mixed_vs_fp64_" + k] <= 1e-7, (k, worst)
