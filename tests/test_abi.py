"""CPU checks of the C ABI library: it builds for sm_103a, loads, and exports
every entry point that include/gb2d.h declares (no GPU calls)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "gb2d.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(gb2d_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("gb2d_create", "gb2d_projection", "gb2d_levelset_rk3", "gb2d_reinitialization", "gb2d_poisson_solve"):
        assert must in names


def test_library_exports_every_declared_symbol(gb):
    lib = ctypes.CDLL(gb.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_signatures_cover_header(gb):
    lib = gb.library()
    for n in declared_symbols():
        assert getattr(lib, n).argtypes is not None, n


def test_field_extents_match_reference_layout(gb):
    lib = gb.library()
    g = gb.GridT(33, 17, 0.0, 0.0, 1.0, 1.0)
    want = {gb.FIELD_PHI: (37, 21), gb.FIELD_U: (38, 21), gb.FIELD_V: (37, 22), gb.FIELD_UA: (40, 23),
            gb.FIELD_VA: (39, 24), gb.FIELD_P: (35, 19), gb.FIELD_KAPPA: (33, 17)}
    for f, (ir, jr) in want.items():
        a, b = ctypes.c_int(), ctypes.c_int()
        assert lib.gb2d_field_extent(ctypes.byref(g), f, ctypes.byref(a), ctypes.byref(b)) == 0
        assert (a.value, b.value) == (ir, jr)
    a, b = ctypes.c_int(), ctypes.c_int()
    assert lib.gb2d_field_extent(ctypes.byref(g), 99, ctypes.byref(a), ctypes.byref(b)) == -1


def test_create_rejects_bad_arguments(gb):
    lib = gb.library()
    h = ctypes.c_void_p()
    p = gb.ParamsT(1000.0, 1.0, 0.07, 1e-6, 25, 5, 0)
    assert lib.gb2d_create(ctypes.byref(gb.GridT(3, 10, 0, 0, 1, 1)), ctypes.byref(p), ctypes.byref(h)) == -1
    assert lib.gb2d_create(ctypes.byref(gb.GridT(10, 10, 1, 0, 1, 1)), ctypes.byref(p), ctypes.byref(h)) == -1
    bad = gb.ParamsT(1000.0, 1.0, 0.07, 1e-6, 25, 0, 0)
    assert lib.gb2d_create(ctypes.byref(gb.GridT(10, 10, 0, 0, 1, 1)), ctypes.byref(bad), ctypes.byref(h)) == -1


def test_cpp_adapter_compiles(tmp_path):
    """include/gb2d_adapter.hpp (the C++ mirror a reference maintainer includes) compiles
    against the header with the reference's C++ dialect."""
    import shutil
    import subprocess
    import pytest
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "use_adapter.cpp"
    src.write_text('#include "gb2d_adapter.hpp"\n'
                   'void step(GB2D_FLUID_STEP& s, double dt) {\n'
                   '  s.Levelset_RK3(dt, 0); s.SolveForRK(dt, 0); s.AdvanceOneTimeStepThread(dt, 0);\n'
                   '  double d = s.CFLOneTimeStep(); s.AdvanceOneFrame(1.0, d); s.Projection(dt, 0);\n'
                   '  gb2d_flow_params f = {1.0, 0.01, 0.0, -9.8, 0.5, 0}; s.SetFlowParams(f);\n'
                   '}\n')
    r = subprocess.run([cxx, "-std=c++14", "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_field_density_extent(gb):
    g = gb.GridT(33, 17, 0.0, 0.0, 1.0, 1.0)
    a, b = ctypes.c_int(), ctypes.c_int()
    assert gb.library().gb2d_field_extent(ctypes.byref(g), gb.FIELD_DENSITY, ctypes.byref(a), ctypes.byref(b)) == 0
    assert (a.value, b.value) == (37, 21)


def test_create_rejects_non_positive_densities(gb):
    """The face weights divide by both densities (POISSON_SOLVER.cpp:743-746 with
    v = 1/rho): zero, negative or NaN densities are rejected before any device work."""
    lib = gb.library()
    h = ctypes.c_void_p()
    g = gb.GridT(10, 10, 0, 0, 1, 1)
    for water, air in ((0.0, 1.0), (1000.0, 0.0), (-1.0, 1.0), (float("nan"), 1.0), (1000.0, float("nan"))):
        p = gb.ParamsT(water, air, 0.07, 1e-6, 25, 5, 0)
        assert lib.gb2d_create(ctypes.byref(g), ctypes.byref(p), ctypes.byref(h)) == -1, (water, air)
        assert not h.value


def test_batch_entry_points_reject_bad_arguments(gb):
    """The batch run, its schedule query and the tile-plan knob check their arguments before any
    device work (no GPU needed)."""
    lib = gb.library()
    st = gb.BatchStatsT()
    o = gb.solve_opts()
    dts = (ctypes.c_double * 1)()
    assert lib.gb2d_batch_run_graph(None, 1, 1.0, dts, ctypes.byref(o), ctypes.byref(st)) == -1
    assert lib.gb2d_batch_advance(None, 1, 1.0, dts, ctypes.byref(o), ctypes.byref(st)) == -1
    sw, tp = ctypes.c_int(), ctypes.c_int()
    assert lib.gb2d_batch_schedule(None, 0, ctypes.byref(sw), ctypes.byref(tp)) == -1
    assert lib.gb2d_set_tile_plan(None, 1) == -1


def test_reference_solver_links_with_the_dropin(gb):
    """The drop-in in the reference's own solver class: oracle/ref/patch_gpu_step.py applies
    the member hooks INTEGRATION.md describes to a copy of EULERIAN_FLUID_SOLVER_2D.h, and the
    headless reference build links that class against libgb2d.so with no undefined symbol.
    Runs where the reference sources are (it needs them to build); calling it needs a GPU
    and those sources together, which no machine of this project has."""
    import shutil
    import subprocess
    ref = os.environ.get("REFERENCE", "/root/reference")
    if not os.path.exists(os.path.join(ref, "EULERIAN_FLUID_SOLVER_2D.h")) or shutil.which("make") is None:
        pytest.skip("reference sources not present")
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "gpu", f"REFERENCE={ref}"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    so = os.path.join(ROOT, "oracle", "_ref", "libref2d_gpu.so")
    lib = ctypes.CDLL(so)
    for name in ("ref_create", "ref_enable_gpu", "ref_gpu_download", "ref_step", "ref_cfl_dt"):
        assert hasattr(lib, name), name
    nm = subprocess.run(["nm", "-D", "--undefined-only", so], capture_output=True, text=True).stdout
    for name in ("gb2d_create", "gb2d_advance_time_step", "gb2d_cfl_time_step", "gb2d_projection", "gb2d_levelset_advection"):
        assert name in nm, name
    patched = open(os.path.join(ROOT, "oracle", "_ref", "patched", "EULERIAN_FLUID_SOLVER_2D.h")).read()
    assert patched.count("if (gpu_step)") == 6
