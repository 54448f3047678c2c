"""The headless .sim driver (2d_engine_gb300/_build/gb2d_sim): it reads the reference's
script format (blocks, comments, #INCLUDE, reference defaults for missing keys) and, on
a GPU, advances frames as SIMULATION_WORLD::AdvanceOneFrame does."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

SCRIPT = os.path.join(GOLDEN, "rising_bubble_128.sim")


@pytest.fixture(scope="module")
def sim(gb):
    build = __import__("importlib").import_module("2d_engine_gb300.build")
    return build.build_driver()


def dry(sim, script):
    r = subprocess.run([sim, script, "--dry-run"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def test_dry_run_reads_the_script(sim):
    c = dry(sim, SCRIPT)
    assert c["grid"] == [128, 128, 0, 0, 1, 1]
    assert c["CFL"] == 1 and c["dt"] == 1e-6 and c["last_frame"] == 100
    assert (c["water_density"], c["air_density"], c["surface_tension"]) == (1000, 1, 0.0728)
    assert (c["reinit_iterations"], c["reinit_scaling"], c["cfl_number"]) == (25, 5, 0.5)
    assert c["gravity"] == [0, -9.8] and c["viscosity"] == 0 and c["precision"] == 0
    assert c["bubble"] == [0.5, 0.3, 0.15] and c["output_every"] == 10


def test_reader_includes_comments_and_reference_defaults(sim, tmp_path):
    (tmp_path / "fluid.sim").write_text(
        "FLUID_SOLVER_UNIFORM { AIR_WATER_SIMULATION { water_density = 3; air_density = 1 // light\n"
        "  /* surface tension and reinit numbers left to the defaults */ gravity = (0, -1) } }\n")
    (tmp_path / "main.sim").write_text(
        "// small bubble of the reference script\n"
        "SIMULATION_WORLD { CFL = 0.9 fluid_solver = true\n"
        "  FLUID_SOLVER_OPTIONS { air_water_simulation = true }\n"
        "  WORLD_DISCRETIZATION { AIR_WATER_SIMULATION { small_bubble = true\n"
        "    GRID_STRUCTURE_2D_SMALL { base_grid_resolution = (81, 121) base_grid_min = ( -0.01, -0.015)\n"
        "      base_grid_max = ( 0.01, 0.015) } } } }\n"
        "#INCLUDE <fluid.sim>\n")
    c = dry(sim, str(tmp_path / "main.sim"))
    assert c["grid"] == [81, 121, -0.01, -0.015, 0.01, 0.015]
    assert c["water_density"] == 3 and c["gravity"] == [0, -1] and c["CFL"] == 0.9
    # EULERIAN_FLUID_SOLVER_2D.h / ADVECTION_2D.cpp defaults
    assert c["surface_tension"] == 1 and c["reinit_iterations"] == 10 and c["reinit_scaling"] == 5
    assert c["weno_epsilon"] == float(np.float32(1e-6)) and c["dt"] == 0.01 and c["max_dt"] == 100
    assert c["bubble"] == [0, -0.005, 1 / 300] and c["bubble_source"] == "small_bubble"


def test_rejects_scripts_it_cannot_run(sim, tmp_path):
    (tmp_path / "oil.sim").write_text("SIMULATION_WORLD { fluid_solver = true FLUID_SOLVER_OPTIONS { oil_water_simulation = true } }\n")
    r = subprocess.run([sim, str(tmp_path / "oil.sim"), "--dry-run"], capture_output=True, text=True)
    assert r.returncode == 1 and "air/water" in r.stderr
    (tmp_path / "bad.sim").write_text("SIMULATION_WORLD { CFL = 1 \n")
    r = subprocess.run([sim, str(tmp_path / "bad.sim"), "--dry-run"], capture_output=True, text=True)
    assert r.returncode == 1 and "}" in r.stderr


@pytest.mark.gpu
def test_ten_frames_match_the_reference(sim, tmp_path):
    out = tmp_path / "out"
    r = subprocess.run([sim, SCRIPT, "--frames", "10", "--out", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert sum(1 for line in r.stdout.splitlines() if line.startswith("frame ")) == 10
    g = load_golden("rising_bubble_128_frames")
    for k in ("phi", "u", "v", "p"):
        got = np.load(out / f"{k}_000010.npy")
        want = g[f"{k}10"]
        assert got.shape == want.shape
        assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-8, k
