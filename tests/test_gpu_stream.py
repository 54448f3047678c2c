"""The streaming smoother (gb2d_stream.cuh, GB2D_SMOOTHER=stream) performs exactly the
red-black Gauss-Seidel sweeps, residual restriction and prolongation of the tiled smoother
(the default, GB2D_SMOOTHER=tiled): one V-cycle of the preconditioner gives bit-identical z on grids
with even and odd row lengths, 1, 2 and 3 sweeps per side, FP64 and FP32 levels, with the
cluster tail and with the single-CTA tail (which leaves the 128^2 level to the smoother).
Each variant runs in a child process (the library reads the switches once)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def _run(tmp_path, name, **env):
    out = os.path.join(str(tmp_path), name + ".npz")
    e = dict(os.environ, **env)
    subprocess.run([sys.executable, "-m", "tests.vcycle_child", out], cwd=ROOT, env=e, check=True, timeout=600)
    with np.load(out) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("cluster", ["1", "0"])
def test_streaming_vcycle_bit_identical_to_tiled(gb, tmp_path, cluster):
    tiled = _run(tmp_path, "tiled", GB2D_SMOOTHER="tiled", GB2D_CLUSTER_TAIL=cluster)
    stream = _run(tmp_path, "stream", GB2D_SMOOTHER="stream", GB2D_CLUSTER_TAIL=cluster)
    assert tiled.keys() == stream.keys()
    for k in tiled:
        assert np.all(np.isfinite(stream[k])), k
        assert np.array_equal(tiled[k], stream[k]), (k, float(np.abs(tiled[k] - stream[k]).max()))
