"""The command line end to end on the GPU: its Energy_<E>.h5 files hold what
cuda_main computes for the same inputs."""
import os

import numpy as np
import pytest

from test_config_cli import make_run_dir

pytestmark = pytest.mark.gpu


def test_cli_writes_the_patterns_cuda_main_computes(tmp_path, monkeypatch):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cyrsoxs_gb300 import _native, cli, config, h5io

    make_run_dir(str(tmp_path))
    monkeypatch.chdir(tmp_path)
    assert cli.main(["morph.h5", "results"]) == 0
    morph = h5io.read_morphology("morph.h5", 0)
    cfg = config.read_config("config.txt")
    inp = cli.build_input(cfg, morph)
    want = _native.cuda_main(inp._options(), config.read_materials(2, cfg["energies"]), morph.voxels)
    for i, e in enumerate(cfg["energies"]):
        f = h5io.File(os.path.join("results", f"Energy_{e:.2f}.h5"))
        got = f.read("K0/projection")
        np.testing.assert_array_equal(np.isnan(got), np.isnan(want[i, 0]))
        np.testing.assert_array_equal(got[~np.isnan(got)], want[i, 0][~np.isnan(got)])
    assert os.path.exists("CyRSoXS.log")
