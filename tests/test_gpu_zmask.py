"""The FIELDS z pass stores only the planes that the Ewald projection and the
DC replacement read (k_zmask builds the mask; k_fft_cols_tma_ws applies it) and
skips the tiles that hold none of them.  The planes it does store come out of
the same kernels either way, so a request gives bit-identical projections with
the mask (the default) and without it (CYRSOXS_GB300_ZMASK=0).  Both runs use
the fixed launch forms (CYRSOXS_GB300_AUTOTUNE=0) in child processes.

Cases: k along z with linear and nearest-plane interpolation, two tilted k
vectors (beam divergence), grazing incidence, a non-square detector, the
three masked z lengths (128, 256, 512), windowing with the rotation mask, and
a wide Ewald band whose corners are NaN (physSize 2 nm, as on the headline
workload: tiles of those columns are skipped).  The tilted case is also compared with
the oracle.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import cases
import oracle
from test_gpu_parity import TOL, native, options_for, rel_err

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

ZCASES = [
    cases.Case("zm_tilted_k", 64, 48, 128, 2, [282.0, 288.0], case_type=1, kvecs=[[0.0, 0.15, 1.0], [0.1, 0.0, 1.0]],
               seed=91, geometry="blobs", angles=(0.0, 150.0, 30.0)),
    cases.Case("zm_grazing", 48, 64, 128, 2, [285.0], case_type=2, kvecs=[[0.0, 0.1, 1.0]], detector=(0.0, 0.1, 1.0),
               seed=92, geometry="blobs", angles=(0.0, 90.0, 45.0)),
    cases.Case("zm_nn_256", 32, 32, 256, 2, [284.0, 290.0], interpolation=cases.NN, seed=93, geometry="blobs",
               angles=(0.0, 120.0, 60.0)),
    cases.Case("zm_vector_512", 16, 32, 512, 3, [285.0], morphology=cases.VECTOR, seed=94, geometry="blobs",
               angles=(0.0, 90.0, 45.0)),
    cases.Case("zm_hann_mask", 64, 64, 128, 2, [283.0, 287.0], windowing=1, rot_mask=1, seed=95,
               angles=(0.0, 150.0, 75.0)),
    cases.Case("zm_wide_band", 64, 64, 128, 2, [280.0, 285.0, 290.0], phys_size=2.0, seed=96),
]

CHILD = r"""
import sys
import numpy as np
sys.path[:0] = [{root!r}, {root!r} + "/tests", {root!r} + "/tests/golden", {root!r} + "/oracle"]
import cases
from test_gpu_parity import options_for
from cyrsoxs_gb300 import _native
import test_gpu_zmask as t
out = {{}}
_native.profile_begin()
for c in t.ZCASES:
    out[c.name] = _native.cuda_main(options_for(c, strategy=2), cases.optical_constants(c), cases.voxels(c))
prof, _ = _native.profile_end()
np.savez(sys.argv[1], **out)
print("zmask launches:", prof.get("k_zmask", (0,))[0])
"""


def _run(tmp_path, tag, **env_extra):
    path = str(tmp_path / f"{tag}.npz")
    env = dict(os.environ, CYRSOXS_GB300_AUTOTUNE="0", **env_extra)
    p = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT), path], capture_output=True, text=True, env=env,
                       timeout=900, cwd=ROOT)
    assert p.returncode == 0, p.stdout + p.stderr
    launches = int(p.stdout.strip().rsplit(":", 1)[1])
    return np.load(path), launches


def test_masked_z_pass_gives_identical_projections(tmp_path):
    native()  # skips without a GPU
    masked, n_masked = _run(tmp_path, "masked")
    full, n_full = _run(tmp_path, "full", CYRSOXS_GB300_ZMASK="0")
    assert n_masked == len(ZCASES), n_masked  # one mask per request
    assert n_full == 0
    for c in ZCASES:
        a, b = masked[c.name], full[c.name]
        assert np.array_equal(a, b, equal_nan=True), c.name


def test_masked_z_pass_with_tilted_k_matches_oracle():
    nat = native()
    case = ZCASES[0]
    got = nat.cuda_main(options_for(case, strategy=2), cases.optical_constants(case),
                        cases.voxels(case)).astype(np.float64)
    want = oracle.run_case(case)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    e = rel_err(got, want)
    assert e.max() <= TOL, e.max()
