"""The FIELDS path's autotuner: on the first device-resident request of a shape
it times the fused and separate build + x pass and the launch forms of the y
and z passes, and keeps the fastest.  Every candidate computes the same
numbers up to float rounding (the fused and separate builds contract the
same field arithmetic into fused multiply-adds differently), so the tuned
configuration must reproduce the fixed choices (CYRSOXS_GB300_AUTOTUNE=0, in a
second process) to 2e-6 relative with identical NaN masks, and the choice is
listed by cyr_tuning_report.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import cases
from test_gpu_parity import native, options_for

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASE = cases.Case("tune_fields", 256, 256, 64, 2, [282.0, 287.0], seed=81, geometry="blobs", angles=(0.0, 150.0, 30.0))

CHILD = r"""
import sys
import numpy as np
sys.path[:0] = [{root!r}, {root!r} + "/tests", {root!r} + "/tests/golden", {root!r} + "/oracle"]
import cases
from test_gpu_parity import options_for
from cyrsoxs_gb300 import _native
import test_gpu_autotune as t
c = t.CASE
out = _native.cuda_main(options_for(c, strategy=2), cases.optical_constants(c), cases.voxels(c))
np.save(sys.argv[1], out)
print(_native.tuning_report())
"""


def _device_resident(nat, case):
    import torch

    vox = torch.from_numpy(np.ascontiguousarray(cases.voxels(case), np.float32)).cuda()
    out = torch.empty(len(case.energies) * case.nx * case.ny, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    nat.simulate_device(options_for(case, strategy=2), cases.optical_constants(case), vox.data_ptr(), out.data_ptr(),
                        stream.cuda_stream)
    stream.synchronize()
    return out.cpu().numpy().reshape(len(case.energies), 1, case.ny, case.nx)


def test_tuned_fields_transform_equals_the_fixed_choices(tmp_path):
    nat = native()
    tuned = _device_resident(nat, CASE)  # the first device-resident request of this shape tunes it
    report = nat.tuning_report()
    assert "fields[256,256,64," in report, report
    path = str(tmp_path / "fixed.npy")
    env = dict(os.environ, CYRSOXS_GB300_AUTOTUNE="0")
    p = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT), path], capture_output=True, text=True, env=env,
                       timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "fields[" not in p.stdout  # nothing was tuned in that process
    fixed = np.load(path)
    assert np.array_equal(np.isnan(tuned), np.isnan(fixed))
    ok = ~np.isnan(fixed)
    peak = np.abs(fixed[ok]).max()
    sel = ok & (np.abs(fixed) > 1e-6 * peak)
    assert (np.abs(tuned[sel] - fixed[sel]) / np.abs(fixed[sel])).max() <= 2e-6
