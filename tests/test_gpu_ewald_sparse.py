"""The FIELDS Ewald kernel skips the structural zeros of its combination.

Tensor entry v takes packed volume j only when one of the volume's two fields
enters that entry (coef_used in csrc/fields.cuh): u_x u_y only xy, u_x u_z
only xz, u_y u_z only yz, the squares, phi_ui and T only the diagonal.  For
1-4 materials in the LAB frame with k along z the kernel walks the volumes at
compile time and never forms the zero terms; CYRSOXS_GB300_SPARSE_EWALD=0 forms
every term.  Adding a zero term changes no bit of a finite sum, so both runs
(child processes, fixed launch forms) must give bit-identical projections,
single requests and a request group served together alike.  One case is also
compared with the oracle.
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

SCASES = [
    cases.Case("sp_m1", 48, 48, 32, 1, [283.0, 287.0], seed=101, geometry="blobs", angles=(0.0, 150.0, 30.0)),
    cases.Case("sp_m2_nn", 64, 64, 16, 2, [281.0, 285.0, 289.0], interpolation=cases.NN, seed=102, geometry="blobs",
               angles=(0.0, 150.0, 30.0)),
    cases.Case("sp_m3_vector_hann", 40, 56, 32, 3, [284.0, 286.0], morphology=cases.VECTOR, windowing=1, rot_mask=1,
               seed=103, geometry="blobs", angles=(0.0, 120.0, 40.0)),
    cases.Case("sp_m4_wide", 64, 64, 128, 4, [280.0, 285.0, 290.0], phys_size=2.0, seed=104, geometry="blobs",
               angles=(0.0, 175.0, 5.0)),
]
# same-shape requests on device buffers, queued behind a running one: served as one group
GROUP = [cases.Case(f"sp_grp{i}", 64, 64, 16, 3, [282.0 + i, 286.0 + i], seed=110 + i, geometry="blobs",
                    angles=(0.0, 150.0, 30.0)) for i in range(5)]

CHILD = r"""
import sys
import numpy as np
import torch
sys.path[:0] = [{root!r}, {root!r} + "/tests", {root!r} + "/tests/golden", {root!r} + "/oracle"]
import cases
from test_gpu_parity import options_for
from cyrsoxs_gb300 import _native, serving
import test_gpu_ewald_sparse as t
out = {{}}
for c in t.SCASES:
    out[c.name] = _native.cuda_main(options_for(c, strategy=2), cases.optical_constants(c), cases.voxels(c))
dev = [(options_for(c, strategy=2), cases.optical_constants(c),
        torch.from_numpy(np.ascontiguousarray(cases.voxels(c), np.float32)).cuda(),
        torch.zeros(len(c.energies) * c.nx * c.ny, dtype=torch.float32, device="cuda")) for c in t.GROUP]
torch.cuda.synchronize()
with serving.Server(slots=1, groups=True) as srv:
    ids = [srv.submit(o, opt, dv.data_ptr(), do.data_ptr(), device=True) for o, opt, dv, do in dev]
    for i in ids:
        srv.wait(i)
    st = srv.stats()
for c, (_, _, _, do) in zip(t.GROUP, dev):
    out[c.name] = do.cpu().numpy()
np.savez(sys.argv[1], **out)
print("grouped requests:", st["grouped_requests"])
"""


def _run(tmp_path, name, sparse):
    path = str(tmp_path / f"{name}.npz")
    env = dict(os.environ, CYRSOXS_GB300_AUTOTUNE="0", CYRSOXS_GB300_SPARSE_EWALD="1" if sparse else "0")
    p = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT), path], capture_output=True, text=True, env=env,
                       timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "grouped requests: 0" not in p.stdout, p.stdout
    return np.load(path)


def test_sparse_combination_is_bit_identical_to_the_dense_one(tmp_path):
    native()
    sparse = _run(tmp_path, "sparse", True)
    dense = _run(tmp_path, "dense", False)
    for c in SCASES + GROUP:
        a, b = sparse[c.name], dense[c.name]
        assert a.shape == b.shape
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), c.name


def test_sparse_combination_matches_oracle():
    nat = native()
    c = SCASES[2]  # three materials, vector morphology, windowing and the rotation mask
    got = nat.cuda_main(options_for(c, strategy=2), cases.optical_constants(c), cases.voxels(c)).astype(np.float64)
    want = oracle.run_case(c)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    assert rel_err(got, want).max() <= TOL
