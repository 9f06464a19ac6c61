"""GPU parity of the engine, through its C ABI, against the FP64 oracle and the
reference's own outputs.

Tolerance (the engine's precision contract): over detector pixels above 1e-6
of the peak, max relative error <= 1e-4 against the FP64 oracle, and NaN
masks identical to the oracle's and to the reference FP32 build's.
"""
import numpy as np
import pytest

import cases
import npp_cases
import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-4
GOLDEN = cases.__file__.rsplit("/", 1)[0]


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def native():
    _torch()
    from cyrsoxs_gb300 import _native

    return _native


def options_for(case, **over):
    from cyrsoxs_gb300 import _native

    kv = [[0.0, 0.0, 1.0]] if case.case_type == 0 else [cases._normalize32(k).tolist() for k in case.kvecs]
    kw = dict(nx=case.nx, ny=case.ny, nz=case.nz, num_material=case.num_material, energies=case.energies,
              start_angle=case.angles[0], end_angle=case.angles[1], increment_angle=case.angles[2],
              phys_size=case.phys_size, case_type=case.case_type, k_vectors=kv, detector=case.detector,
              morphology_type=case.morphology, ewald_interpolation=case.interpolation, windowing=case.windowing,
              scatter_approach=case.scatter, algorithm=case.algorithm, max_streams=case.max_streams,
              rot_mask=case.rot_mask, reference_frame=case.frame)
    kw.update(over)
    return _native.Options(**kw)


def rel_err(a, ref, thr=1e-6):
    both = ~np.isnan(a) & ~np.isnan(ref)
    peak = np.abs(ref[both]).max()
    sel = both & (np.abs(ref) > thr * peak)
    return np.abs(a[sel] - ref[sel]) / np.abs(ref[sel])


@pytest.mark.parametrize("shape,count", [((4, 8, 16), 1), ((7, 15, 20), 2), ((1, 64, 48), 1), ((16, 32, 32), 3),
                                         ((32, 256, 256), 1), ((9, 25, 49), 1), ((3, 128, 512), 2),
                                         ((128, 20, 24), 1), ((256, 6, 40), 1), ((512, 512, 8), 1),
                                         ((2, 512, 128), 3), ((2, 8, 1024), 2), ((4, 1024, 24), 1), ((1024, 4, 40), 1),
                                         ((16, 64, 40), 2), ((32, 8, 16), 1),
                                         # TMA column passes: 32-column tiles, 16-column tiles (nx not a
                                         # multiple of 32), 512-point lines on several volumes
                                         ((4, 256, 64), 2), ((256, 4, 48), 1), ((2, 256, 80), 2), ((2, 512, 16), 3),
                                         # TMA column passes on 128-point lines (16- and 32-column tiles)
                                         ((128, 8, 48), 1), ((4, 128, 64), 2), ((128, 4, 32), 3),
                                         # Bluestein: lengths with a prime factor above 7 on every axis
                                         ((3, 11, 13), 2), ((2, 97, 101), 1), ((61, 6, 40), 1), ((2, 4, 2039), 1),
                                         ((17, 256, 48), 1), ((5, 127, 64), 2), ((1, 22, 1031), 1)])
def test_fft3d_matches_numpy(shape, count):
    torch = _torch()
    nat = native()
    rng = np.random.default_rng(sum(shape) + count)
    a = (rng.standard_normal((count,) + shape) + 1j * rng.standard_normal((count,) + shape)).astype(np.complex64)
    d = torch.from_numpy(a.view(np.float32)).cuda()
    nz, ny, nx = shape
    nat.fft3d_device(d.data_ptr(), nx, ny, nz, count, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = d.cpu().numpy().view(np.complex64)
    ref = np.fft.fftn(a.astype(np.complex128), axes=(1, 2, 3))
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 2e-6, err


def test_tma_wait_limit_reports_and_recovers():
    """The TMA column pass bounds every barrier wait.  A tile whose copies
    deliver fewer bytes than the barrier expects never completes: the kernel
    must give up, report it, let its copies land, and leave the context usable
    for the transforms that follow."""
    _torch()
    nat = native()
    assert nat.selftest_wait_limit() is True
    test_fft3d_matches_numpy((4, 256, 64), 2)


def test_warp_is_bit_exact_with_npp_probes():
    torch = _torch()
    nat = native()
    outs = npp_cases.read_outputs(f"{GOLDEN}/npp_warp_out.bin")
    for i, ((w, h, c, pre, img), ref) in enumerate(zip(npp_cases.probes(), outs)):
        src = torch.from_numpy(np.ascontiguousarray(img, np.float32)).cuda()
        dst = torch.full((h, w), pre, dtype=torch.float32, device="cuda")
        nat.warp_affine_device(src.data_ptr(), dst.data_ptr(), w, h, c, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        got = dst.cpu().numpy()
        assert np.array_equal(np.isnan(got), np.isnan(ref)), i
        ok = ~np.isnan(ref)
        assert np.array_equal(got[ok], ref[ok]), (i, np.abs(got[ok] - ref[ok]).max())


PROJ = [n for n, c in cases.CASES.items() if c.mode == 0]


@pytest.mark.parametrize("name", PROJ)
def test_projection_matches_oracle_and_reference(name):
    nat = native()
    case = cases.CASES[name]
    opts = options_for(case)
    got = nat.cuda_main(opts, cases.optical_constants(case), cases.voxels(case),
                        streams_variant=case.algorithm == 1).astype(np.float64)
    want = oracle.run_case(case)
    r32 = np.fromfile(f"{GOLDEN}/ref_{name}_fp32.bin", np.float32).reshape(want.shape)
    assert np.array_equal(np.isnan(got), np.isnan(want)), "NaN mask differs from the FP64 oracle"
    assert np.array_equal(np.isnan(got), np.isnan(r32)), "NaN mask differs from the reference FP32 build"
    e = rel_err(got, want)
    assert e.max() <= TOL, e.max()


@pytest.mark.parametrize("name", [n for n, c in cases.CASES.items() if c.mode == 1])
def test_polarization_matches_oracle(name):
    nat = native()
    case = cases.CASES[name]
    opts = options_for(case)
    eid = int(np.searchsorted(np.asarray(case.energies, np.float32), np.float32(case.pol_energy)))
    px, py, pz = nat.compute_polarization(opts, cases.optical_constants(case), cases.voxels(case), case.pol_eangle, eid)
    want = oracle.polarization_case(case)
    got = np.stack([px, py, pz]).astype(np.complex128)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


# Long z axes take the warp-FFT form of the fused build + z FFT (nz = 128, 256, 512) with z pruning;
# these cases are checked against the oracle (which is itself pinned to the reference's outputs).
LONG_Z = [
    cases.Case("z128_euler", 64, 48, 128, 2, [282.0, 288.0], seed=31, geometry="blobs", angles=(0.0, 150.0, 30.0)),
    cases.Case("z256_vector_hann", 32, 32, 256, 3, [285.0], seed=32, morphology=cases.VECTOR, windowing=1,
               geometry="blobs", angles=(0.0, 90.0, 45.0)),
    cases.Case("z512_euler_nn", 16, 24, 512, 2, [284.0], seed=33, interpolation=cases.NN, geometry="blobs",
               angles=(15.0, 75.0, 30.0)),
    cases.Case("z256_mask_alg1", 40, 40, 256, 2, [286.0], seed=34, rot_mask=1, algorithm=1, geometry="blobs",
               angles=(0.0, 120.0, 60.0)),
]


@pytest.mark.parametrize("case", LONG_Z, ids=[c.name for c in LONG_Z])
def test_long_z_axes_match_oracle(case):
    nat = native()
    got = nat.cuda_main(options_for(case), cases.optical_constants(case), cases.voxels(case),
                        streams_variant=case.algorithm == 1).astype(np.float64)
    want = oracle.run_case(case)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    e = rel_err(got, want)
    assert e.max() <= TOL, e.max()
    assert nat.device_errors() == 0


# FIELDS strategy: the morphology's energy independent fields are transformed once per request and
# every energy and angle is combined from them (fields.cuh).  Same tolerance, same NaN masks.
@pytest.mark.parametrize("name", PROJ)
def test_field_strategy_matches_oracle_and_reference(name):
    nat = native()
    case = cases.CASES[name]
    got = nat.cuda_main(options_for(case, strategy=2), cases.optical_constants(case), cases.voxels(case),
                        streams_variant=case.algorithm == 1).astype(np.float64)
    want = oracle.run_case(case)
    r32 = np.fromfile(f"{GOLDEN}/ref_{name}_fp32.bin", np.float32).reshape(want.shape)
    assert np.array_equal(np.isnan(got), np.isnan(want)), "NaN mask differs from the FP64 oracle"
    assert np.array_equal(np.isnan(got), np.isnan(r32)), "NaN mask differs from the reference FP32 build"
    e = rel_err(got, want)
    assert e.max() <= TOL, e.max()


@pytest.mark.parametrize("case", LONG_Z, ids=[c.name for c in LONG_Z])
def test_field_strategy_long_z_axes(case):
    nat = native()
    got = nat.cuda_main(options_for(case, strategy=2), cases.optical_constants(case), cases.voxels(case),
                        streams_variant=case.algorithm == 1).astype(np.float64)
    want = oracle.run_case(case)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    e = rel_err(got, want)
    assert e.max() <= TOL, e.max()


def test_strategies_agree_and_auto_picks_fields_for_many_energies():
    nat = native()
    case = cases.Case("strat", 64, 64, 32, 3, [280.0, 283.0, 285.0, 288.0, 291.0, 296.0], seed=41,
                      geometry="blobs", angles=(0.0, 170.0, 10.0))
    per = nat.cuda_main(options_for(case, strategy=1), cases.optical_constants(case), cases.voxels(case))
    fld = nat.cuda_main(options_for(case, strategy=2), cases.optical_constants(case), cases.voxels(case))
    assert nat.plan_info(options_for(case))["fields"] == 1
    assert np.array_equal(np.isnan(per), np.isnan(fld))
    e = rel_err(fld.astype(np.float64), per.astype(np.float64))
    assert e.max() <= TOL, e.max()


# Lengths with a prime factor above 7 (Bluestein transforms on the affected axes), both strategies.
PRIME = [
    cases.Case("prime_xyz", 37, 29, 11, 2, [282.0, 286.0], seed=51, geometry="blobs", angles=(0.0, 150.0, 30.0)),
    cases.Case("prime_z_vector", 32, 32, 23, 3, [285.0], seed=52, morphology=cases.VECTOR, geometry="blobs",
               angles=(0.0, 90.0, 45.0)),
    cases.Case("prime_x_2d", 101, 64, 1, 2, [284.0], seed=53, geometry="blobs", angles=(0.0, 120.0, 60.0)),
]


@pytest.mark.parametrize("strategy", [1, 2])
@pytest.mark.parametrize("case", PRIME, ids=[c.name for c in PRIME])
def test_prime_lengths_match_oracle(case, strategy):
    nat = native()
    got = nat.cuda_main(options_for(case, strategy=strategy), cases.optical_constants(case),
                        cases.voxels(case)).astype(np.float64)
    want = oracle.run_case(case)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    e = rel_err(got, want)
    assert e.max() <= TOL, e.max()


# The field build fused with the x-row FFT (k_build_fields_rows) for every warp-FFT row length, Euler and vector
# morphologies, windowed and not, with 2 to 5 materials (up to 18 packed volumes in shared memory).
FUSED_ROWS = [
    cases.Case("rows128_vector_hann", 128, 128, 8, 3, [284.0, 286.0], seed=71, morphology=cases.VECTOR, windowing=1,
               geometry="blobs", angles=(0.0, 120.0, 60.0)),
    cases.Case("rows512_euler", 512, 512, 4, 2, [285.0], seed=72, geometry="blobs", angles=(0.0, 90.0, 45.0)),
    cases.Case("rows1024_euler_mask", 1024, 1024, 4, 5, [283.0], seed=73, geometry="blobs", rot_mask=1,
               angles=(0.0, 150.0, 75.0)),
]


@pytest.mark.parametrize("case", FUSED_ROWS, ids=[c.name for c in FUSED_ROWS])
def test_fused_field_rows_match_oracle(case):
    nat = native()
    got = nat.cuda_main(options_for(case, strategy=2), cases.optical_constants(case),
                        cases.voxels(case)).astype(np.float64)
    want = oracle.run_case(case)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    e = rel_err(got, want)
    assert e.max() <= TOL, e.max()
