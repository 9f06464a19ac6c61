"""Pins the CPU oracle against outputs of the reference itself.

The golden vectors in tests/golden/ were produced by running the reference's
own CUDA path (usnistgov/cyrsoxs src/cudaMain.cu, unmodified, FP32 "as
shipped" with --use_fast_math and its -DDOUBLE_PRECISION build) and
nppiWarpAffine_32f_C1R on a GB300 (tests/golden/make_reference_golden.py).

Tolerances, over pixels above 1e-6 of the peak:
* NaN masks: identical to the reference's FP32 build (the oracle mirrors its
  float geometry).
* vs the reference's FP64 build: <= 5e-5 relative (the residual is the float
  geometry the oracle shares with the FP32 build).  With RotMask the FP64
  build's double-precision warp decides a few edge pixels differently; at
  most 3% of pixels may differ there.
* vs the FP32 build: <= 5e-3 relative.  That build rounds n = 1 - delta to
  float before forming n^2 - 1, so it is itself up to ~2.3e-3 away from its
  FP64 build on these cases.
"""
import numpy as np
import pytest

import cases
import npp_cases
import oracle

PROJ_CASES = [n for n, c in cases.CASES.items() if c.mode == 0]
POL_CASES = [n for n, c in cases.CASES.items() if c.mode == 1]


def _ref(name, prec, shape):
    dt = {"fp32": np.float32, "fp64": np.float64}[prec]
    return np.fromfile(f"{cases.__file__.rsplit('/', 1)[0]}/ref_{name}_{prec}.bin", dt).reshape(shape).astype(np.float64)


def rel_err(a, ref, thr=1e-6):
    both = ~np.isnan(a) & ~np.isnan(ref)
    peak = np.abs(ref[both]).max()
    sel = both & (np.abs(ref) > thr * peak)
    return np.abs(a[sel] - ref[sel]) / np.abs(ref[sel])


@pytest.fixture(scope="module")
def oracle_outputs():
    return {}


def test_npp_warp_probes_pin_oracle_warp():
    outs = npp_cases.read_outputs(f"{cases.__file__.rsplit('/', 1)[0]}/npp_warp_out.bin")
    for (w, h, c, pre, img), ref in zip(npp_cases.probes(), outs):
        mine = oracle.warp(img, c, pre)
        assert np.array_equal(np.isnan(mine), np.isnan(ref))
        ok = ~np.isnan(ref)
        np.testing.assert_allclose(mine[ok], ref[ok], rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("name", PROJ_CASES)
def test_projection_matches_reference(name, oracle_outputs):
    case = cases.CASES[name]
    out = oracle.run_case(case)
    r32 = _ref(name, "fp32", out.shape)
    r64 = _ref(name, "fp64", out.shape)
    assert np.array_equal(np.isnan(out), np.isnan(r32)), "NaN mask differs from the reference FP32 build"
    assert rel_err(out, r32).max() <= 5e-3
    e64 = rel_err(out, r64)
    if case.rot_mask:
        assert np.mean(e64 > 5e-5) <= 0.03
    else:
        assert e64.max() <= 5e-5


@pytest.mark.parametrize("name", POL_CASES)
def test_polarization_matches_reference(name):
    case = cases.CASES[name]
    p = oracle.polarization_case(case)
    shape = (3, case.nz, case.ny, case.nx)
    r32 = np.fromfile(f"{cases.__file__.rsplit('/', 1)[0]}/ref_{name}_fp32.bin", np.complex64).reshape(shape)
    r64 = np.fromfile(f"{cases.__file__.rsplit('/', 1)[0]}/ref_{name}_fp64.bin", np.complex128).reshape(shape)
    peak = np.abs(r64).max()
    assert np.abs(p - r64).max() <= 1e-6 * peak
    assert np.abs(p - r32).max() <= 2e-4 * peak


@pytest.mark.parametrize("shape", [(4, 8, 16), (7, 15, 20), (1, 11, 13), (5, 3, 49), (16, 32, 32)])
def test_fft_matches_numpy(shape):
    rng = np.random.default_rng(sum(shape))
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    np.testing.assert_allclose(oracle.fft3d(a), np.fft.fftn(a), rtol=0, atol=1e-10 * np.sqrt(a.size) * 4)


def test_default_k_rotation_is_plain_rotation_about_z():
    for ang in (0.0, 0.3, 1.2, 2.9):
        R, base = oracle.rotation([0, 0, 1], ang)
        assert base == 0.0
        np.testing.assert_allclose(R[:, 0], [np.cos(ang), np.sin(ang), 0.0], atol=2e-6)
