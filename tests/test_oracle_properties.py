"""Analytical properties of the Born-approximation path, checked on the CPU
oracle without the reference.

For isotropic materials (S = 0, n_par = n_perp = n) the polarization is
p = sum_m vf_m (n_m^2 - 1) E / 4 pi (include/uniaxial.h:58-169), and every
later stage - window-free FFT, DC replacement (src/cudaMain.cu:123-176),
shift, Ewald projection of |(k^2 I - q q^T) p|^2 (include/uniaxial.h:876-947)
and the angle average - is linear in p before the square.  Hence:
* scaling every (n_m^2 - 1) by one complex c scales every pattern by |c|^2;
* adding one constant to every n_m^2 (volume fractions summing to 1) changes
  only the q = 0 bin, which the DC replacement overwrites: nothing changes;
* exchanging the two materials of a two-phase morphology together with their
  constants leaves the patterns unchanged.
Tolerance: 1e-5 relative over pixels above 1e-6 of the peak (the inputs are
float32; the oracle computes in FP64), NaN masks identical.
"""
import numpy as np
import pytest

import cases
import oracle

CASE = cases.Case("iso_blobs", 32, 32, 16, 2, [282.0, 287.0], seed=51, geometry="blobs",
                  angles=(0.0, 150.0, 30.0))
CASE_NN3 = cases.Case("iso_blobs_nn_3mat", 40, 40, 16, 3, [285.0], seed=52, geometry="blobs",
                      interpolation=cases.NN, angles=(0.0, 120.0, 40.0))
TOL = 1e-5


def _run(case, optical, vox):
    out, _ = oracle.run_arrays(nx=case.nx, ny=case.ny, nz=case.nz, energies=case.energies, optical=optical,
                               voxels=vox, angles=case.angles, phys_size=case.phys_size,
                               interpolation=case.interpolation)
    return out


def _max_rel(a, ref, thr=1e-6):
    assert np.array_equal(np.isnan(a), np.isnan(ref))
    both = ~np.isnan(ref)
    peak = np.abs(ref[both]).max()
    sel = both & (np.abs(ref) > thr * peak)
    assert sel.sum() > 100
    return float((np.abs(a[sel] - ref[sel]) / np.abs(ref[sel])).max())


def _base(case):
    n2 = cases.n2_from_constants(cases.optical_constants(case))
    return n2, cases.isotropic_voxels(case)


@pytest.mark.parametrize("case", [CASE, CASE_NN3], ids=lambda c: c.name)
def test_patterns_scale_with_the_square_of_the_contrast(case):
    n2, vox = _base(case)
    c = 1.6 * np.exp(0.7j)
    ref = _run(case, cases.constants_from_n2(n2), vox)
    got = _run(case, cases.constants_from_n2(1.0 + c * (n2 - 1.0)), vox)
    assert _max_rel(got, abs(c) ** 2 * ref) <= TOL


@pytest.mark.parametrize("case", [CASE, CASE_NN3], ids=lambda c: c.name)
def test_a_common_index_offset_changes_nothing(case):
    n2, vox = _base(case)
    ref = _run(case, cases.constants_from_n2(n2), vox)
    got = _run(case, cases.constants_from_n2(n2 + (-3e-3 + 1.5e-3j)), vox)
    assert _max_rel(got, ref) <= TOL


def test_exchanging_two_materials_with_their_constants_changes_nothing():
    n2, vox = _base(CASE)
    opt = cases.constants_from_n2(n2)
    ref = _run(CASE, opt, vox)
    got = _run(CASE, opt[:, ::-1].copy(), vox[::-1].copy())
    assert _max_rel(got, ref) <= TOL


def test_contrast_free_morphology_scatters_nothing_but_nan_mask():
    # equal constants in both materials: p is a constant field, removed with the DC bin
    n2, vox = _base(CASE)
    same = np.repeat(n2[:, :1], 2, axis=1)
    out = _run(CASE, cases.constants_from_n2(same), vox)
    ref = _run(CASE, cases.constants_from_n2(n2), vox)
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    peak = np.nanmax(np.abs(ref))
    assert np.nanmax(np.abs(out)) <= 1e-9 * peak
