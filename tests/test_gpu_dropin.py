"""The drop-in CyRSoXS module end to end on the GPU, used the way the
reference's notebook uses its pybind11 module (setters, addData, addVoxelData,
launch, dataToNumpy), against the FP64 oracle within the parity tolerance."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-4


def test_notebook_style_workflow_matches_the_oracle():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cyrsoxs_gb300 import CyRSoXS as cy

    Z, Y, X = 8, 32, 32  # square: the reference's dataToNumpy view (row stride Ny) is valid only then
    energies = [284.0, 285.0, 286.5]
    inp = cy.InputData(NumMaterial=2)
    inp.setEnergies(energies)
    inp.setERotationAngle(StartAngle=0.0, EndAngle=150.0, IncrementAngle=30.0)
    inp.setPhysSize(5.0)
    inp.setDimensions([Z, Y, X], cy.MorphologyOrder.ZYX)
    inp.setMorphologyType(cy.MorphologyType.EulerAngles)
    inp.setCaseType(cy.CaseType.Default)  # also sets the k vector and the detector, as the reference's setter does
    inp.interpolationType = cy.InterpolationType.Linear
    assert inp.validate()

    rng = np.random.default_rng(11)
    optical = np.zeros((len(energies), 2, 4), np.float32)
    ri = cy.RefractiveIndex(inp)
    for i, e in enumerate(energies):
        optical[i] = 1e-3 * (1 + rng.random((2, 4)))
        ri.addData(OpticalConstants=optical[i].tolist(), Energy=e)
    assert ri.validate()

    vd = cy.VoxelData(InputData=inp)
    vox = np.zeros((2, Z, Y, X, 4), np.float32)
    vf = rng.random((Z, Y, X)).astype(np.float32)
    for m, frac in ((1, vf), (2, 1 - vf)):
        S = rng.random((Z, Y, X)).astype(np.float32)
        th = (rng.random((Z, Y, X)) * np.pi).astype(np.float32)
        ps = (rng.random((Z, Y, X)) * 2 * np.pi).astype(np.float32)
        vd.addVoxelData(S, th, ps, frac, m)
        vox[m - 1] = np.stack([S, th, ps, frac], -1)
    assert vd.validate()

    sp = cy.ScatteringPattern(inp)
    cy.launch(VoxelData=vd, RefractiveIndexData=ri, InputData=inp, ScatteringPattern=sp, WriteMetaData=False)
    want, _ = oracle.run_arrays(nx=X, ny=Y, nz=Z, energies=energies, optical=optical, voxels=vox,
                                angles=(0.0, 150.0, 30.0), phys_size=5.0)
    for i, e in enumerate(energies):
        got = np.array(sp.dataToNumpy(e, 0), np.float64)
        w = want[i, 0]
        assert np.array_equal(np.isnan(got), np.isnan(w))
        ok = ~np.isnan(w)
        sel = ok & (np.abs(w) > 1e-6 * np.abs(w[ok]).max())
        assert (np.abs(got[sel] - w[sel]) / np.abs(w[sel])).max() <= TOL
