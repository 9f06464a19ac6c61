"""HDF5 subset reader/writer for the CyRSoXS file formats (no libhdf5):
round trips, the reference's output layouts, the drop-in readFromH5, and the
reference's own example morphology when it is available."""
import os

import numpy as np
import pytest

from cyrsoxs_gb300 import h5io
from reference_tree import reference_file

REF_FIXTURE = reference_file("Data", "edgeSphereZYX.h5")


def test_round_trip_datasets_groups_and_labels(tmp_path):
    rng = np.random.default_rng(0)
    a = rng.standard_normal((3, 4, 5)).astype(np.float32)
    b = rng.standard_normal((2, 3)).astype(np.float64)
    n = np.array([7], np.int32)
    p = str(tmp_path / "t.h5")
    h5io.write(p, {"g1/a": (a, ["Z", "Y", "X"]), "g1/sub/b": b, "n": n})
    f = h5io.File(p)
    assert f.keys("/") == ["g1", "n"] and f.keys("g1") == ["a", "sub"]
    np.testing.assert_array_equal(f.read("g1/a"), a)
    np.testing.assert_array_equal(f.read("g1/sub/b"), b)
    assert f.read("n")[0] == 7 and f.labels("g1/a") == ["Z", "Y", "X"] and f.labels("n") is None


def test_group_with_many_members(tmp_path):
    p = str(tmp_path / "many.h5")
    h5io.write(p, {f"Material_{m}/S": np.full((2, 2, 2), m, np.float32) for m in range(1, 33)})
    f = h5io.File(p)
    assert len(f.keys("/")) == 32
    assert f.read("Material_17/S")[1, 1, 1] == 17


def _euler_file(path, order):
    rng = np.random.default_rng(1)
    Z, Y, X = 4, 6, 5
    ds = {"Morphology_Parameters/PhysSize": np.array([2.5]), "Morphology_Parameters/NumMaterial": np.array([2], np.int32)}
    want = np.zeros((2, Z, Y, X, 4), np.float32)
    for m in (1, 2):
        comp = {k: rng.random((Z, Y, X)).astype(np.float64) for k in ("Vfrac", "S", "Theta", "Psi")}
        comp["S"][0, 0, :] = 0.0
        for c, k in enumerate(("S", "Theta", "Psi", "Vfrac")):
            want[m - 1, ..., c] = comp[k]
        want[m - 1, 0, 0, :, 1:3] = 0.0  # theta, psi zeroed where S = 0
        for k, v in comp.items():
            if order == "ZYX":
                ds[f"Euler_Angles/Mat_{m}_{k}"] = (v, ["Z", "Y", "X"])
            else:
                ds[f"Euler_Angles/Mat_{m}_{k}"] = (np.ascontiguousarray(v.transpose(2, 1, 0)), ["X", "Y", "Z"])
    h5io.write(path, ds)
    return want


@pytest.mark.parametrize("order", ["ZYX", "XYZ"])
def test_read_morphology_euler_orders(tmp_path, order):
    p = str(tmp_path / "m.h5")
    want = _euler_file(p, order)
    m = h5io.read_morphology(p, 0)
    assert m.num_material == 2 and m.phys_size == 2.5 and m.dims_xyz == (5, 6, 4)
    assert m.order == (0 if order == "ZYX" else 1)  # MorphologyOrder ZYX = 0, XYZ = 1
    np.testing.assert_array_equal(m.voxels, want)


def test_scattering_files_follow_the_reference_layout(tmp_path):
    from cyrsoxs_gb300 import CyRSoXS as cy

    inp = cy.InputData(NumMaterial=1)
    inp.setEnergies([280.0, 285.5])
    inp.setDimensions([4, 6, 5], cy.MorphologyOrder.ZYX)
    data = np.arange(2 * 6 * 5, dtype=np.float32)
    h5io.write_scattering(inp, data, str(tmp_path / "HDF5"))
    assert sorted(os.listdir(tmp_path / "HDF5")) == ["Energy_280.00.h5", "Energy_285.50.h5"]
    f = h5io.File(str(tmp_path / "HDF5" / "Energy_285.50.h5"))
    np.testing.assert_array_equal(f.read("K0/projection"), data[30:].reshape(6, 5))
    assert f.labels("K0/projection") == ["Qy", "Qx"]
    np.testing.assert_array_equal(f.read("KIDList/KVec"), np.array([[0, 0, 1]], np.float32))


def test_drop_in_read_from_h5(tmp_path, capsys):
    from cyrsoxs_gb300 import CyRSoXS as cy

    p = str(tmp_path / "m.h5")
    want = _euler_file(p, "ZYX")
    inp = cy.InputData(NumMaterial=2)
    inp.setDimensions([4, 6, 5], cy.MorphologyOrder.ZYX)
    inp.setPhysSize(2.5)
    inp.setMorphologyType(cy.MorphologyType.EulerAngles)
    vd = cy.VoxelData(InputData=inp)
    vd.readFromH5(Filename=p)
    assert vd.validate()
    np.testing.assert_array_equal(vd.data().reshape(want.shape), want)
    inp2 = cy.InputData(NumMaterial=2)
    inp2.setDimensions([4, 6, 5], cy.MorphologyOrder.ZYX)
    inp2.setPhysSize(3.0)
    inp2.setMorphologyType(cy.MorphologyType.EulerAngles)
    cy.VoxelData(InputData=inp2).readFromH5(Filename=p)
    assert "PhysSize mismatch" in capsys.readouterr().out


@pytest.mark.skipif(REF_FIXTURE is None, reason="the reference's example morphology is not here")
def test_reads_the_reference_example_morphology():
    m = h5io.read_morphology(REF_FIXTURE, 1)  # vector morphology, ZYX
    assert m.num_material == 2 and m.phys_size == 5.0 and m.order == 0 and m.dims_xyz == (32, 32, 16)
    v = m.voxels
    assert v.shape == (2, 16, 32, 32, 4) and np.isfinite(v).all()
    # alignment vectors are unit or zero length; fractions in [0, 1]
    s = np.linalg.norm(v[..., :3], axis=-1)
    assert s.max() <= 1.0 + 1e-6 and v[..., 3].min() >= -1e-6 and v[..., 3].max() <= 1.0 + 1e-6
