"""config.txt / Material<N>.txt readers (libconfig subset) and the command
line's host logic, without a GPU."""
import os

import numpy as np
import pytest

from cyrsoxs_gb300 import cli, config, h5io
from reference_tree import reference_file

REF_DATA = reference_file("Data")

CONFIG = """# a comment
CaseType = 1;
Energies = [285.0, 280.5]
EAngleRotation=[10.0, 5.0, 40.0];   // start, increment, end
MorphologyType: 0
RotMask = 1;
Algorithm = 1; MaxStreams = 2;
/* block
   comment */
HDF5DirName = "out dir";
listKVectors = (
  { k = [0.0, 3.0, 4.0]; },
  { k = [1.0, 0.0, 0.0] }
);
"""


def material(energies, scale):
    groups = []
    for i, e in enumerate(energies):
        groups.append(f"EnergyData{i}:\n{{\nEnergy = {e};\nBetaPara = {1e-4 * scale};\nBetaPerp = {2e-4 * scale};\n"
                      f"DeltaPara = {3e-4 * scale};\nDeltaPerp = {4e-4 * scale};\n}}\n")
    return "".join(groups)


def test_parser_covers_the_libconfig_subset():
    cfg = config.parse(CONFIG)
    assert cfg["Energies"] == [285.0, 280.5] and cfg["MorphologyType"] == 0 and cfg["MaxStreams"] == 2
    assert cfg["HDF5DirName"] == "out dir" and cfg["listKVectors"][1]["k"] == [1.0, 0.0, 0.0]
    with pytest.raises(config.ConfigError):
        config.parse("A = [1, 2")


def test_read_config_follows_the_reference_constructor(tmp_path):
    p = tmp_path / "config.txt"
    p.write_text(CONFIG)
    c = config.read_config(str(p))
    assert (c["startAngle"], c["incrementAngle"], c["endAngle"]) == (10.0, 5.0, 40.0)
    assert c["caseType"] == 1 and c["rotMask"] == 1 and c["algorithmType"] == 1 and c["numMaxStreams"] == 2
    np.testing.assert_allclose(c["kVectors"][0], [0.0, 0.6, 0.8], rtol=1e-6)
    assert c["ewaldsInterpolation"] == 1 and c["windowingType"] == 0 and c["referenceFrame"] == 1
    p.write_text("CaseType=0\nEnergies=[280.0]\nEAngleRotation=[5.0, 0.0, 5.0]\nMorphologyType=0\n")
    c = config.read_config(str(p))
    assert c["incrementAngle"] == 1.0 and c["kVectors"] == [[0.0, 0.0, 1.0]]
    p.write_text("CaseType=0\nEnergies=[280.0]\nEAngleRotation=[5.0, 0.0, 6.0]\nMorphologyType=0\n")
    with pytest.raises(config.ConfigError, match="Increment angle"):
        config.read_config(str(p))


def test_read_materials(tmp_path):
    (tmp_path / "Material1.txt").write_text(material([285.0, 280.5], 1))
    (tmp_path / "Material2.txt").write_text(material([285.0, 280.5], 2))
    opt = config.read_materials(2, [285.0, 280.5], str(tmp_path))
    assert opt.shape == (2, 2, 4)
    np.testing.assert_allclose(opt[1, 1], [6e-4, 2e-4, 8e-4, 4e-4], rtol=1e-6)
    with pytest.raises(config.ConfigError, match="No energy found"):
        config.read_materials(2, [285.0, 281.0], str(tmp_path))


@pytest.mark.skipif(REF_DATA is None, reason="the reference's example inputs are not here")
def test_reads_the_reference_example_inputs():
    c = config.read_config(os.path.join(REF_DATA, "config.txt"))
    assert c["energies"] == [280.0] and c["morphologyType"] == 1
    cfg = config.parse_file(os.path.join(REF_DATA, "Material0.txt"))
    assert cfg["EnergyData0"]["Energy"] == 280.0


def make_run_dir(d, nmat=2, dims=(8, 16, 12)):
    """A morphology, config.txt and Material<N>.txt in directory d."""
    Z, Y, X = dims
    rng = np.random.default_rng(3)
    ds = {"Morphology_Parameters/PhysSize": np.array([5.0]),
          "Morphology_Parameters/NumMaterial": np.array([nmat], np.int32)}
    vf = rng.random((nmat, Z, Y, X))
    vf /= vf.sum(0)
    for m in range(1, nmat + 1):
        ds[f"Euler_Angles/Mat_{m}_Vfrac"] = (vf[m - 1], ["Z", "Y", "X"])
        ds[f"Euler_Angles/Mat_{m}_S"] = (rng.random((Z, Y, X)), ["Z", "Y", "X"])
        ds[f"Euler_Angles/Mat_{m}_Theta"] = (rng.random((Z, Y, X)) * np.pi, ["Z", "Y", "X"])
        ds[f"Euler_Angles/Mat_{m}_Psi"] = (rng.random((Z, Y, X)) * 2 * np.pi, ["Z", "Y", "X"])
    h5io.write(os.path.join(d, "morph.h5"), ds)
    with open(os.path.join(d, "config.txt"), "w") as f:
        f.write("CaseType=0;\nEnergies=[284.0, 286.0];\nEAngleRotation=[0.0, 30.0, 150.0];\nMorphologyType=0;\n")
    for m in range(1, nmat + 1):
        with open(os.path.join(d, f"Material{m}.txt"), "w") as f:
            f.write(material([284.0, 286.0], m))


def test_cli_without_a_gpu_fails_loudly(tmp_path, monkeypatch, capsys):
    from cyrsoxs_gb300 import _native

    try:
        _native.lib()
    except Exception as exc:  # pragma: no cover
        pytest.skip(f"native library unavailable: {exc}")
    if _native.device_count() > 0:
        pytest.skip("a GPU is visible")
    make_run_dir(str(tmp_path))
    monkeypatch.chdir(tmp_path)
    assert cli.main(["morph.h5"]) == 1
    assert "no device" in capsys.readouterr().out
    assert cli.main([]) == 1


def test_constants_interpolation_and_material_files(tmp_path):
    from cyrsoxs_gb300 import constants

    table = np.array([[280.0, 1e-3, 1e-4, 2e-3, 2e-4],
                      [282.0, 3e-3, 3e-4, 4e-3, 4e-4],
                      [282.0, 9e-3, 9e-4, 9e-3, 9e-4],   # duplicate energy: the first row is kept
                      [281.0, 2e-3, 2e-4, 3e-3, 3e-4]])
    c = constants.interpolate(table, [280.5, 282.0])
    np.testing.assert_allclose(c[0], [1.5e-3, 1.5e-4, 2.5e-3, 2.5e-4])
    np.testing.assert_allclose(c[1], [3e-3, 3e-4, 4e-3, 4e-4])
    with pytest.raises(ValueError):
        constants.interpolate(table, [279.0])
    constants.write_material(str(tmp_path / "Material1.txt"), [280.5, 282.0], c)
    constants.write_material(str(tmp_path / "Material2.txt"), [280.5, 282.0])  # vacuum
    opt = config.read_materials(2, [280.5, 282.0], str(tmp_path))
    np.testing.assert_allclose(opt[:, 0], c, rtol=1e-6)
    assert not opt[:, 1].any()


def test_morphology_dump_writes_h5_and_xdmf(tmp_path, monkeypatch):
    from cyrsoxs_gb300 import CyRSoXS as cy

    monkeypatch.chdir(tmp_path)
    inp = cy.InputData(NumMaterial=2)
    inp.setDimensions([2, 3, 4], cy.MorphologyOrder.ZYX)
    vox = np.arange(2 * 24 * 4, dtype=np.float32).reshape(2, 24, 4)
    h5io.write_morphology_dump(inp, vox)
    f = h5io.File("Morphology/Morphology.h5")
    np.testing.assert_array_equal(f.read("Material_2/Psi"), vox[1, :, 2].reshape(2, 3, 4))
    x = open("Morphology/Morphology.xdmf").read()
    assert 'NumberOfElements="2 3 4"' in x and "Morphology.h5:/Material_2/Vfrac" in x
