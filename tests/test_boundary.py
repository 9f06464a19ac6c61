"""The C ABI boundary and the host-side logic, without a GPU.

* every function include/cyrsoxs.h declares is exported by the library;
* the ctypes mirror of struct cyr_options has the C layout;
* with no CUDA device the engine fails loudly (no CPU fallback);
* the drop-in CyRSoXS API reproduces the reference's host-side behaviour
  (setters, validation messages, voxel layout rules, numpy view quirks).
"""
import ctypes
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cyrsoxs.h")


def _native():
    from cyrsoxs_gb300 import _native

    try:
        _native.lib()
    except Exception as exc:  # pragma: no cover - needs nvcc or a prebuilt library
        pytest.skip(f"native library unavailable: {exc}")
    return _native


def declared_functions():
    text = open(HEADER).read()
    return re.findall(r"CYR_API\s+[\w\s\*]*?\b(cyr_\w+)\s*\(", text)


def test_header_declares_the_boundary():
    names = declared_functions()
    for want in ("cyr_cuda_main", "cyr_cuda_main_streams", "cyr_compute_polarization", "cyr_simulate_device",
                 "cyr_last_error"):
        assert want in names


def test_python_binding_covers_every_declared_symbol():
    """Every entry point the header declares has a ctypes signature in the Python binding."""
    src = "".join(open(os.path.join(ROOT, "cyrsoxs_gb300", f)).read() for f in ("_native.py", "serving.py"))
    missing = [n for n in declared_functions() if n not in src]
    assert not missing, missing


def test_library_exports_every_declared_symbol():
    nat = _native()
    L = ctypes.CDLL(nat.library_path())
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_fft_entry_points_refuse_volumes_beyond_32_bit_offsets():
    """Both FFT entry points refuse a volume of 2^32 or more elements before touching the device
    (the pointer is never dereferenced: the size check comes first)."""
    nat = _native()
    for fn in (nat.fft3d_device, nat.fft3d_device_static):
        with pytest.raises(nat.CyrError) as ei:
            fn(16, 4096, 4096, 256)
        assert ei.value.code == 1 and "2^32" in str(ei.value)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_options_struct_layout_matches_header(tmp_path):
    nat = _native()
    fields = [f for f, _ in nat.CyrOptions._fields_]
    src = tmp_path / "lay.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"cyrsoxs.h\"\nint main(void){\n"
                   f'printf("%zu\\n", sizeof(cyr_options));\n'
                   + "".join(f'printf("%zu\\n", offsetof(cyr_options, {f}));\n' for f in fields) + "return 0;}\n")
    exe = tmp_path / "lay"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == ctypes.sizeof(nat.CyrOptions)
    assert vals[1:] == [getattr(nat.CyrOptions, f).offset for f in fields]


def test_without_gpu_the_engine_fails_loudly():
    nat = _native()
    if nat.device_count() > 0:
        pytest.skip("a GPU is visible")
    opts = nat.Options(nx=8, ny=8, nz=4, num_material=1, energies=[285.0], start_angle=0, end_angle=0,
                       increment_angle=0, phys_size=5.0)
    with pytest.raises(nat.CyrError) as ei:
        nat.cuda_main(opts, np.zeros((1, 1, 4), np.float32), np.zeros((1, 4, 8, 8, 4), np.float32))
    assert ei.value.code == 5  # CYR_ERR_NO_DEVICE


def test_host_arrays_of_the_wrong_size_or_type_are_refused_before_the_engine_reads_them():
    nat = _native()
    opts = nat.Options(nx=8, ny=8, nz=4, num_material=2, energies=[285.0, 286.0], start_angle=0, end_angle=0,
                       increment_angle=0, phys_size=5.0)
    opt = np.zeros((2, 2, 4), np.float32)
    vox = np.zeros((2, 4, 8, 8, 4), np.float32)
    with pytest.raises(ValueError, match="optical constants"):
        nat.cuda_main(opts, opt[:1], vox)
    with pytest.raises(ValueError, match="voxels"):
        nat.cuda_main(opts, opt, vox[:1])
    with pytest.raises(ValueError, match="out"):
        nat.cuda_main(opts, opt, vox, out=np.zeros((1, 1, 8, 8), np.float32))
    with pytest.raises(TypeError, match="out"):
        nat.cuda_main(opts, opt, vox, out=np.zeros((2, 1, 8, 8), np.float64))
    with pytest.raises(TypeError, match="out"):
        nat.cuda_main(opts, opt, vox, out=np.zeros((2, 1, 8, 16), np.float32)[..., ::2])
    with pytest.raises(ValueError, match="voxels"):
        nat.compute_polarization(opts, opt, vox[:, :2], 0.0, 0)
    with pytest.raises(ValueError, match="optical constants"):
        nat.simulate_device(opts, opt[:, :1], 0, 0)
    # other dtypes and layouts of the inputs are converted, not refused
    if nat.device_count() == 0:
        with pytest.raises(nat.CyrError) as ei:
            nat.cuda_main(opts, opt.astype(np.float64), np.asfortranarray(vox))
        assert ei.value.code == 5


def test_invalid_options_are_rejected_before_any_device_work():
    nat = _native()
    opts = nat.Options(nx=8, ny=8, nz=4, num_material=1, energies=[285.0], start_angle=10, end_angle=0,
                       increment_angle=1, phys_size=5.0)
    with pytest.raises(nat.CyrError) as ei:
        nat.required_device_bytes(opts)
    assert ei.value.code == 1
    bad = nat.Options(nx=4099, ny=8, nz=4, num_material=1, energies=[285.0], start_angle=0, end_angle=0,
                      increment_angle=0, phys_size=5.0)  # prime, beyond the Bluestein limit
    with pytest.raises(nat.CyrError) as ei:
        nat.required_device_bytes(bad)
    assert ei.value.code == 2


GOOD = dict(nx=16, ny=16, nz=8, num_material=2, energies=[285.0], start_angle=0.0, end_angle=90.0,
            increment_angle=30.0, phys_size=5.0)


@pytest.mark.parametrize("over,code,words", [
    (dict(nx=1), 1, "dimensions"),
    (dict(ny=1), 1, "dimensions"),
    (dict(nz=0), 1, "dimensions"),
    (dict(num_material=0), 1, "num_material"),
    (dict(num_material=33), 1, "num_material"),
    (dict(energies=[]), 1, "no energies"),
    (dict(energies=[285.0, 0.0]), 1, "energies must be positive"),
    (dict(energies=[float("nan")]), 1, "energies must be positive"),
    (dict(phys_size=0.0), 1, "phys_size"),
    (dict(phys_size=float("nan")), 1, "phys_size"),
    (dict(case_type=3), 1, "case_type"),
    (dict(ewald_interpolation=2), 1, "enumerated"),
    (dict(reference_frame=2), 1, "enumerated"),
    (dict(strategy=3), 1, "enumerated"),
    (dict(start_angle=90.0, end_angle=0.0), 1, "start angle"),
    (dict(increment_angle=0.0), 1, "increment angle is 0"),
    (dict(end_angle=4096.0, increment_angle=0.5), 1, "angle count"),
    (dict(nz=2053), 2, "Bluestein limit"),  # prime: its padded length would exceed one block's FFT
    (dict(nx=6561, ny=2, nz=1), 2, "single-block FFT limit"),  # 3^8: factorable, above one block
    (dict(nx=2048, ny=2048, nz=1024), 2, "2^32"),  # 2^32 voxels: beyond 32-bit offsets in a volume
], ids=lambda v: str(v) if not isinstance(v, dict) else ",".join(f"{k}={w}" for k, w in v.items()))
def test_each_invalid_option_is_rejected_with_its_reason(over, code, words):
    nat = _native()
    with pytest.raises(nat.CyrError) as ei:
        nat.required_device_bytes(nat.Options(**{**GOOD, **over}))
    assert ei.value.code == code
    assert words in str(ei.value)


def test_edge_shapes_that_are_valid_plan_on_the_host():
    nat = _native()
    for over in (dict(nz=1), dict(nx=2, ny=2, nz=1), dict(num_material=32), dict(start_angle=30.0, end_angle=30.0,
                                                                                   increment_angle=0.0),
                 dict(nx=7, ny=5, nz=3), dict(end_angle=4095.0, increment_angle=1.0),
                 # lengths with a prime factor above 7 run as Bluestein transforms
                 dict(nx=101, ny=97, nz=13), dict(nx=2039, ny=2, nz=1), dict(nx=22, ny=8, nz=4)):
        assert nat.required_device_bytes(nat.Options(**{**GOOD, **over})) > 0


def test_required_bytes_counts_the_tensor_volumes():
    nat = _native()
    opts = nat.Options(nx=64, ny=64, nz=16, num_material=2, energies=[280.0, 285.0], start_angle=0, end_angle=165,
                       increment_angle=15, phys_size=5.0)
    b = nat.required_device_bytes(opts)
    # 5 complex tensor volumes, pruned to at least the 3 planes around the DC bin, 12 images and the
    # trigonometry-free copy of the Euler morphology (2 materials x float4)
    conv = 2 * 64 * 64 * 16 * 16
    lo = 5 * 3 * 64 * 64 * 8 + 12 * 64 * 64 * 4 + conv
    assert lo <= b <= lo + 5 * 64 * 64 * 16 * 8 + (1 << 20)


# ---------------------------------------------------------------------------
# drop-in API host logic
# ---------------------------------------------------------------------------
def cy():
    from cyrsoxs_gb300 import CyRSoXS

    return CyRSoXS


def make_input(M=2, dims=(4, 8, 6), order=None):
    c = cy()
    inp = c.InputData(NumMaterial=M)
    inp.setCaseType(c.CaseType.Default)
    inp.setEnergies([285.0, 280.0])
    inp.setERotationAngle(StartAngle=0, EndAngle=90, IncrementAngle=30)
    inp.setDimensions(list(dims), order if order is not None else c.MorphologyOrder.ZYX)
    inp.setMorphologyType(c.MorphologyType.EulerAngles)
    inp.setPhysSize(5.0)
    return inp


from reference_tree import reference_file  # noqa: E402

REF_PYMAIN = reference_file("src", "pymain.cpp")


@pytest.mark.skipif(REF_PYMAIN is None, reason="the reference's pybind11 module source is not here")
def test_module_exposes_every_name_the_reference_binds():
    """Every class, enum value, method and property src/pymain.cpp binds exists in the drop-in."""
    c = cy()
    src = open(REF_PYMAIN).read()
    instances = {"InputData": lambda: c.InputData(NumMaterial=2)}
    missing, seen = [], 0
    for block in re.split(r"(?=py::(?:class_|enum_)<)", src)[1:]:
        m = re.match(r'py::(?:class_|enum_)<[^>]*>\s*\(\s*\w+\s*,\s*"(\w+)"', block)
        if not m:
            continue
        name = m.group(1)
        body = block[:block.find(";")]
        members = re.findall(r'\.def(?:_readwrite|_readonly|_property\w*)?\(\s*"(\w+)"', body)
        members += re.findall(r'\.value\(\s*"(\w+)"', body)
        obj = getattr(c, name, None)
        if obj is None:
            missing.append(name)
            continue
        inst = instances[name]() if name in instances else None
        for n in members:
            seen += 1
            if not hasattr(obj, n) and not (inst is not None and hasattr(inst, n)):
                missing.append(f"{name}.{n}")
    for n in re.findall(r'\b(?:m|module)\.def\(\s*"(\w+)"', src):
        seen += 1
        if not hasattr(c, n):
            missing.append(n)
    assert seen > 50 and not missing, missing


def test_input_data_setters_follow_the_reference(capsys):
    c = cy()
    inp = make_input()
    assert inp.energies == [280.0, 285.0]  # sorted (InputData.h:443)
    assert inp.voxelDims == [6, 8, 4]  # ZYX dims stored as X, Y, Z
    assert inp.validate()
    inp2 = c.InputData(NumMaterial=1)
    assert not inp2.validate()
    assert "is not set" in capsys.readouterr().out
    inp2.setEnergies([280.0, 280.0])
    assert "duplicate" in capsys.readouterr().out
    inp2.setERotationAngle(StartAngle=10, EndAngle=0, IncrementAngle=1)
    assert "Start EAngle" in capsys.readouterr().out
    inp2.setERotationAngle(StartAngle=5, EndAngle=5, IncrementAngle=0)
    assert inp2.incrementAngle == 1.0
    inp2.setCaseType(c.CaseType.BeamDivergence)
    inp2.setKVectors([0.0, 3.0, 4.0])
    np.testing.assert_allclose(inp2.kVectors[-1], [0.0, 0.6, 0.8], rtol=1e-6)


def test_refractive_index_rejects_unknown_energy(capsys):
    c = cy()
    inp = make_input()
    ri = c.RefractiveIndex(inp)
    ri.addData(OpticalConstants=[[1e-3, 2e-4, 1e-3, 2e-4]] * 2, Energy=281.0)
    assert "Bad Energy" in capsys.readouterr().out
    assert not ri.validate()
    for e in (280.0, 285.0):
        ri.addData(OpticalConstants=[[1e-3, 2e-4, 1e-3, 2e-4]] * 2, Energy=e)
    assert ri.validate()


def test_voxel_data_euler_zeroes_angles_where_s_is_zero():
    c = cy()
    inp = make_input(M=1)
    vd = c.VoxelData(InputData=inp)
    shape = (4, 8, 6)
    S = np.zeros(shape, np.float32)
    S[0, 0, 0] = 0.5
    th = np.full(shape, 1.0, np.float32)
    vd.addVoxelData(S, th, th, np.ones(shape, np.float32), 1)
    v = vd.data()[0]
    assert v[0, 1] == 1.0 and v[1, 1] == 0.0 and v[1, 2] == 0.0
    assert vd.validate()


def test_voxel_data_xyz_order_is_transposed_to_zyx():
    c = cy()
    inp = make_input(M=1, dims=(6, 8, 4), order=c.MorphologyOrder.XYZ)
    inp.setMorphologyType(c.MorphologyType.VectorMorphology)
    vd = c.VoxelData(InputData=inp)
    X, Y, Z = 6, 8, 4
    al = np.arange(X * Y * Z * 3, dtype=np.float32).reshape(X, Y, Z, 3)
    un = np.arange(X * Y * Z, dtype=np.float32).reshape(X, Y, Z)
    vd.addVoxelData(AlignedData=al, UnalignedData=un, MaterialID=1)
    v = vd.data()[0].reshape(Z, Y, X, 4)
    assert v[2, 3, 1, 3] == un[1, 3, 2]
    np.testing.assert_array_equal(v[2, 3, 1, :3], al[1, 3, 2])


def test_voxel_data_rejects_bad_material_and_nan(capsys):
    c = cy()
    inp = make_input(M=1)
    vd = c.VoxelData(InputData=inp)
    with pytest.raises(RuntimeError):
        vd.addVoxelData(np.ones((4, 8, 6), np.float32), 2)
    vf = np.ones((4, 8, 6), np.float32)
    vf[0, 0, 0] = np.nan
    vd.addVoxelData(vf, 1)
    assert not vd.validate()
    assert "Nan" in capsys.readouterr().out


def test_scattering_pattern_views_keep_the_reference_strides():
    c = cy()
    inp = make_input(dims=(4, 8, 6))
    sp = c.ScatteringPattern(inp)
    X, Y = 6, 8
    sp.data()[:] = np.arange(sp.data().size, dtype=np.float32)
    v = sp.dataToNumpy(285.0, 0)
    assert v.shape == (Y, X) and v.strides == (4 * Y, 4)
    assert v[0, 0] == X * Y  # second energy starts after one [Ny][Nx] image
    allv = sp.writeAllToNumpy(kID=0)
    assert allv.shape == (2, Y, X)
    assert sp.dataToNumpy(281.0, 0).size == 0
