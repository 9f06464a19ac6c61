"""The reference's C++ entry points over the engine's C ABI
(cyrsoxs_gb300/csrc/cudaMain_shim.cpp).

* CPU: the shim compiles against the reference's own headers
  (include/cudaMain.h:53-87) and defines cudaMain, cudaMainStreams and
  computePolarization with exactly the reference's signatures; linked with the
  reference's harness and RotationMatrix.cpp it needs libcyrsoxs_gb300.so and
  none of cuFFT, NPP or cuBLAS.
* GPU: the reference's harness (oracle/ref/ref_driver.cpp, which drives the
  reference the way its pybind11 front end does) runs golden cases through the
  shim.  The shim hands the engine (delta, beta) as 1 - Re n, the exact value
  the reference's float n = 1 - delta + i beta represents
  (include/PyClass/RefractiveIndex.h:101-106), so the oracle is run on those
  same constants.  Tolerance: max relative error <= 1e-4 over pixels above
  1e-6 of the peak, identical NaN masks (projections); <= 1e-5 of the largest
  component (polarization).
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import cases
import oracle
from reference_tree import reference_tree

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "cyrsoxs_gb300", "csrc", "cudaMain_shim.cpp")
SHIM_BIN = os.path.join(ROOT, "oracle", "_ref", "cyrsoxs_gb300_shim_fp32")
GOLDEN = os.path.dirname(cases.__file__)
TREE = reference_tree()
NVCC = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)

SIGNATURES = [
    "cudaMain(unsigned int const*, InputData const&, std::vector<Material, std::allocator<Material> > const&, "
    "float*, RotationMatrix&, Voxel const*)",
    "cudaMainStreams(unsigned int const*, InputData const&, std::vector<Material, std::allocator<Material> > const&, "
    "float*, RotationMatrix&, Voxel const*)",
    "computePolarization(unsigned int const*, InputData const&, std::vector<Material, std::allocator<Material> > "
    "const&, float2*, float2*, float2*, RotationMatrix&, Voxel const*, float, unsigned int, int)",
]


def _flags():
    return ["-std=c++17", "-O2", "-DPYBIND", "-DMAX_NUM_MATERIAL=32", "-I", os.path.join(TREE, "include"),
            "-I", os.path.join(ROOT, "oracle", "ref", "stub"), "-I", os.path.join(ROOT, "include"),
            "-include", os.path.join(ROOT, "oracle", "ref", "npp_stream_shim.h"), "-w"]


@pytest.mark.skipif(TREE is None or NVCC is None, reason="needs the reference's headers and nvcc")
def test_shim_defines_the_reference_signatures():
    with tempfile.TemporaryDirectory() as tmp:
        obj = os.path.join(tmp, "shim.o")
        subprocess.run([NVCC, "-c", *_flags(), SHIM, "-o", obj], check=True)
        syms = subprocess.run(["nm", "-C", obj], capture_output=True, text=True, check=True).stdout
    defined = [ln.split(" T ", 1)[1].strip() for ln in syms.splitlines() if " T " in ln]
    for sig in SIGNATURES:
        assert sig in defined, (sig, defined)


@pytest.mark.skipif(TREE is None or NVCC is None, reason="needs the reference's headers and nvcc")
def test_harness_links_through_the_shim_without_cufft_or_npp():
    from cyrsoxs_gb300 import build

    lib = build.build()
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "h")
        subprocess.run([NVCC, *_flags(), os.path.join(TREE, "src", "RotationMatrix.cpp"),
                        os.path.join(ROOT, "oracle", "ref", "ref_driver.cpp"), SHIM, "-L", os.path.dirname(lib),
                        "-lcyrsoxs_gb300", "-Xcompiler", "-fopenmp", "-o", exe], check=True)
        needed = subprocess.run(["readelf", "-d", exe], capture_output=True, text=True, check=True).stdout
    assert "libcyrsoxs_gb300.so" in needed
    for closed in ("cufft", "nppi", "nppc", "cublas"):
        assert closed not in needed, closed


def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not os.path.exists(SHIM_BIN):
        pytest.skip("the shim harness was not built (the reference sources are not staged)")


def _as_reference_sees_it(optical):
    """(delta, beta) as the reference's float n = 1 - delta + i beta holds them: delta -> 1 - fl(1 - delta)."""
    o = np.array(optical, np.float32)
    for c in (0, 2):
        o[..., c] = np.float32(1.0) - (np.float32(1.0) - o[..., c])
    return o


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["euler_sphere", "alg1_streams", "four_materials", "vector_nn_full"])
def test_reference_harness_through_the_shim_matches_oracle(name):
    _gpu()
    case = cases.CASES[name]
    with tempfile.TemporaryDirectory() as tmp:
        cpath, opath, rpath = (os.path.join(tmp, n) for n in ("c.case", "o.bin", "r.case"))
        cases.write_case(case, cpath)
        p = subprocess.run([SHIM_BIN, cpath, opath], capture_output=True, text=True, timeout=600)
        assert p.returncode == 0, p.stdout + p.stderr
        shape = cases.output_shape(case)
        got = np.fromfile(opath, np.float32).reshape(shape).astype(np.float64)
        cases.write_case_arrays(case, rpath, _as_reference_sees_it(cases.optical_constants(case)), cases.voxels(case))
        want, _ = oracle.run_case_file(rpath, shape)
    r32 = np.fromfile(f"{GOLDEN}/ref_{name}_fp32.bin", np.float32).reshape(shape)
    assert np.array_equal(np.isnan(got), np.isnan(want)), "NaN mask differs from the FP64 oracle"
    assert np.array_equal(np.isnan(got), np.isnan(r32)), "NaN mask differs from the reference FP32 build"
    both = ~np.isnan(want)
    peak = np.abs(want[both]).max()
    sel = both & (np.abs(want) > 1e-6 * peak)
    err = (np.abs(got[sel] - want[sel]) / np.abs(want[sel])).max()
    assert err <= 1e-4, err


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["pol_euler", "pol_vector"])
def test_compute_polarization_through_the_shim_matches_oracle(name):
    _gpu()
    case = cases.CASES[name]
    shape = (3, case.nz, case.ny, case.nx)
    with tempfile.TemporaryDirectory() as tmp:
        cpath, opath, rpath = (os.path.join(tmp, n) for n in ("c.case", "o.bin", "r.case"))
        cases.write_case(case, cpath)
        p = subprocess.run([SHIM_BIN, cpath, opath], capture_output=True, text=True, timeout=600)
        assert p.returncode == 0, p.stdout + p.stderr
        got = np.fromfile(opath, np.complex64).reshape(shape).astype(np.complex128)
        cases.write_case_arrays(case, rpath, _as_reference_sees_it(cases.optical_constants(case)), cases.voxels(case))
        want = oracle.polarization_case_file(rpath, shape)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()
