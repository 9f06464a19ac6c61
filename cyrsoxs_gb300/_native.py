"""ctypes binding of the engine's C ABI (include/cyrsoxs.h).

The engine exists only as CUDA code: if the shared library cannot be loaded
this module raises, and nothing falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

CYR_OK = 0
STATUS_NAMES = {0: "ok", 1: "argument", 2: "unsupported", 3: "cuda", 4: "memory", 5: "no device", 6: "timeout"}

_lib = None


class CyrOptions(ctypes.Structure):
    """Mirror of struct cyr_options."""

    _fields_ = [
        ("nx", ctypes.c_uint32), ("ny", ctypes.c_uint32), ("nz", ctypes.c_uint32),
        ("num_material", ctypes.c_uint32),
        ("num_energies", ctypes.c_uint32),
        ("energies", ctypes.POINTER(ctypes.c_float)),
        ("start_angle", ctypes.c_float), ("end_angle", ctypes.c_float), ("increment_angle", ctypes.c_float),
        ("phys_size", ctypes.c_float),
        ("case_type", ctypes.c_uint32),
        ("num_k", ctypes.c_uint32),
        ("k_vectors", ctypes.POINTER(ctypes.c_float)),
        ("detector", ctypes.c_float * 3),
        ("morphology_type", ctypes.c_uint32),
        ("ewald_interpolation", ctypes.c_uint32),
        ("windowing", ctypes.c_uint32),
        ("scatter_approach", ctypes.c_uint32),
        ("algorithm", ctypes.c_uint32),
        ("max_streams", ctypes.c_uint32),
        ("rot_mask", ctypes.c_uint32),
        ("reference_frame", ctypes.c_uint32),
        ("strategy", ctypes.c_uint32),
    ]


class CyrError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"cyrsoxs_gb300 error {code} ({STATUS_NAMES.get(code, '?')}): {message}")
        self.code = code


def library_path() -> str:
    return _build.LIB


def lib():
    """Loads (building first when the library is missing or stale and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    try:
        _build.build()
    except Exception as exc:  # no nvcc on this machine: the library must already exist
        if not os.path.exists(_build.LIB):
            raise RuntimeError(f"cyrsoxs_gb300 native library missing and could not be built: {exc}") from exc
    L = ctypes.CDLL(_build.LIB)
    c_float_p = ctypes.POINTER(ctypes.c_float)
    opt_p = ctypes.POINTER(CyrOptions)
    L.cyr_last_error.restype = ctypes.c_char_p
    L.cyr_version.restype = ctypes.c_char_p
    L.cyr_device_count.restype = ctypes.c_int
    L.cyr_cuda_main.argtypes = [opt_p, c_float_p, c_float_p, c_float_p]
    L.cyr_cuda_main_streams.argtypes = [opt_p, c_float_p, c_float_p, c_float_p]
    L.cyr_compute_polarization.argtypes = [opt_p, c_float_p, c_float_p, ctypes.c_float, ctypes.c_uint32,
                                           c_float_p, c_float_p, c_float_p]
    L.cyr_simulate_device.argtypes = [opt_p, c_float_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.cyr_required_device_bytes.argtypes = [opt_p, ctypes.POINTER(ctypes.c_size_t)]
    L.cyr_fft3d_device.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                   ctypes.c_uint32, ctypes.c_void_p]
    L.cyr_selftest_wait_limit.argtypes = [ctypes.POINTER(ctypes.c_int)]
    L.cyr_fft3d_device_static.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                          ctypes.c_uint32, ctypes.c_void_p]
    L.cyr_warp_affine_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    L.cyr_plan_info.argtypes = [opt_p, ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32]
    L.cyr_device_errors.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
    L.cyr_tuning_report.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.cyr_profile_begin.argtypes = [ctypes.c_uint32]
    L.cyr_profile_end.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                                  ctypes.POINTER(ctypes.c_double), ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
    L.cyr_stage_name.argtypes = [ctypes.c_uint32]
    L.cyr_stage_name.restype = ctypes.c_char_p
    L.cyr_num_stages.restype = ctypes.c_uint32
    L.cyr_release_scratch.argtypes = []
    d_p = ctypes.POINTER(ctypes.c_double)
    L.cyr_cuda_main_fp64.argtypes = [opt_p, d_p, d_p, d_p]
    L.cyr_simulate_device_fp64.argtypes = [opt_p, d_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                           ctypes.c_void_p]
    L.cyr_compute_polarization_fp64.argtypes = [opt_p, d_p, d_p, ctypes.c_double, ctypes.c_uint32, d_p, d_p, d_p]
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != CYR_OK:
        raise CyrError(rc, lib().cyr_last_error().decode(errors="replace"))


def fptr(a: np.ndarray):
    if not isinstance(a, np.ndarray) or a.dtype != np.float32 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float32 numpy array")
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def expect_size(a: np.ndarray, n: int, what: str) -> np.ndarray:
    """a as C-contiguous float32 with exactly n elements: the engine reads or writes that many."""
    if not isinstance(a, np.ndarray) or a.dtype != np.float32 or not a.flags.c_contiguous:
        raise TypeError(f"{what} must be a C-contiguous float32 numpy array")
    if a.size != n:
        raise ValueError(f"{what} has {a.size} elements; these options need {n}")
    return a


def optical_array(opts: "Options", optical) -> np.ndarray:
    s = opts.struct
    return expect_size(np.ascontiguousarray(optical, np.float32), s.num_energies * s.num_material * 4,
                       "optical constants [E][M][4]")


def voxel_count(opts: "Options") -> int:
    s = opts.struct
    return s.num_material * s.nz * s.ny * s.nx * 4


def voxel_array(opts: "Options", voxels) -> np.ndarray:
    return expect_size(np.ascontiguousarray(voxels, np.float32), voxel_count(opts), "voxels [M][Z][Y][X][4]")


def pattern_count(opts: "Options") -> int:
    s = opts.struct
    return s.num_energies * opts.num_k * s.ny * s.nx


class Options:
    """Owns the arrays a cyr_options points into."""

    def __init__(self, *, nx, ny, nz, num_material, energies, start_angle, end_angle, increment_angle, phys_size,
                 case_type=0, k_vectors=None, detector=(0.0, 0.0, 1.0), morphology_type=0, ewald_interpolation=1,
                 windowing=0, scatter_approach=0, algorithm=0, max_streams=1, rot_mask=0, reference_frame=1,
                 strategy=0):
        self.energies = np.ascontiguousarray(energies, np.float32)
        kv = [[0.0, 0.0, 1.0]] if k_vectors is None else k_vectors
        self.k_vectors = np.ascontiguousarray(np.asarray(kv, np.float32).reshape(-1, 3))
        s = CyrOptions()
        s.nx, s.ny, s.nz = int(nx), int(ny), int(nz)
        s.num_material = int(num_material)
        s.num_energies = int(self.energies.size)
        s.energies = fptr(self.energies)
        s.start_angle, s.end_angle, s.increment_angle = float(start_angle), float(end_angle), float(increment_angle)
        s.phys_size = float(phys_size)
        s.case_type = int(case_type)
        s.num_k = int(self.k_vectors.shape[0])
        s.k_vectors = fptr(self.k_vectors)
        s.detector = (ctypes.c_float * 3)(*[float(v) for v in detector])
        s.morphology_type = int(morphology_type)
        s.ewald_interpolation = int(ewald_interpolation)
        s.windowing = int(windowing)
        s.scatter_approach = int(scatter_approach)
        s.algorithm = int(algorithm)
        s.max_streams = int(max_streams)
        s.rot_mask = int(rot_mask)
        s.reference_frame = int(reference_frame)
        s.strategy = int(strategy)
        self.struct = s

    @property
    def ref(self):
        return ctypes.byref(self.struct)

    @property
    def num_k(self) -> int:
        return int(self.struct.num_k)


def cuda_main(opts: Options, optical: np.ndarray, voxels: np.ndarray, streams_variant: bool = False,
              out: np.ndarray | None = None) -> np.ndarray:
    """Full simulation from host arrays -> float32 [E][K][ny][nx] (written into `out` when given)."""
    s = opts.struct
    shape = (s.num_energies, opts.num_k, s.ny, s.nx)
    if out is None:
        out = np.empty(shape, np.float32)
    expect_size(out, pattern_count(opts), "out [E][K][Ny][Nx]")
    opt_arr, vox = optical_array(opts, optical), voxel_array(opts, voxels)
    fn = lib().cyr_cuda_main_streams if streams_variant else lib().cyr_cuda_main
    check(fn(opts.ref, fptr(opt_arr), fptr(vox), fptr(out)))
    return out


def compute_polarization(opts: Options, optical, voxels, eangle: float, energy_id: int):
    s = opts.struct
    shape = (s.nz, s.ny, s.nx)
    px, py, pz = (np.empty(shape, np.complex64) for _ in range(3))
    as_f = lambda a: a.view(np.float32)  # noqa: E731
    check(lib().cyr_compute_polarization(opts.ref, fptr(optical_array(opts, optical)), fptr(voxel_array(opts, voxels)),
                                         float(eangle), int(energy_id), fptr(as_f(px)), fptr(as_f(py)),
                                         fptr(as_f(pz))))
    return px, py, pz


def required_device_bytes(opts: Options) -> int:
    n = ctypes.c_size_t(0)
    check(lib().cyr_required_device_bytes(opts.ref, ctypes.byref(n)))
    return int(n.value)


def simulate_device(opts: Options, optical: np.ndarray, d_voxels: int, d_out: int, stream: int = 0) -> None:
    check(lib().cyr_simulate_device(opts.ref, fptr(optical_array(opts, optical)), ctypes.c_void_p(d_voxels),
                                    ctypes.c_void_p(d_out), ctypes.c_void_p(stream)))


def selftest_wait_limit() -> bool:
    """Runs the TMA column pass with a barrier that can never complete; True if its bounded waits reported it."""
    flag = ctypes.c_int(0)
    check(lib().cyr_selftest_wait_limit(ctypes.byref(flag)))
    return bool(flag.value)


def fft3d_device(d_data: int, nx: int, ny: int, nz: int, count: int = 1, stream: int = 0) -> None:
    check(lib().cyr_fft3d_device(ctypes.c_void_p(d_data), nx, ny, nz, count, ctypes.c_void_p(stream)))


def fft3d_device_static(d_data: int, nx: int, ny: int, nz: int, count: int = 1, stream: int = 0) -> None:
    """The allocation-free variant of fft3d_device (twiddles in a fixed device array)."""
    check(lib().cyr_fft3d_device_static(ctypes.c_void_p(d_data), nx, ny, nz, count, ctypes.c_void_p(stream)))


def warp_affine_device(d_src: int, d_dst: int, width: int, height: int, coeffs, stream: int = 0) -> None:
    c = np.ascontiguousarray(np.asarray(coeffs, np.float64).reshape(6))
    check(lib().cyr_warp_affine_device(ctypes.c_void_p(d_src), ctypes.c_void_p(d_dst), width, height,
                                       c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_void_p(stream)))


def plan_info(opts: Options) -> dict:
    info = (ctypes.c_uint32 * 9)()
    check(lib().cyr_plan_info(opts.ref, info, 9))
    return {"nvol": info[0], "planes": info[1], "zlo": info[2], "pruned": bool(info[3]), "angles": info[4],
            "k": info[5], "fields": info[6], "packed_volumes": info[7], "energy_batch": info[8]}


def tuning_report() -> str:
    buf = ctypes.create_string_buffer(8192)
    check(lib().cyr_tuning_report(buf, 8192))
    return buf.value.decode()


def device_errors() -> int:
    n = ctypes.c_uint32(0)
    check(lib().cyr_device_errors(ctypes.byref(n)))
    return int(n.value)


def profile_begin(max_launches: int = 65536) -> None:
    check(lib().cyr_profile_begin(int(max_launches)))


def profile_end():
    """{kernel name: (launches, total ms, timed calls)} since profile_begin, and the dropped count."""
    n = int(lib().cyr_num_stages())
    launches = (ctypes.c_uint32 * n)()
    calls = (ctypes.c_uint32 * n)()
    ms = (ctypes.c_double * n)()
    dropped = ctypes.c_uint32(0)
    check(lib().cyr_profile_end(launches, calls, ms, n, ctypes.byref(dropped)))
    out = {}
    for i in range(n):
        if launches[i]:
            out[lib().cyr_stage_name(i).decode()] = (int(launches[i]), float(ms[i]), int(calls[i]))
    return out, int(dropped.value)


def _dptr(a: np.ndarray):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 numpy array")
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def cuda_main_fp64(opts: Options, optical, voxels, out: np.ndarray | None = None) -> np.ndarray:
    """The FP64 pipeline from host arrays (optical [E][M][4], voxels [M][Z][Y][X][4], both converted to
    float64) -> float64 [E][K][ny][nx] (cyr_cuda_main_fp64)."""
    s = opts.struct
    shape = (s.num_energies, opts.num_k, s.ny, s.nx)
    opt = np.ascontiguousarray(optical, np.float64)
    vox = np.ascontiguousarray(voxels, np.float64)
    if opt.size != s.num_energies * s.num_material * 4:
        raise ValueError(f"optical has {opt.size} elements; these options need {s.num_energies * s.num_material * 4}")
    if vox.size != voxel_count(opts):
        raise ValueError(f"voxels has {vox.size} elements; these options need {voxel_count(opts)}")
    if out is None:
        out = np.empty(shape, np.float64)
    if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != pattern_count(opts):
        raise ValueError("out must be a C-contiguous float64 array of [E][K][Ny][Nx]")
    check(lib().cyr_cuda_main_fp64(opts.ref, _dptr(opt), _dptr(vox), _dptr(out)))
    return out


def simulate_device_fp64(opts: Options, optical, d_voxels: int, voxels_fp64: bool, d_out: int, stream: int = 0) -> None:
    """Device-resident FP64 pipeline: d_voxels float4 (voxels_fp64 False) or double4; d_out doubles."""
    opt = np.ascontiguousarray(optical, np.float64)
    if opt.size != opts.struct.num_energies * opts.struct.num_material * 4:
        raise ValueError("optical constants do not match the options")
    check(lib().cyr_simulate_device_fp64(opts.ref, _dptr(opt), ctypes.c_void_p(d_voxels), int(bool(voxels_fp64)),
                                         ctypes.c_void_p(d_out), ctypes.c_void_p(stream)))


def compute_polarization_fp64(opts: Options, optical, voxels, eangle: float, energy_id: int):
    s = opts.struct
    shape = (s.nz, s.ny, s.nx)
    px, py, pz = (np.empty(shape, np.complex128) for _ in range(3))
    opt = np.ascontiguousarray(optical, np.float64)
    vox = np.ascontiguousarray(voxels, np.float64)
    if vox.size != voxel_count(opts) or opt.size != s.num_energies * s.num_material * 4:
        raise ValueError("arrays do not match the options")
    as_d = lambda a: a.view(np.float64)  # noqa: E731
    check(lib().cyr_compute_polarization_fp64(opts.ref, _dptr(opt), _dptr(vox), float(eangle), int(energy_id),
                                              _dptr(as_d(px)), _dptr(as_d(py)), _dptr(as_d(pz))))
    return px, py, pz


def release_scratch() -> None:
    """Frees the library's cached scratch space on the current device (cyr_release_scratch)."""
    check(lib().cyr_release_scratch())


def device_count() -> int:
    return int(lib().cyr_device_count())


def version() -> str:
    return lib().cyr_version().decode()
