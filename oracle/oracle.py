"""ctypes wrapper for the CPU oracle (oracle/_build/libcyr_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, as the checker or the timed CPU baseline.  The product
path never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcyr_oracle.so")
_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        fp = ctypes.POINTER(ctypes.c_float)
        L.oracle_run_case.argtypes = [ctypes.c_char_p, dp, ctypes.c_uint32, ctypes.c_uint32, dp]
        L.oracle_polarization_case.argtypes = [ctypes.c_char_p, dp]
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.oracle_run_arrays.argtypes = [u32p, fp, fp, fp, fp, fp, dp, ctypes.c_uint32, ctypes.c_uint32, dp]
        L.oracle_fft3d.argtypes = [dp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
        L.oracle_warp.argtypes = [dp, dp, ctypes.c_int, ctypes.c_int, dp]
        L.oracle_rotation.argtypes = [fp, ctypes.c_int, ctypes.c_float, fp, fp]
        L.oracle_last_error.restype = ctypes.c_char_p
        L.oracle_num_threads.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def run_case_file(path: str, out_shape, angle_limit: int = 0, energy_limit: int = 0):
    """Full pipeline on a case file; returns (out[E][K][Ny][Nx] float64, seconds)."""
    out = np.full(out_shape, np.nan, np.float64)
    secs = np.zeros(1, np.float64)
    rc = lib().oracle_run_case(path.encode(), _dp(out), angle_limit, energy_limit, _dp(secs))
    if rc:
        raise RuntimeError(lib().oracle_last_error().decode())
    return out, float(secs[0])


def run_case(case, angle_limit: int = 0, energy_limit: int = 0):
    """Runs a tests/golden/cases.py Case; returns the [E][K][Ny][Nx] output."""
    import cases as _cases  # tests/golden on sys.path

    with tempfile.TemporaryDirectory() as tmp:
        p = os.path.join(tmp, "c.case")
        _cases.write_case(case, p)
        out, _ = run_case_file(p, _cases.output_shape(case), angle_limit, energy_limit)
    return out


def run_arrays(*, nx, ny, nz, energies, optical, voxels, angles, phys_size, morphology=0, windowing=0,
               interpolation=1, rot_mask=0, algorithm=0, frame=1, case_type=0, kvecs=((0.0, 0.0, 1.0),),
               detector=(0.0, 0.0, 1.0), angle_limit=0, energy_limit=0):
    """Pipeline on in-memory arrays (voxels float32 [M][Z][Y][X][4]); returns (out, seconds)."""
    vox = np.ascontiguousarray(voxels, np.float32)
    opt = np.ascontiguousarray(optical, np.float32)
    nmat = vox.shape[0]
    es = np.ascontiguousarray(energies, np.float32)
    kv = np.ascontiguousarray(np.asarray(kvecs, np.float32).reshape(-1, 3))
    hdr = np.array([nx, ny, nz, nmat, es.size, kv.shape[0], morphology, windowing, interpolation, 0, rot_mask,
                    algorithm, 1, frame, case_type, 0], np.uint32)
    fl = np.array([phys_size, angles[0], angles[1], angles[2], 0, 0, *detector], np.float32)
    ne_out = min(energy_limit, es.size) if energy_limit else es.size
    out = np.full((es.size, kv.shape[0], ny, nx), np.nan, np.float64)
    secs = np.zeros(1, np.float64)
    fp = ctypes.POINTER(ctypes.c_float)
    rc = lib().oracle_run_arrays(hdr.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), fl.ctypes.data_as(fp),
                                 es.ctypes.data_as(fp), kv.ctypes.data_as(fp), opt.ctypes.data_as(fp),
                                 vox.ctypes.data_as(fp), _dp(out), angle_limit, energy_limit, _dp(secs))
    if rc:
        raise RuntimeError(lib().oracle_last_error().decode())
    return out[:ne_out], float(secs[0])


def polarization_case_file(path: str, shape):
    """computePolarization debug path on a case file -> complex [3][nz][ny][nx]."""
    nv = int(np.prod(shape[1:]))
    out = np.zeros((3, nv, 2), np.float64)
    rc = lib().oracle_polarization_case(path.encode(), _dp(out))
    if rc:
        raise RuntimeError(lib().oracle_last_error().decode())
    return (out[..., 0] + 1j * out[..., 1]).reshape(shape)


def polarization_case(case):
    import cases as _cases

    nv = case.nx * case.ny * case.nz
    out = np.zeros((3, nv, 2), np.float64)
    with tempfile.TemporaryDirectory() as tmp:
        p = os.path.join(tmp, "c.case")
        _cases.write_case(case, p)
        rc = lib().oracle_polarization_case(p.encode(), _dp(out))
    if rc:
        raise RuntimeError(lib().oracle_last_error().decode())
    c = out[..., 0] + 1j * out[..., 1]
    return c.reshape(3, case.nz, case.ny, case.nx)


def fft3d(a: np.ndarray) -> np.ndarray:
    """Forward unnormalised 3D DFT of a complex [nz][ny][nx] array."""
    nz, ny, nx = a.shape
    buf = np.ascontiguousarray(a, np.complex128).copy()
    lib().oracle_fft3d(buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nx, ny, nz)
    return buf


def warp(src: np.ndarray, coeffs, prefill: float) -> np.ndarray:
    """NPP-semantics bilinear warp of src [h][w]; coeffs is the 2x3 matrix."""
    h, w = src.shape
    s = np.ascontiguousarray(src, np.float64)
    d = np.full((h, w), prefill, np.float64)
    c = np.ascontiguousarray(np.asarray(coeffs, np.float64).reshape(6))
    lib().oracle_warp(_dp(s), _dp(d), w, h, _dp(c))
    return d


def rotation(k, eangle: float, normalize: bool = True):
    """(R 3x3 float32, base angle) for an E angle in radians about k."""
    kk = np.asarray(k, np.float32)
    R = np.zeros(9, np.float32)
    base = np.zeros(1, np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    lib().oracle_rotation(kk.ctypes.data_as(fp), int(normalize), float(eangle), R.ctypes.data_as(fp),
                          base.ctypes.data_as(fp))
    return R.reshape(3, 3), float(base[0])


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def num_threads() -> int:
    return int(lib().oracle_num_threads())
