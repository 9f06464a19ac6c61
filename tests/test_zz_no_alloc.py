"""The allocation-free FFT entry point, cyr_fft3d_device_static.

Some callers cannot allocate device memory at the point where they need a
transform.  For example, code running inside a memory pool or arena that owns
the whole device forbids cudaMalloc/cudaFree, and latency-critical paths must
not call allocating routines.  For them the library keeps the twiddle tables
in a fixed device array instead of allocating them.  This test calls that
entry point through the C ABI and checks it against the allocating entry
point, cyr_fft3d_device, on two calls in a row with different shapes.  Each
call rewrites the shared array, so the second call must not see the first
call's tables.  It also checks that axes longer than the array's limit are
refused.

The file is named so that pytest collects it last.  It needs no other test and
passes when run alone.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-6  # the FFT parity tolerance of tests/test_gpu_parity.py (relative to the largest bin)


def _setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cyrsoxs_gb300 import _native

    return torch, _native


def _run_both(torch, nat, shape, count, seed):
    rng = np.random.default_rng(seed)
    a = (rng.standard_normal((count,) + shape) + 1j * rng.standard_normal((count,) + shape)).astype(np.complex64)
    nz, ny, nx = shape
    stream = torch.cuda.current_stream().cuda_stream
    d_alloc = torch.from_numpy(a.view(np.float32).copy()).cuda()
    d_static = torch.from_numpy(a.view(np.float32).copy()).cuda()
    nat.fft3d_device(d_alloc.data_ptr(), nx, ny, nz, count, stream)
    nat.fft3d_device_static(d_static.data_ptr(), nx, ny, nz, count, stream)
    torch.cuda.synchronize()
    want = d_alloc.cpu().numpy().view(np.complex64)
    got = d_static.cpu().numpy().view(np.complex64)
    ref = np.fft.fftn(a.astype(np.complex128), axes=(1, 2, 3))
    return got, want, ref


def test_static_fft_matches_allocating_fft_on_two_calls_in_a_row():
    torch, nat = _setup()
    for shape, count, seed in (((16, 32, 48), 2, 1), ((7, 20, 64), 3, 2)):
        got, want, ref = _run_both(torch, nat, shape, count, seed)
        scale = np.abs(want).max()
        assert np.abs(got - want).max() <= TOL * scale
        assert np.abs(got.astype(np.complex128) - ref).max() <= TOL * np.abs(ref).max()


def test_static_fft_refuses_axes_beyond_its_limit():
    torch, nat = _setup()
    d = torch.zeros(2 * 8192, dtype=torch.float32, device="cuda")
    with pytest.raises(nat.CyrError) as ei:
        nat.fft3d_device_static(d.data_ptr(), 8192, 1, 1, 1)
    assert ei.value.code == 1 and "4096" in str(ei.value)
