"""The allocation-free FFT entry point, cyr_fft3d_device_static.

Some callers cannot allocate device memory at the point where they need a
transform.  For example, code running inside a memory pool or arena that owns
the whole device forbids cudaMalloc/cudaFree, and latency-critical paths must
not call allocating routines.  For them the library keeps the twiddle tables
in a fixed device array instead of allocating them.  This test calls that
entry point through the C ABI and checks it against the allocating entry
point, cyr_fft3d_device, on two calls in a row with different shapes.  Each
call rewrites the shared array, so the second call must not see the first
call's tables; the x length also changes and comes back (48, 64, 48), so
stale entries left in the array by a longer axis would show.  The shapes
reach the entry point's limit of 4096 points along x, y and z.  It also
checks that axes longer than the array's limit are refused.

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


def _check(got, want, ref):
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= TOL * scale
    assert np.abs(got.astype(np.complex128) - ref).max() <= TOL * np.abs(ref).max()


def test_static_fft_matches_allocating_fft_on_two_calls_in_a_row():
    torch, nat = _setup()
    for shape, count, seed in (((16, 32, 48), 2, 1), ((7, 20, 64), 3, 2)):
        _check(*_run_both(torch, nat, shape, count, seed))


def test_static_fft_when_an_axis_length_changes_between_calls():
    torch, nat = _setup()
    for i, nx in enumerate((48, 64, 48)):
        _check(*_run_both(torch, nat, (6, 10, nx), 2, 10 + i))


@pytest.mark.parametrize("shape,count", [((2, 256, 4096), 1), ((4, 1000, 512), 1), ((3, 2048, 7), 2),
                                         ((8, 4096, 3), 1), ((4096, 2, 8), 1)])
def test_static_fft_long_axes_up_to_its_limit(shape, count):
    torch, nat = _setup()
    _check(*_run_both(torch, nat, shape, count, sum(shape)))


def test_static_fft_refuses_axes_beyond_its_limit():
    torch, nat = _setup()
    d = torch.zeros(2 * 8192, dtype=torch.float32, device="cuda")
    with pytest.raises(nat.CyrError) as ei:
        nat.fft3d_device_static(d.data_ptr(), 8192, 1, 1, 1)
    assert ei.value.code == 1 and "4096" in str(ei.value)
