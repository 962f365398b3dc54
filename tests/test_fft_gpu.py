"""The library's own FFT against numpy (FP64) for every length the hot path uses.

Lengths (those of the reference's cuFFT plans in sac2spec, xc and the
stacking stages): segment 36000,
filter 36288, output 37044 / 36750 / 38400, the half-lengths 18000, 18144,
18522, NCF lengths 2001 (3*23*29) and 1001 (7*11*13), plus small edge cases.
Tolerance: FP32 transforms, relative L2 error <= 2e-6 against FP64.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 2e-6


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 12, 16, 60, 64, 124, 323, 646, 1001, 2001, 4096, 18000, 18144,
                               18522, 19200])
@pytest.mark.parametrize("inverse", [False, True])
def test_c2c(ctx, torch_cuda, n, inverse):
    torch = torch_cuda
    rng = np.random.default_rng(n)
    batch = 3
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    d_in = torch.from_numpy(x).cuda()
    d_out = torch.empty_like(d_in)
    ctx.fft_c2c(d_in, d_out, n, batch, inverse=inverse)
    ctx.synchronize()
    got = d_out.cpu().numpy()
    ref = np.fft.ifft(x.astype(np.complex128), axis=-1) * n if inverse else np.fft.fft(x.astype(np.complex128), axis=-1)
    assert rel_l2(got, ref) < RTOL


@pytest.mark.parametrize("n", [2, 8, 10, 1000, 1001, 2000, 2001, 2002, 36000, 36288, 36750, 37044, 38400])
def test_r2c(ctx, torch_cuda, n):
    torch = torch_cuda
    rng = np.random.default_rng(100 + n)
    batch = 4
    x = rng.standard_normal((batch, n)).astype(np.float32)
    d_in = torch.from_numpy(x).cuda()
    d_out = torch.empty((batch, n // 2 + 1), dtype=torch.complex64, device="cuda")
    ctx.fft_r2c(d_in, d_out, n, batch)
    ctx.synchronize()
    ref = np.fft.rfft(x.astype(np.float64), axis=-1)
    assert rel_l2(d_out.cpu().numpy(), ref) < RTOL


@pytest.mark.parametrize("n", [2, 8, 10, 1000, 2000, 2002, 36000, 36288, 36750, 37044, 38400])
def test_c2r(ctx, torch_cuda, n):
    torch = torch_cuda
    rng = np.random.default_rng(200 + n)
    batch = 4
    m = n // 2 + 1
    X = (rng.standard_normal((batch, m)) + 1j * rng.standard_normal((batch, m))).astype(np.complex64)
    d_in = torch.from_numpy(X).cuda()
    d_out = torch.empty((batch, n), dtype=torch.float32, device="cuda")
    ctx.fft_c2r(d_in, d_out, n, batch)
    ctx.synchronize()
    # unnormalised C2R; DC and Nyquist imaginary parts ignored like numpy irfft
    ref = np.fft.irfft(X.astype(np.complex128), n=n, axis=-1) * n
    got = d_out.cpu().numpy()
    assert rel_l2(got, ref) < RTOL


def test_pitched_rows(ctx, torch_cuda):
    torch = torch_cuda
    n, batch, ip, op = 36000, 3, 36100, 18010
    rng = np.random.default_rng(7)
    x = rng.standard_normal((batch, ip)).astype(np.float32)
    d_in = torch.from_numpy(x).cuda()
    d_out = torch.zeros((batch, op), dtype=torch.complex64, device="cuda")
    ctx.fft_r2c(d_in, d_out, n, batch, in_pitch=ip, out_pitch=op)
    ctx.synchronize()
    ref = np.fft.rfft(x[:, :n].astype(np.float64), axis=-1)
    got = d_out.cpu().numpy()
    assert rel_l2(got[:, : n // 2 + 1], ref) < RTOL
    assert np.all(got[:, n // 2 + 1:] == 0)


def test_unsupported_length_reports_error(ctx, torch_cuda):
    from fastxc_gb300 import FxcError

    torch = torch_cuda
    n = 4001  # prime above the in-CTA radix set
    d = torch.zeros((1, n), dtype=torch.complex64, device="cuda")
    with pytest.raises(FxcError):
        ctx.fft_c2c(d, d, n, 1)
