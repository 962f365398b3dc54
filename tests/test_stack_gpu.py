"""Stacking parity: linear stack (bit-exact with the reference's Python),
PWS and TF-PWS against the FP64 oracle on seeded Ricker-plus-noise NCFs.

Tolerances (relative L2 per pair): linear stack exact; PWS 1e-5; TF-PWS
1e-5 (FP32 voices and weights against FP64; the Gaussian window is FP64 on
both sides).
"""

from pathlib import Path

import numpy as np
import pytest

from fastxc_gb300.synthetic import ncf_traces
from oracle import stack_oracle as sto

pytestmark = pytest.mark.gpu
G = Path(__file__).resolve().parent / "golden"


def rel(a, b):
    return np.linalg.norm(a - b, axis=-1) / np.maximum(np.linalg.norm(b, axis=-1), 1e-30)


def test_linear_stack_matches_reference_golden(ctx, torch_cuda):
    torch = torch_cuda
    from fastxc_gb300 import stack

    d = np.load(G / "linear_stack_golden.npz")
    tr = torch.from_numpy(d["traces"]).cuda()
    out = torch.empty((1, tr.shape[1]), dtype=torch.float32, device="cuda")
    stack.linear_stack(ctx, tr, [0], [tr.shape[0]], tr.shape[1], out)
    ctx.synchronize()
    assert np.array_equal(out.cpu().numpy()[0], d["stacked"])


def _adversarial_traces(cnt, n, seed):
    """Columns by t mod 10: noise; terms across 80 decades; one term 2^-30
    of the rest; all -0; mixed signed zeros; subnormals; a NaN; +-inf;
    exact cancellations; cnt-scaled large values."""
    rng = np.random.default_rng(seed)
    tr = (rng.standard_normal((cnt, n)) * 0.3).astype(np.float32)
    kind = np.arange(n) % 10
    wide = rng.standard_normal((cnt, n)) * 10.0 ** rng.integers(-40, 38, (cnt, n))
    tr[:, kind == 1] = wide[:, kind == 1].astype(np.float32)
    tr[cnt // 2, kind == 2] *= np.float32(2.0 ** -30)
    tr[:, kind == 3] = -0.0
    tr[:, kind == 4] = np.where(rng.random((cnt, (kind == 4).sum())) < 0.5, -0.0, 0.0)
    sub = rng.integers(-5, 6, (cnt, (kind == 5).sum())) * 2.0 ** rng.integers(-149, -126, (cnt, (kind == 5).sum()))
    tr[:, kind == 5] = sub.astype(np.float32)
    tr[cnt - 1, kind == 6] = np.nan
    tr[0, kind == 7] = np.inf
    if cnt > 1:
        tr[1, kind == 7] = -np.inf if cnt > 2 else np.inf
    half = cnt // 2
    tr[half:2 * half, kind == 8] = -tr[:half, kind == 8]
    tr[:, kind == 9] = (rng.standard_normal((cnt, (kind == 9).sum())) * 3e37).astype(np.float32)
    return tr


@pytest.mark.parametrize("cnt", [1, 2, 7, 720])
def test_linear_stack_bits_on_adversarial_columns(ctx, torch_cuda, cnt):
    """The fixed-point sum gives the reference's FP64 sequence bit for bit,
    and the columns it cannot prove exact take the FP64 loop."""
    torch = torch_cuda
    from fastxc_gb300 import stack

    n = 1100  # two CTAs per pair, the second one partly past the trace end
    trs = [_adversarial_traces(c, n, seed=c) for c in (cnt, 3)]
    allt = np.concatenate(trs)
    counts = [cnt, 3]
    offs = [0, cnt]
    out = torch.empty((2, n), dtype=torch.float32, device="cuda")
    stack.linear_stack(ctx, torch.from_numpy(allt).cuda(), offs, counts, n, out)
    ctx.synchronize()
    got = out.cpu().numpy()
    with np.errstate(all="ignore"):
        ref = np.stack([sto.linear_stack(t) for t in trs])
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got[~nan].view(np.uint32), ref[~nan].view(np.uint32))


def _prestacked(ctx, torch, tr, substack, mode):
    from fastxc_gb300 import stack

    npairs, nt, n = tr.shape
    d_tr = torch.from_numpy(tr.reshape(-1, n)).cuda()
    offs = np.arange(npairs) * nt
    return stack.prestack(ctx, torch, d_tr, offs, [nt] * npairs, n, substack, mode)


@pytest.mark.parametrize("substack,power", [(1, 1.0), (3, 1.0), (1, 2.0)])
def test_pws_matches_oracle(ctx, torch_cuda, substack, power):
    torch = torch_cuda
    from fastxc_gb300 import stack

    tr = ncf_traces(5, 17, 2001, seed=3)
    g, w, lin, goff, gcnt = _prestacked(ctx, torch, tr, substack, stack.MODE_PWS)
    out = torch.empty((5, 2001), dtype=torch.float32, device="cuda")
    stack.pws(ctx, g, w, goff, gcnt, lin, 2001, out, power)
    got = out.cpu().numpy()
    ref = np.stack([sto.pws(tr[p], substack, power) for p in range(5)])
    err = rel(got, ref)
    print("pws rel err", err)
    assert err.max() < 1e-5


def test_prestack_matches_oracle(ctx, torch_cuda):
    torch = torch_cuda
    from fastxc_gb300 import stack

    tr = ncf_traces(3, 10, 1001, seed=4)
    for mode, fn in ((stack.MODE_PWS, sto.pws_prestack), (stack.MODE_TFPWS, sto.tfpws_prestack)):
        g, w, lin, goff, gcnt = _prestacked(ctx, torch, tr, 4, mode)
        assert list(gcnt) == [3, 3, 3] and list(goff) == [0, 3, 6]
        for p in range(3):
            rg, rw, rl = fn(tr[p], 4)
            assert np.allclose(g.cpu().numpy()[3 * p: 3 * p + 3], rg, rtol=1e-6, atol=1e-6)
            assert np.allclose(w.cpu().numpy()[3 * p: 3 * p + 3], rw, rtol=1e-7)
            assert np.allclose(lin.cpu().numpy()[p], rl, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("band,power", [(None, 1.0), ((0.05, 2.0), 1.0), (None, 2.0)])
def test_tfpws_matches_oracle(ctx, torch_cuda, band, power):
    torch = torch_cuda
    from fastxc_gb300 import stack

    n = 1001
    tr = ncf_traces(2, 9, n, seed=5)
    g, w, lin, goff, gcnt = _prestacked(ctx, torch, tr, 3, stack.MODE_TFPWS)
    out = torch.empty((2, n), dtype=torch.float32, device="cuda")
    stack.tfpws(ctx, g, w, goff, gcnt, lin, n, out, 0.1, band=band, power=power)
    got = out.cpu().numpy()
    ref = np.stack([sto.tfpws(tr[p], 3, power, band=band, delta=0.1) for p in range(2)])
    err = rel(got, ref)
    print("tfpws rel err", err)
    assert err.max() < 1e-5


@pytest.mark.parametrize("n,ngroups", [(2000, 7), (2001, 1), (2001, 2)])
def test_pws_group_parity_and_even_length(ctx, torch_cuda, n, ngroups):
    """Odd N pairs the groups two per transform (one group left alone when
    their count is odd, a single group on its own); even N keeps one
    transform pair per group."""
    torch = torch_cuda
    from fastxc_gb300 import stack

    tr = ncf_traces(3, ngroups, n, seed=9)
    g, w, lin, goff, gcnt = _prestacked(ctx, torch, tr, 1, stack.MODE_PWS)
    out = torch.empty((3, n), dtype=torch.float32, device="cuda")
    stack.pws(ctx, g, w, goff, gcnt, lin, n, out, 1.0)
    got = out.cpu().numpy()
    ref = np.stack([sto.pws(tr[p], 1, 1.0) for p in range(3)])
    assert rel(got, ref).max() < 1e-5


@pytest.mark.parametrize("n", [4001, 1009, 3937])
def test_pws_prime_lengths_bluestein(ctx, torch_cuda, n):
    """NCF lengths with a prime factor above 31 (4001 = lag 200 s at 10 Hz,
    prime; 3937 = 31 * 127) run through the Bluestein transform."""
    torch = torch_cuda
    from fastxc_gb300 import stack

    tr = ncf_traces(3, 8, n, seed=6)
    g, w, lin, goff, gcnt = _prestacked(ctx, torch, tr, 2, stack.MODE_PWS)
    out = torch.empty((3, n), dtype=torch.float32, device="cuda")
    stack.pws(ctx, g, w, goff, gcnt, lin, n, out, 1.0)
    got = out.cpu().numpy()
    ref = np.stack([sto.pws(tr[p], 2, 1.0) for p in range(3)])
    err = rel(got, ref)
    print("pws bluestein rel err", n, err)
    assert err.max() < 1e-5


@pytest.mark.parametrize("n,band", [(211, None), (401, (0.2, 1.5))])
def test_tfpws_prime_lengths_bluestein(ctx, torch_cuda, n, band):
    torch = torch_cuda
    from fastxc_gb300 import stack

    tr = ncf_traces(2, 6, n, seed=7)
    g, w, lin, goff, gcnt = _prestacked(ctx, torch, tr, 2, stack.MODE_TFPWS)
    out = torch.empty((2, n), dtype=torch.float32, device="cuda")
    stack.tfpws(ctx, g, w, goff, gcnt, lin, n, out, 0.1, band=band, power=1.0)
    got = out.cpu().numpy()
    ref = np.stack([sto.tfpws(tr[p], 2, 1.0, band=band, delta=0.1) for p in range(2)])
    err = rel(got, ref)
    print("tfpws bluestein rel err", n, err)
    assert err.max() < 1e-5


@pytest.mark.parametrize("n,power,npairs", [(2001, 1.0, 4), (4001, 2.0, 5), (2000, 1.0, 3)])
def test_streaming_pws_matches_oracle(ctx, torch_cuda, n, power, npairs):
    """One group per call (weight 1/G): the same PWS as prestack(1) + run.
    Odd lengths pair rows per transform (an odd row count leaves one row
    alone); even lengths take the masked analytic spectrum."""
    torch = torch_cuda
    from fastxc_gb300 import stack

    G = 7
    tr = ncf_traces(npairs, G, n, seed=8)
    acc = torch.zeros((npairs, 2 * n), dtype=torch.float32, device="cuda")
    lin = torch.zeros((npairs, n), dtype=torch.float32, device="cuda")
    for g in range(G):
        rows = torch.from_numpy(np.ascontiguousarray(tr[:, g, :])).cuda()
        stack.pws_stream_add(ctx, rows, n, npairs, n, 1.0 / G, acc, lin)
    out = torch.empty((npairs, n), dtype=torch.float32, device="cuda")
    stack.pws_stream_finish(ctx, acc, lin, npairs, n, power, out)
    ctx.synchronize()
    ref = np.stack([sto.pws(tr[p], 1, power) for p in range(npairs)])
    assert rel(out.cpu().numpy(), ref).max() < 1e-5
    assert rel(lin.cpu().numpy(), tr.mean(axis=1)).max() < 1e-6
