"""xc_fast parity: library correlation + stack + finalize against the FP64 oracle.

Tolerance: every NCF within relative L2 1e-5 of the FP64 restatement (the
bound the tensor path is held to); the stacked spectra within 2e-6.
"""

import numpy as np
import pytest

from oracle import xc_oracle as xo

pytestmark = pytest.mark.gpu

NCF_RTOL = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def per_row_rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    num = np.linalg.norm(a - b, axis=-1)
    den = np.maximum(np.linalg.norm(b, axis=-1), 1e-300)
    return num / den


def station_pairs(nsta, ncomp=3, auto=False):
    src, rec = [], []
    for s in range(nsta):
        for t in range(s if auto else s + 1, nsta):
            for i in range(ncomp):
                for j in range(ncomp):
                    src.append(s * ncomp + i)
                    rec.append(t * ncomp + j)
    return np.array(src, np.int32), np.array(rec, np.int32)


def make_spec(rng, nwin, nchan, nspec, coherent=True):
    y = rng.standard_normal((nwin, nchan, nspec)) + 1j * rng.standard_normal((nwin, nchan, nspec))
    if coherent:
        common = rng.standard_normal((nwin, 1, nspec)) + 1j * rng.standard_normal((nwin, 1, nspec))
        y = y + 2.0 * common
    return y.astype(np.complex64)


def run_xc(ctx, torch, spec, src, rec, shape, scale, mask=None, method=0):
    from fastxc_gb300.core import PairPlan

    nwin, nchan, pitch = spec.shape
    plan = PairPlan(ctx, src, rec, nchan)
    d_spec = torch.from_numpy(spec).cuda()
    d_mask = torch.from_numpy(mask).cuda() if mask is not None else None
    d_ncf = torch.empty((len(src), shape.cc_size), dtype=torch.float32, device="cuda")
    ctx.xc_run(plan, d_spec, nwin, nchan, pitch, d_mask, scale, shape, d_ncf, method)
    ctx.synchronize()
    return d_ncf.cpu().numpy(), plan


@pytest.mark.parametrize("method", [0, 1], ids=["plain", "tensor"])
@pytest.mark.parametrize("nspec,nwin,nsta", [(1001, 5, 4), (18523, 24, 4), (1001, 75, 8)])
def test_xc_ncf_matches_oracle(ctx, torch_cuda, nspec, nwin, nsta, method):
    rng = np.random.default_rng(nspec + nwin)
    nchan = 3 * nsta
    spec = make_spec(rng, nwin, nchan, nspec)
    src, rec = station_pairs(nsta)
    shape = ctx_shape(nspec, nwin, 0.1, 100.0 if nspec > 5000 else 20.0)
    scale = 1.0 / nwin
    got, _ = run_xc(ctx, torch_cuda, spec, src, rec, shape, scale, method=method)
    oshape = xo.finalize_shape(nspec, nwin, 0.1, 100.0 if nspec > 5000 else 20.0)
    assert (shape.nfft, shape.half_cc, shape.cc_size) == (oshape.nfft, oshape.half_cc, oshape.cc_size)
    ref = xo.xc_run(spec, src, rec, scale, oshape)
    assert got.shape == ref.shape
    assert per_row_rel_l2(got, ref).max() < NCF_RTOL


def ctx_shape(nspec, nstep, dt, cc):
    from fastxc_gb300.core import xc_shape

    return xc_shape(nspec, nstep, dt, cc)


@pytest.mark.parametrize("method,tol", [(0, 2e-6), (1, 2e-5)], ids=["plain", "tensor"])
def test_stack_matches_oracle_with_mask_and_ragged_tiles(ctx, torch_cuda, method, tol):
    """nchan not a multiple of the tile, masked windows, autocorrelations,
    duplicate, reversed and unordered pairs. The tensor path computes BF16
    hi/lo products (about 2^-16 relative per term), hence its bound."""
    torch = torch_cuda
    from fastxc_gb300.core import PairPlan

    rng = np.random.default_rng(3)
    nwin, nchan, nspec, pitch = 7, 37, 300, 304
    spec = make_spec(rng, nwin, nchan, pitch)
    src, rec = station_pairs(12, auto=True)
    src = np.concatenate([src, [36, 5, 5, 0, 30, 2]]).astype(np.int32)
    rec = np.concatenate([rec, [0, 5, 5, 36, 1, 2]]).astype(np.int32)
    perm = rng.permutation(src.size)
    src, rec = src[perm], rec[perm]
    mask = (rng.random((nwin, nchan)) > 0.2).astype(np.uint8)
    plan = PairPlan(ctx, src, rec, nchan)
    d_spec = torch.from_numpy(spec).cuda()
    d_mask = torch.from_numpy(mask).cuda()
    spitch = 304
    d_stack = torch.zeros((src.size, spitch), dtype=torch.complex64, device="cuda")
    ctx.xc_stack(plan, d_spec, nwin, nchan, nspec, pitch, d_mask, 0.25, d_stack, spitch, method)
    ctx.synchronize()
    got = d_stack.cpu().numpy()[:, :nspec]
    ref = xo.xc_stack(spec[:, :, :nspec], src, rec, 0.25, mask)
    assert rel_l2(got, ref) < tol
    assert np.all(d_stack.cpu().numpy()[:, nspec:] == 0)


@pytest.mark.parametrize("nchan", [150, 192, 96])
def test_whole_bin_contraction_matches_oracle_and_tiled(ctx, torch_cuda, nchan, monkeypatch):
    """Up to 192 channels one CTA contracts a whole bin and writes it as a
    bin-major row that a transpose moves into the stack: persistent CTAs,
    one per SM, or one CTA per bin (FXC_GEMM_BIN_PERCTA=1), bit-identical.
    An odd number of pairs, autocorrelations, reversed (conjugated) pairs
    and a shuffled pair order; same stack as the FP64 oracle and as the
    tiled contraction."""
    torch = torch_cuda
    from fastxc_gb300.core import PairPlan

    rng = np.random.default_rng(17)
    nwin, nspec = 130, 257  # more than three 32-window K-blocks: whole-bin below 129 channels too
    spec = make_spec(rng, nwin, nchan, nspec)
    iu, ju = np.triu_indices(nchan)
    keep = rng.random(iu.size) < 0.3
    src, rec = iu[keep].astype(np.int32), ju[keep].astype(np.int32)
    if src.size % 2 == 0:
        src, rec = src[:-1], rec[:-1]
    flip = rng.random(src.size) < 0.3
    src, rec = np.where(flip, rec, src).astype(np.int32), np.where(flip, src, rec).astype(np.int32)
    perm = rng.permutation(src.size)
    src, rec = src[perm], rec[perm]
    plan = PairPlan(ctx, src, rec, nchan)
    d_spec = torch.from_numpy(spec).cuda()
    a = torch.zeros((src.size, nspec), dtype=torch.complex64, device="cuda")
    b = torch.zeros_like(a)
    ctx.xc_stack(plan, d_spec, nwin, nchan, nspec, nspec, None, 0.5, a, nspec, 1)
    c = torch.full_like(a, float("nan"))
    monkeypatch.setenv("FXC_GEMM_BIN_PERCTA", "1")
    ctx.xc_stack(plan, d_spec, nwin, nchan, nspec, nspec, None, 0.5, c, nspec, 1)
    monkeypatch.delenv("FXC_GEMM_BIN_PERCTA")
    ctx.synchronize()
    assert torch.equal(a, c)
    monkeypatch.setenv("FXC_GEMM_TILED", "1")
    ctx.xc_stack(plan, d_spec, nwin, nchan, nspec, nspec, None, 0.5, b, nspec, 1)
    monkeypatch.delenv("FXC_GEMM_TILED")
    ctx.synchronize()
    ref = xo.xc_stack(spec, src, rec, 0.5)
    assert rel_l2(a.cpu().numpy(), ref) < 2e-5
    assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("nchan,nwin,nspec", [(192, 70, 301), (150, 33, 256), (96, 130, 301)])
def test_fused_pack_contraction_equals_packed(ctx, torch_cuda, monkeypatch, nchan, nwin, nspec):
    """The whole-bin contraction that reads the FP32 spectra itself
    (FXC_GEMM_FUSED=1: clusters of 4 CTAs, one per bin, each loading a
    quarter of the rows of all 4 bins as whole 32-byte sectors and storing
    the other bins' bf16 hi/lo chunks into its peers' operand rings) forms
    the same operands as k_xc_pack and runs the same MMAs in the same order:
    its stack equals the packed path's bit for bit, with a partial last
    K-block, a last cluster past nspec, autocorrelations and reversed
    pairs; and the FP64 oracle within 2e-5. Rows padded to a multiple of 4
    bins; an odd pitch, or a window mask, falls back to the packed path."""
    torch = torch_cuda
    from fastxc_gb300._lib import FXC_XC_LAYOUT_WHOLE_BIN as WHOLE
    from fastxc_gb300._lib import lib
    from fastxc_gb300.core import PairPlan

    rng = np.random.default_rng(nchan * 7 + nwin)
    pitch = (nspec + 3) // 4 * 4
    spec = make_spec(rng, nwin, nchan, nspec)
    padded = np.zeros((nwin, nchan, pitch), np.complex64)
    padded[:, :, :nspec] = spec
    iu, ju = np.triu_indices(nchan)
    keep = rng.random(iu.size) < 0.4
    src, rec = iu[keep].astype(np.int32), ju[keep].astype(np.int32)
    flip = rng.random(src.size) < 0.3
    src, rec = np.where(flip, rec, src).astype(np.int32), np.where(flip, src, rec).astype(np.int32)
    mask = (rng.random((nwin, nchan)) > 0.1).astype(np.uint8)
    plan = PairPlan(ctx, src, rec, nchan)
    plan.set_layout(WHOLE)
    assert plan.layouts(nwin)[1] == WHOLE
    d_spec = torch.from_numpy(padded).cuda()
    d_mask = torch.from_numpy(mask).cuda()
    out, launches = {}, {}
    for packed in (False, True):
        monkeypatch.setenv("FXC_GEMM_FUSED", "0" if packed else "1")
        ctx.kernel_timing(True)
        st = torch.zeros((src.size, nspec), dtype=torch.complex64, device="cuda")
        lib().fxc_launch_count_reset()
        ctx.xc_stack(plan, d_spec, nwin, nchan, nspec, pitch, None, 0.5, st, nspec, 1)
        ctx.synchronize()
        launches[packed] = lib().fxc_launch_count()
        assert ctx.kernel_time("k_xc_tc_gemm_bin")[1] == 1
        ctx.kernel_timing(False)
        out[packed] = st.cpu().numpy()
    assert launches == {False: 2, True: 3}, launches  # the fused path launches no pack
    assert np.array_equal(out[False], out[True])
    ref = xo.xc_stack(spec, src, rec, 0.5)
    assert rel_l2(out[False], ref) < 2e-5
    # an odd pitch (no 16-byte copies of bin pairs) or a mask: the packed path
    monkeypatch.setenv("FXC_GEMM_FUSED", "1")
    odd = np.zeros((nwin, nchan, pitch + 1), np.complex64)
    odd[:, :, :nspec] = spec
    for arr, pt, m in ((odd, pitch + 1, None), (padded, pitch, d_mask)):
        st = torch.zeros((src.size, nspec), dtype=torch.complex64, device="cuda")
        lib().fxc_launch_count_reset()
        ctx.xc_stack(plan, torch.from_numpy(arr).cuda(), nwin, nchan, nspec, pt, m, 0.5, st, nspec, 1)
        ctx.synchronize()
        assert lib().fxc_launch_count() == 3
        if m is None:
            assert np.array_equal(st.cpu().numpy(), out[True])
        else:
            assert rel_l2(st.cpu().numpy(), xo.xc_stack(spec, src, rec, 0.5, mask)) < 2e-5


@pytest.mark.parametrize("nchan,nwin", [(96, 24), (192, 130)])
def test_layout_autotune_and_preference(ctx, torch_cuda, nchan, nwin):
    """The autotuner times the plain kernel and the tensor contraction in
    both layouts the plan admits, sets the plan's layout to the faster, and
    a layout preference changes which kernel runs, not the stack (same
    stack as the FP64 oracle in either layout). A plan without the whole-bin
    geometry (more than 192 channels) admits only the tiled layout and runs
    tiled under a whole-bin preference."""
    torch = torch_cuda
    from fastxc_gb300._lib import FXC_XC_LAYOUT_TILED as TILED
    from fastxc_gb300._lib import FXC_XC_LAYOUT_WHOLE_BIN as WHOLE
    from fastxc_gb300.core import PairPlan

    rng = np.random.default_rng(nchan + nwin)
    nspec = 257
    spec = make_spec(rng, nwin, nchan, nspec)
    src, rec = station_pairs(nchan // 3)
    plan = PairPlan(ctx, src, rec, nchan)
    d_spec = torch.from_numpy(spec).cuda()
    admitted, _ = plan.layouts(nwin)
    assert admitted == (1 << WHOLE) | (1 << TILED)
    method, layout, ms = ctx.xc_autotune_layout(plan, d_spec, nwin, nchan, nspec, nspec)
    assert ms["plain"] > 0 and ms["whole_bin"] > 0 and ms["tiled"] > 0
    assert layout == (WHOLE if ms["whole_bin"] <= ms["tiled"] else TILED)
    assert method == (1 if min(ms["whole_bin"], ms["tiled"]) < ms["plain"] else 0)
    assert plan.layouts(nwin)[1] == layout
    ref = xo.xc_stack(spec, src, rec, 0.5)
    got = {}
    for lay in (WHOLE, TILED):
        plan.set_layout(lay)
        assert plan.layouts(nwin)[1] == lay
        ctx.kernel_timing(True)
        out = torch.zeros((src.size, nspec), dtype=torch.complex64, device="cuda")
        ctx.xc_stack(plan, d_spec, nwin, nchan, nspec, nspec, None, 0.5, out, nspec, 1)
        ctx.synchronize()
        ran = {k: ctx.kernel_time(k)[1] for k in ("k_xc_tc_gemm_bin", "k_xc_tc_gemm")}
        ctx.kernel_timing(False)
        assert ran["k_xc_tc_gemm_bin" if lay == WHOLE else "k_xc_tc_gemm"] >= 1
        got[lay] = out.cpu().numpy()
        assert rel_l2(got[lay], ref) < 2e-5
    assert rel_l2(got[WHOLE], got[TILED]) < 1e-6
    wide = PairPlan(ctx, *station_pairs(100), 300)
    assert wide.layouts(nwin)[0] == 1 << TILED
    wide.set_layout(WHOLE)
    assert wide.layouts(nwin)[1] == TILED


@pytest.mark.parametrize("nwin", [24, 70])
def test_tiled_contraction_above_256_channels(ctx, torch_cuda, nwin):
    """Above 192 channels the persistent tiled contraction runs (bin, tile)
    items: several 256-column chunks per row block, pairs listed twice (an
    extra tile layer), reversed pairs, a partial K-block, few bins per CTA
    and many; same stack as the FP64 oracle."""
    torch = torch_cuda
    from fastxc_gb300.core import PairPlan

    rng = np.random.default_rng(23)
    nchan, nspec = 300, 129
    spec = make_spec(rng, nwin, nchan, nspec)
    iu, ju = np.triu_indices(nchan)
    keep = rng.random(iu.size) < 0.05
    src, rec = iu[keep].astype(np.int32), ju[keep].astype(np.int32)
    dup = rng.choice(src.size, 500, replace=False)
    src, rec = np.concatenate([src, src[dup]]), np.concatenate([rec, rec[dup]])
    flip = rng.random(src.size) < 0.3
    src, rec = np.where(flip, rec, src).astype(np.int32), np.where(flip, src, rec).astype(np.int32)
    plan = PairPlan(ctx, src, rec, nchan)
    d_spec = torch.from_numpy(spec).cuda()
    got = torch.zeros((src.size, nspec), dtype=torch.complex64, device="cuda")
    ctx.xc_stack(plan, d_spec, nwin, nchan, nspec, nspec, None, 0.5, got, nspec, 1)
    ctx.synchronize()
    ref = xo.xc_stack(spec, src, rec, 0.5)
    assert rel_l2(got.cpu().numpy(), ref) < 2e-5


@pytest.mark.parametrize("env", [{}, {"FXC_GEMM_TILED": "1"}, {"FXC_FINALIZE": "pruned"}])
def test_stack_finalize_packed_equals_stack_then_finalize(ctx, torch_cuda, env, monkeypatch):
    """fxc_xc_stack_finalize_packed gives the same NCF bits as
    fxc_xc_stack_packed + fxc_xc_finalize, for the whole-bin and the tiled
    contraction and the output-pruned finalize, and so does fxc_xc_run."""
    torch = torch_cuda
    from fastxc_gb300.core import Context, PairPlan

    for k, v in env.items():
        monkeypatch.setenv(k, v)
    rng = np.random.default_rng(14)
    nwin, nsta, nspec = 40, 5, 1001
    nchan = 3 * nsta
    spec = make_spec(rng, nwin, nchan, nspec)
    src, rec = station_pairs(nsta, auto=True)
    plan = PairPlan(ctx, src, rec, nchan)
    shape = ctx_shape(nspec, nwin, 0.1, 20.0)
    d_spec = torch.from_numpy(spec).cuda()
    nb = Context.xc_packed_bytes(nchan, nwin, nspec)
    d_packed = torch.zeros((nb // 16, 4), dtype=torch.int32, device="cuda")
    ctx.xc_pack(d_spec, nwin, nchan, nspec, nspec, None, d_packed)
    pitch = (nspec + 3) // 4 * 4
    d_stack = torch.zeros((src.size, pitch), dtype=torch.complex64, device="cuda")
    a = torch.zeros((src.size, shape.cc_size), dtype=torch.float32, device="cuda")
    b = torch.zeros_like(a)
    c = torch.zeros_like(a)
    ctx.xc_stack_packed(plan, d_packed, nwin, nspec, 0.25, d_stack, pitch)
    ctx.xc_finalize(d_stack, src.size, pitch, shape, a)
    ctx.xc_stack_finalize_packed(plan, d_packed, nwin, nspec, 0.25, shape, b)
    ctx.xc_run(plan, d_spec, nwin, nchan, nspec, None, 0.25, shape, c, 1)
    ctx.synchronize()
    assert torch.equal(a, b) and torch.equal(a, c)
    ref = xo.xc_run(spec, src, rec, 0.25, xo.finalize_shape(nspec, nwin, 0.1, 20.0))
    assert per_row_rel_l2(b.cpu().numpy(), ref).max() < NCF_RTOL


def _bf16_rne(x):
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def test_pack_bits_match_numpy_restatement(ctx, torch_cuda):
    """The bf16 hi/lo planes of fxc_xc_pack, bit for bit: per bin, plane
    (Re-hi, Re-lo, Im-hi, Im-lo), 32-window block, 8-window chunk, channel
    row padded to 8, 8 windows; hi = RNE bf16(x), lo = RNE bf16(x - hi);
    masked, missing and padding entries are zero."""
    torch = torch_cuda
    from fastxc_gb300.core import Context

    rng = np.random.default_rng(12)
    nwin, nchan, nspec = 45, 13, 37
    spec = make_spec(rng, nwin, nchan, nspec)
    mask = (rng.random((nwin, nchan)) > 0.2).astype(np.uint8)
    nb = Context.xc_packed_bytes(nchan, nwin, nspec)
    d_packed = torch.zeros((nb // 16, 4), dtype=torch.int32, device="cuda")
    ctx.xc_pack(torch.from_numpy(spec).cuda(), nwin, nchan, nspec, nspec, torch.from_numpy(mask).cuda(), d_packed)
    ctx.synchronize()
    nkb, cpad = (nwin + 31) // 32, (nchan + 7) // 8 * 8
    got = d_packed.cpu().numpy().view(np.uint16).reshape(nspec, 4, nkb, 4, cpad, 8)
    v = np.zeros((nkb * 32, cpad, nspec), np.complex64)
    v[:nwin, :nchan] = np.where(mask[:, :, None] != 0, spec, np.complex64(0))  # +0.0 where masked
    v = v.reshape(nkb, 4, 8, cpad, nspec).transpose(4, 0, 1, 3, 2)  # [f][kb][kc][row][e]
    planes = []
    for part in (v.real, v.imag):
        hi = _bf16_rne(part)
        lo = _bf16_rne(part - (hi.astype(np.uint32) << 16).view(np.float32))
        planes += [hi, lo]
    want = np.stack(planes, axis=1)  # [f][plane][kb][kc][row][e]
    assert np.array_equal(got, want)


def test_packed_resident_path_equals_tensor_stack(ctx, torch_cuda):
    """fxc_xc_pack + fxc_xc_stack_packed (spectra kept in packed form) gives
    bit-identical stacks to fxc_xc_stack(FXC_XC_TENSOR), for two pair plans
    on the same packed spectra."""
    torch = torch_cuda
    from fastxc_gb300.core import Context, PairPlan

    rng = np.random.default_rng(21)
    nwin, nchan, nspec = 45, 20, 257
    spec = make_spec(rng, nwin, nchan, nspec)
    d_spec = torch.from_numpy(spec).cuda()
    nbytes = Context.xc_packed_bytes(nchan, nwin, nspec)
    d_packed = torch.zeros((nbytes // 16, 4), dtype=torch.int32, device="cuda")
    ctx.xc_pack(d_spec, nwin, nchan, nspec, nspec, None, d_packed)
    for src, rec in (station_pairs(6), station_pairs(5, auto=True)):
        plan = PairPlan(ctx, src, rec, nchan)
        a = torch.zeros((src.size, nspec), dtype=torch.complex64, device="cuda")
        b = torch.zeros_like(a)
        ctx.xc_stack_packed(plan, d_packed, nwin, nspec, 0.5, a, nspec)
        ctx.xc_stack(plan, d_spec, nwin, nchan, nspec, nspec, None, 0.5, b, nspec, 1)
        ctx.synchronize()
        assert torch.equal(a, b)
        ref = xo.xc_stack(spec, src, rec, 0.5)
        assert rel_l2(a.cpu().numpy(), ref) < 2e-5


def test_zero_windows_contribute_zero(ctx, torch_cuda):
    """A gap window (all-zero spectrum) changes nothing but the divisor stays nstep."""
    rng = np.random.default_rng(11)
    nwin, nsta, nspec = 6, 3, 1001
    spec = make_spec(rng, nwin, 3 * nsta, nspec)
    spec[2] = 0
    src, rec = station_pairs(nsta)
    shape = ctx_shape(nspec, nwin, 0.1, 20.0)
    got, _ = run_xc(ctx, torch_cuda, spec, src, rec, shape, 1.0 / nwin)
    keep = np.array([0, 1, 3, 4, 5])
    ref = xo.xc_run(spec[keep], src, rec, 1.0 / nwin, xo.finalize_shape(nspec, nwin, 0.1, 20.0))
    assert per_row_rel_l2(got, ref).max() < NCF_RTOL


def test_empty_pair_list(ctx, torch_cuda):
    torch = torch_cuda
    from fastxc_gb300.core import PairPlan

    plan = PairPlan(ctx, np.zeros(0, np.int32), np.zeros(0, np.int32), 6)
    shape = ctx_shape(1001, 2, 0.1, 20.0)
    d_spec = torch.zeros((2, 6, 1001), dtype=torch.complex64, device="cuda")
    d_ncf = torch.zeros((1,), dtype=torch.float32, device="cuda")
    ctx.xc_run(plan, d_spec, 2, 6, 1001, None, 0.5, shape, d_ncf)
    ctx.synchronize()


@pytest.mark.parametrize("nwin,method,masked,tiled",
                         [(4, 0, False, False), (150, 0, True, False), (150, 1, True, False),
                          (200, 1, False, False), (400, 1, True, False), (400, 1, True, True)])
def test_host_entry_matches_oracle_and_device_entry(ctx, torch_cuda, nwin, method, masked, tiled, monkeypatch):
    """The host-buffer entry streams windows in 64-window chunks through a
    ring of device buffers (ragged last chunk, gap mask) and stacks them as
    they land: chunk by chunk (plain, and the whole-bin tensor contraction),
    or in groups of up to four chunks whose partial stacks are added to the
    running one (the tiled tensor contraction; 400 windows make groups of 4,
    2 and 1 chunks). Same NCFs as the FP64 oracle, and as the device entry
    up to the FP32 summation order."""
    if tiled:
        monkeypatch.setenv("FXC_GEMM_TILED", "1")
    rng = np.random.default_rng(5)
    nsta, nspec = 4, 1001
    spec = make_spec(rng, nwin, 3 * nsta, nspec)
    mask = (rng.random((nwin, 3 * nsta)) > 0.1).astype(np.uint8) if masked else None
    src, rec = station_pairs(nsta)
    shape = ctx_shape(nspec, nwin, 0.1, 20.0)
    dev, plan = run_xc(ctx, torch_cuda, spec, src, rec, shape, 1.0 / nwin, mask=mask, method=method)
    host = np.zeros_like(dev)
    ctx.xc_run_host(plan, spec, nwin, 3 * nsta, nspec, mask, 1.0 / nwin, shape, host, method)
    ref = xo.xc_run(spec, src, rec, 1.0 / nwin, xo.finalize_shape(nspec, nwin, 0.1, 20.0), mask=mask)
    assert per_row_rel_l2(host, ref).max() < NCF_RTOL
    assert per_row_rel_l2(host, dev).max() < 1e-5


def test_bad_arguments_raise(ctx, torch_cuda):
    from fastxc_gb300 import FxcError
    from fastxc_gb300.core import PairPlan

    with pytest.raises(FxcError):
        PairPlan(ctx, np.array([0], np.int32), np.array([9], np.int32), 6)
    with pytest.raises(FxcError):
        ctx_shape(1, 1, 0.1, 1.0)


@pytest.mark.parametrize("nspec,dt,lag", [(1001, 0.1, 20.0), (18523, 0.1, 100.0), (9262, 0.2, 200.0)])
def test_pruned_finalize_matches_oracle(ctx, torch_cuda, nspec, dt, lag, monkeypatch):
    """The output-pruned finalize (P length-Q transforms + per-lag sums) on
    lengths the one-CTA transform also covers."""
    rng = np.random.default_rng(31)
    nwin, nsta = 4, 3
    spec = make_spec(rng, nwin, 3 * nsta, nspec)
    src, rec = station_pairs(nsta)
    shape = ctx_shape(nspec, nwin, dt, lag)
    full, _ = run_xc(ctx, torch_cuda, spec, src, rec, shape, 1.0 / nwin)
    monkeypatch.setenv("FXC_FINALIZE", "pruned")
    pruned, _ = run_xc(ctx, torch_cuda, spec, src, rec, shape, 1.0 / nwin)
    monkeypatch.delenv("FXC_FINALIZE")
    ref = xo.xc_run(spec, src, rec, 1.0 / nwin, xo.finalize_shape(nspec, nwin, dt, lag))
    assert per_row_rel_l2(pruned, ref).max() < NCF_RTOL
    assert per_row_rel_l2(full, ref).max() < NCF_RTOL


# nspec - 1 = M, the complex transform length: one stage (31), two (58 =
# 2 x 29), the 256-thread kernel's limit (4096 = 8^4), odd composites
# (3003 = 3 x 7 x 11 x 13), five stages on the 1024-thread kernel
# (5000 = 8 x 5^4), the 37 044-point transform of 0.1 s hourly windows
# (18 522 = 2 x 3^3 x 7^3) and the 1024-thread kernel's limit (20 480)
@pytest.mark.parametrize("nspec", [32, 59, 3004, 4097, 5001, 18523, 20481])
def test_finalize_lag_cuts_match_oracle(ctx, torch_cuda, nspec):
    """fxc_xc_finalize alone on random stacks: the C2R runs with its first
    stage on the loads and its last stage formed only at the kept lags, so
    cuts of one lag, odd and even half-widths and the widest cut (every
    lag but one) are checked against numpy's FP64 irfft."""
    torch = torch_cuda
    from fastxc_gb300.core import xc_shape

    rng = np.random.default_rng(nspec)
    npairs = 5
    M = nspec - 1
    pitch = (nspec + 3) // 4 * 4
    stack = (rng.standard_normal((npairs, pitch)) + 1j * rng.standard_normal((npairs, pitch))).astype(np.complex64)
    d_stack = torch.from_numpy(stack).cuda()
    for half in sorted({0, 1, 7, min(100, M - 1), M // 3 | 1, M - 1}):
        lag = half + 0.25 if half else 0.4  # llround(lag / 1.0) = half
        shape = xc_shape(nspec, 1, 1.0, lag)
        assert shape.half_cc == half
        out = torch.full((npairs, shape.cc_size), float("nan"), dtype=torch.float32, device="cuda")
        ctx.xc_finalize(d_stack, npairs, pitch, shape, out)
        ctx.synchronize()
        got = out.cpu().numpy()
        ref = xo.xc_finalize(stack[:, :nspec], xo.finalize_shape(nspec, 1, 1.0, lag))
        assert np.all(np.isfinite(got)), (nspec, half)
        assert per_row_rel_l2(got, ref).max() < NCF_RTOL, (nspec, half)


@pytest.mark.parametrize("method", [0, 1], ids=["plain", "tensor"])
def test_20hz_long_transform(ctx, torch_cuda, method):
    """delta 0.05 s, 3600-s windows, lag 200 s: nfft 76 000-class transforms
    (nspec 37 045 here, nfft 74 088) above the one-CTA FFT limit, 8001 lags."""
    rng = np.random.default_rng(32)
    nwin, nsta, nspec = 3, 2, 37045
    spec = make_spec(rng, nwin, 3 * nsta, nspec)
    src, rec = station_pairs(nsta, auto=True)
    shape = ctx_shape(nspec, nwin, 0.05, 200.0)
    assert shape.cc_size == 8001 and shape.nfft == 74088
    got, _ = run_xc(ctx, torch_cuda, spec, src, rec, shape, 1.0 / nwin, method=method)
    ref = xo.xc_run(spec, src, rec, 1.0 / nwin, xo.finalize_shape(nspec, nwin, 0.05, 200.0))
    assert per_row_rel_l2(got, ref).max() < NCF_RTOL


def test_kernel_timing_counts_contraction_launches(ctx, torch_cuda):
    """fxc_ctx_kernel_timing brackets each contraction launch with events;
    the query returns their count and summed time once, then forgets them."""
    torch = torch_cuda
    from fastxc_gb300.core import PairPlan

    rng = np.random.default_rng(8)
    nwin, nchan, nspec = 130, 24, 301  # more than three K-blocks: the whole-bin kernel
    spec = make_spec(rng, nwin, nchan, nspec)
    src, rec = station_pairs(8)
    plan = PairPlan(ctx, src, rec, nchan)
    d_spec = torch.from_numpy(spec).cuda()
    d_stack = torch.zeros((src.size, nspec), dtype=torch.complex64, device="cuda")
    ctx.kernel_timing(True)
    for _ in range(3):
        ctx.xc_stack(plan, d_spec, nwin, nchan, nspec, nspec, None, 1.0, d_stack, nspec, 1)
    ms, n = ctx.kernel_time("k_xc_tc_gemm_bin")
    assert n == 3 and ms > 0.0
    assert ctx.kernel_time("k_xc_tc_gemm_bin") == (0.0, 0)
    ctx.kernel_timing(False)
    ctx.xc_stack(plan, d_spec, nwin, nchan, nspec, nspec, None, 1.0, d_stack, nspec, 1)
    assert ctx.kernel_time("k_xc_tc_gemm_bin") == (0.0, 0)
