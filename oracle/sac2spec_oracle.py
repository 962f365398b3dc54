"""FP64 restatement of the sac2spec stage (SAC windows -> output spectra).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Planning (segment/FFT lengths, band indices, taper and smoothing windows)
reproduces the reference's integer and float32 arithmetic exactly and is
pinned against the reference's own C sources compiled on the CPU
(``oracle/build_ref.py``: native/sac2spec/fft_length.c and
native/sac2spec/core/filter_response.c). The signal path restates the kernel
sequence of ComputeWorkerBatch (native/sac2spec/worker/compute.cu:8-272) in
FP64 numpy, with numpy's FFT in place of cuFFT.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

f32 = np.float32
MAXVAL = 20.0  # native/sac2spec/include/config.h:13
MINVAL = 1e-30  # native/sac2spec/include/config.h:14

WHITEN_NONE, WHITEN_BEFORE, WHITEN_AFTER, WHITEN_BOTH = 0, 1, 2, 3
NORM_NONE, NORM_RUNABS_MF, NORM_ONEBIT, NORM_RUNABS = 0, 1, 2, 3


def llround(x: float) -> int:
    return int(math.floor(abs(x) + 0.5)) * (1 if x >= 0 else -1)


# ---------------------------------------------------------------------------
# FFT lengths: native/sac2spec/fft_length.c
# ---------------------------------------------------------------------------


def is_smooth_2357(v: int) -> bool:
    """fft_length.c:20-37."""
    if v < 1:
        return False
    for p in (2, 3, 5, 7):
        while v > 1 and v % p == 0:
            v //= p
    return v == 1


def next_smooth_2357(n: int) -> int:
    """fft_length.c:39-55."""
    n = max(n, 1)
    while not is_smooth_2357(n):
        n += 1
    return n


def next_even_smooth_2357(n: int) -> int:
    """fft_length.c:57-65."""
    n = next_smooth_2357(n)
    while n % 2 != 0:
        n = next_smooth_2357(n + 1)
    return n


def previous_smooth_2357(max_len: int) -> int:
    """fft_length.c:67-88 (returns 0 on failure)."""
    if max_len <= 1:
        return 0
    n = max_len - 1
    while n > 0:
        if is_smooth_2357(n):
            return n
        n -= 1
    return 0


def seconds_to_nearest_samples(seconds: float, delta: float) -> int:
    """fft_length.c:8-18 (seconds, delta are float32)."""
    s, d = float(f32(seconds)), float(f32(delta))
    if s <= 0 or d <= 0:
        return 0
    v = s / d
    if not math.isfinite(v) or v > 2147483647:
        return 2147483647
    return llround(v)


def segment_length_from_seconds(seconds: float, max_samples: int, delta: float) -> int:
    """fft_length.c:90-108."""
    seg = next_smooth_2357(seconds_to_nearest_samples(seconds, delta))
    if seg > max_samples:
        seg = previous_smooth_2357(max_samples)
    return seg


# ---------------------------------------------------------------------------
# Butterworth filters: native/sac2spec/core/filter_response.c
# ---------------------------------------------------------------------------


@dataclass
class ButterworthFilter:
    freq_low: float
    freq_high: float
    b: np.ndarray
    a: np.ndarray


def read_filter_file(path) -> list[ButterworthFilter]:
    """readButterworthFilters (filter_response.c:129-184): '# lo/hi' then a b
    line and an a line of 5 coefficients each."""
    out = []
    state = 0
    lo = hi = 0.0
    b = None
    for line in open(path, encoding="ascii"):
        if line.startswith("#"):
            try:
                tag = line[1:].strip()
                l, h = tag.split("/")
                lo, hi = float(f32(float(l))), float(f32(float(h)))
                state = 1
            except ValueError:
                pass
            continue
        vals = line.split()
        if state == 1:
            if len(vals) >= 5:
                b = np.array([float(v) for v in vals[:5]])
                state = 2
            continue
        if state == 2:
            if len(vals) >= 5:
                out.append(ButterworthFilter(lo, hi, b, np.array([float(v) for v in vals[:5]])))
            state = 0
    return out


def write_filter_file(path, filters: list[ButterworthFilter]) -> None:
    """Format of fastxc/operators/filter_design.py:58-67 ('%.18e' tab-separated)."""
    with open(path, "w", encoding="ascii") as fh:
        for flt in filters:
            fh.write(f"# {flt.freq_low}/{flt.freq_high}\n")
            fh.write("\t".join(f"{v:.18e}" for v in flt.b) + "\n")
            fh.write("\t".join(f"{v:.18e}" for v in flt.a) + "\n")


def design_filters(delta: float, bands: str, order: int = 2) -> list[ButterworthFilter]:
    """design_filter (fastxc/operators/filter_design.py:14-56): the broad band
    first, then every configured band; scipy butter bandpass."""
    from scipy.signal import butter

    pairs = [tuple(map(float, b.split("/"))) for b in bands.split()]
    fnyq = 0.5 / delta
    lo_all = min(p[0] for p in pairs)
    hi_all = max(p[1] for p in pairs)
    out = []
    b, a = butter(order, [lo_all / fnyq, hi_all / fnyq], "bandpass")
    out.append(ButterworthFilter(lo_all, hi_all, b, a))
    for lo, hi in pairs:
        b, a = butter(order, [lo / fnyq, hi / fnyq], "bandpass")
        out.append(ButterworthFilter(lo, hi, b, a))
    return out


def impulse_length(flt: ButterworthFilter, max_samples: int) -> int:
    """estimateSinglePassImpulseLength (filter_response.c:11-72)."""
    a0 = flt.a[0]
    if abs(a0) < 1e-30:
        return max_samples
    xh = [0.0] * 5
    yh = [0.0] * 5
    resp = np.zeros(max_samples)
    total = 0.0
    for n in range(max_samples):
        xh = [1.0 if n == 0 else 0.0] + xh[:4]
        yh = [0.0] + yh[:4]
        y = sum(flt.b[j] * xh[j] for j in range(5))
        for j in range(1, 5):
            y -= flt.a[j] * yh[j]
        y /= a0
        yh[0] = y
        resp[n] = y
        total += y * y
    if total <= 0:
        return 1
    tail = 0.0
    for n in range(max_samples - 1, -1, -1):
        tail += resp[n] * resp[n]
        if tail > total * 1e-6:
            return n + 1
    return 1


def filter_padding(filters, max_padding: int) -> int:
    """estimateButterworthFilterPadding (filter_response.c:74-104)."""
    m = 1
    for f in filters:
        m = max(m, impulse_length(f, max_padding))
    return min(max(2 * m, 1), max_padding)


def filter_power_response(flt: ButterworthFilter, nfft: int) -> np.ndarray:
    """calFilterPowerResp (filter_response.c:186-233): |B/A|^2 on bins
    i/half, i in [0, half], stored as float32."""
    half = nfft // 2
    f = np.arange(half + 1) / half
    j = np.arange(5)
    ang = -np.pi * f[:, None] * j[None, :]
    B = (flt.b[None, :] * np.exp(1j * ang)).sum(1)
    A = (flt.a[None, :] * np.exp(1j * ang)).sum(1)
    num = np.abs(B) ** 2
    den = np.abs(A) ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(den <= np.finfo(np.float64).tiny, 0.0, num / den)
    r = np.where(np.isfinite(r), r, 0.0)
    r = np.minimum(r, np.finfo(np.float32).max)
    return r.astype(np.float32)


# ---------------------------------------------------------------------------
# Plan: native/sac2spec/cuda.main.cu:203-296
# ---------------------------------------------------------------------------


@dataclass
class Sac2SpecPlan:
    delta: float
    npts: int
    segment_pts: int
    shift_pts: int
    nstep: int
    output_nfft: int
    nspec: int
    filter_nfft: int
    filter_padding: int
    freq_low: float
    freq_high: float
    f_idx: tuple
    taper_pts: int
    runabs_win: int
    whiten_win: int
    whiten: int = WHITEN_AFTER
    normalize: int = NORM_RUNABS
    phase_only: int = 0
    freq_lows: list = field(default_factory=list)
    responses: np.ndarray | None = None  # [nfilters][filter_nfft/2+1] float32


def runabs_window(freq_low: float, delta: float) -> int:
    """runabsNormalizeSharedWeight (core/normalization.cu:130-134)."""
    w = 2 * int(1.0 / float(f32(f32(freq_low) * f32(delta)))) + 1
    return max(w, 1)


def make_plan(sac_len: float, win_len: float, shift_len: float, xcorr_lag: float, delta: float,
              filters: list[ButterworthFilter], whiten: int = WHITEN_AFTER, normalize: int = NORM_RUNABS,
              phase_only: int = 0) -> Sac2SpecPlan:
    d32 = f32(delta)
    npts = llround(float(f32(sac_len)) / float(d32))
    seg = segment_length_from_seconds(win_len, npts, delta)
    shift = llround(float(f32(shift_len)) / float(d32))
    if shift < 1:
        shift = seg
    if seg <= npts:
        nstep = max((npts - seg) // shift + 1, 1)
    else:
        nstep = 1
    max_out = seg * 2
    keep = llround(float(f32(xcorr_lag)) / float(d32))
    keep = min(keep, seg)
    out_nfft = min(next_even_smooth_2357(seg + keep), max_out)
    nspec = out_nfft // 2 + 1
    seg_df = f32(1.0) / f32(f32(seg) * d32)
    lo, hi = f32(filters[0].freq_low), f32(filters[0].freq_high)
    f_idx = (int(f32(f32(lo * f32(0.667)) / seg_df)), int(f32(lo / seg_df)), int(f32(hi / seg_df)),
             int(f32(f32(hi * f32(1.333)) / seg_df)))
    pad = filter_padding(filters, seg)
    fnfft = min(next_even_smooth_2357(seg + pad), max_out)
    taper = int(f32(f32(f32(2.0) * f32(f32(1.0) / lo)) / d32))
    raw = runabs_window(float(f32(lo * f32(0.667))), delta)
    ww = max(int(0.02 * seg * float(d32)), 1)
    resp = np.stack([filter_power_response(f, fnfft) for f in filters])
    return Sac2SpecPlan(float(d32), npts, seg, shift, nstep, out_nfft, nspec, fnfft, pad, float(lo), float(hi),
                        f_idx, taper, raw, ww, whiten, normalize, phase_only,
                        [float(f32(f.freq_low)) for f in filters], resp)


# ---------------------------------------------------------------------------
# Signal path (rows = windows of single channels; num_ch consecutive rows
# belong to one station and share normalisation / whitening weights)
# ---------------------------------------------------------------------------


def preprocess(x: np.ndarray, freq_low: float, delta: float) -> np.ndarray:
    """core/preprocess.cu:23-105 with kernels/rdcrtr.cu and kernels/taper.cu:
    NaN/Inf -> 0, demean, detrend (closed-form least squares), Hann taper of
    (int)(2/f_low/delta) samples at both ends."""
    x = np.where(np.isfinite(x), x, 0.0).astype(np.float64)
    n = x.shape[-1]
    x = x - x.sum(-1, keepdims=True) / n
    i = np.arange(n, dtype=np.float64)
    y1 = (x * i).sum(-1, keepdims=True)
    y2 = x.sum(-1, keepdims=True)
    a12 = 0.5 * n * (n - 1)
    a11 = a12 * (2 * n - 1) / 3.0
    a22 = float(n)
    det = a11 * a22 - a12 * a12
    a = (a22 * y1 - a12 * y2) / det
    b = (a11 * y2 - a12 * y1) / det
    x = x - (a * i + b)
    taper = int(f32(f32(f32(2.0) * f32(f32(1.0) / f32(freq_low))) / f32(delta)))
    fac = np.ones(n)
    if taper > 0:
        c = np.arange(n)
        left = c < taper
        fac[left] = 0.5 * (1 - np.cos(np.pi * c[left] / taper))
        right = (~left) & (c >= n - taper)
        fac[right] = 0.5 * (1 - np.cos(np.pi * (n - c[right]) / taper))
    return x * fac


def _rfft(x, n, delta):
    return np.fft.rfft(x, n=n, axis=-1) * delta


def _irfft(X, n, delta):
    # unnormalised C2R (imaginary DC/Nyquist ignored) x 1/(n*delta)
    return np.fft.irfft(X, n=n, axis=-1) * n / (n * delta)


def _sanitize(X):
    bad = ~(np.isfinite(X.real) & np.isfinite(X.imag))
    return np.where(bad, 0, X)


def apply_filter(x: np.ndarray, resp: np.ndarray, nfft: int, delta: float) -> np.ndarray:
    """compute.cu:59-86: zero-pad to nfft, R2C x dt, sanitize, x |H|^2, C2R x
    1/(nfft*dt), truncate."""
    seg = x.shape[-1]
    X = _sanitize(_rfft(x, nfft, delta)) * resp.astype(np.float64)
    return _irfft(X, nfft, delta)[..., :seg]


def smooth_rows(src: np.ndarray, win: int) -> np.ndarray:
    """smoothRowsRollingKernel (kernels/real_matrix.cu:155-191): centred boxcar
    over [c - win//2, c - win//2 + win - 1] clipped to the row, divided by win."""
    n = src.shape[-1]
    cs = np.concatenate([np.zeros(src.shape[:-1] + (1,)), np.cumsum(src, axis=-1)], axis=-1)
    c = np.arange(n)
    lo = np.clip(c - win // 2, 0, n)
    hi = np.clip(c - win // 2 + win, 0, n)
    return (cs[..., hi] - cs[..., lo]) / win


def _group_sum(w: np.ndarray, num_ch: int) -> np.ndarray:
    """Sum of a weight over the num_ch rows of each station (rows are
    [..., group*num_ch + ch]), broadcast back to every row."""
    shp = w.shape
    g = w.reshape(shp[:-2] + (shp[-2] // num_ch, num_ch, shp[-1]))
    s = g.sum(axis=-2, keepdims=True)
    return np.broadcast_to(s, g.shape).reshape(shp)


def runabs(x: np.ndarray, freq_low: float, delta: float, num_ch: int) -> np.ndarray:
    """runabsNormalizeSharedWeight (core/normalization.cu:91-213)."""
    win = runabs_window(freq_low, delta)
    w = _group_sum(smooth_rows(np.abs(x), win), num_ch)
    w = np.where(np.isfinite(w) & (w >= MINVAL), w, MINVAL)
    y = x / w
    y = np.where(np.isfinite(y), y, 0.0)
    return np.clip(y, -MAXVAL, MAXVAL)


def onebit(x: np.ndarray) -> np.ndarray:
    """onebit2DKernel (kernels/real_matrix.cu:127-140)."""
    return np.sign(x)


def spectral_taper(X: np.ndarray, idx) -> np.ndarray:
    """specTaper2DKernel (kernels/taper.cu:8-69), np = 1."""
    i1, i2, i3, i4 = idx
    width = X.shape[-1]
    i4 = min(i4, width)
    c = np.arange(width)
    fac = np.ones(width)
    fac[c < i1] = 0.0
    m = (c >= i1) & (c < i2)
    fac[m] = (1 - np.cos(np.pi / (i2 - i1) * (c[m] - i1))) / 2
    m = (c >= i3) & (c < i4) & ~(c < i2)
    fac[m] = (1 + np.cos(np.pi / (i4 - i3) * (c[m] - i3))) / 2
    fac[(c >= i4) & (c >= i2)] = 0.0
    return X * fac


def freq_whiten(x: np.ndarray, plan: Sac2SpecPlan, num_ch: int) -> np.ndarray:
    """compute.cu:187-217 + freq_whiten (core/spectrum.cu:178-305): R2C(seg)
    x dt, sanitize, |X| boxcar over whiten_win bins summed over the station's
    channels, clamp, X/w, band taper, sanitize, C2R x 1/(seg*dt)."""
    seg = x.shape[-1]
    X = _sanitize(_rfft(x, seg, plan.delta))
    w = _group_sum(smooth_rows(np.abs(X), plan.whiten_win), num_ch)
    w = np.where(np.isfinite(w) & (w >= MINVAL), w, MINVAL)
    X = _sanitize(spectral_taper(X / w, plan.f_idx))
    return _irfft(X, seg, plan.delta)


def output_spectrum(x: np.ndarray, plan: Sac2SpecPlan) -> np.ndarray:
    """compute.cu:226-252: zero-pad to output_nfft, R2C x dt, sanitize,
    optional phase-only (amp <= 1e-30 -> 0)."""
    X = _sanitize(_rfft(x, plan.output_nfft, plan.delta))
    if plan.phase_only:
        amp = np.abs(X)
        X = np.where(amp <= MINVAL, 0, X / np.where(amp <= MINVAL, 1, amp))
    return X


def run_rows(x: np.ndarray, plan: Sac2SpecPlan, num_ch: int) -> np.ndarray:
    """ComputeWorkerBatch (compute.cu:8-272) on rows [..., nrows, seg]; rows
    are ordered group*num_ch + ch. Returns [..., nrows, nspec] complex128."""
    x = preprocess(np.asarray(x, dtype=np.float64), plan.freq_low, plan.delta)
    x = apply_filter(x, plan.responses[0], plan.filter_nfft, plan.delta)
    if plan.whiten in (WHITEN_BEFORE, WHITEN_BOTH):
        x = freq_whiten(x, plan, num_ch)
    if plan.normalize == NORM_RUNABS_MF:
        total = np.zeros_like(x)
        X0 = _sanitize(_rfft(x, plan.filter_nfft, plan.delta))
        for i in range(1, len(plan.freq_lows)):
            xb = _irfft(X0 * plan.responses[i].astype(np.float64), plan.filter_nfft, plan.delta)[..., : x.shape[-1]]
            total = total + runabs(xb, plan.freq_lows[i], plan.delta, num_ch)
        x = total
    elif plan.normalize == NORM_ONEBIT:
        x = onebit(x)
    elif plan.normalize == NORM_RUNABS:
        x = runabs(x, float(f32(f32(plan.freq_low) * f32(0.667))), plan.delta, num_ch)
    if plan.whiten in (WHITEN_AFTER, WHITEN_BOTH):
        x = freq_whiten(x, plan, num_ch)
    return output_spectrum(x, plan)


def windows(series: np.ndarray, plan: Sac2SpecPlan, steps) -> np.ndarray:
    """compute.cu:31-45: window k = samples [k*shift, k*shift+seg) of every
    channel -> [len(steps)][nrows][seg]."""
    return np.stack([series[:, s * plan.shift_pts: s * plan.shift_pts + plan.segment_pts] for s in steps])
