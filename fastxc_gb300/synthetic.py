"""Seeded synthetic inputs with the shapes of the benchmark configurations.

No public dataset is involved. The station model follows the configuration
text: Gaussian noise plus a shared band-limited (0.1-2 Hz) coherent source
delayed per station by distance / 3 km/s, stations 10-80 km apart, and a
seeded fraction of windows zeroed as data gaps.

``spectra_device`` produces whitened-like output spectra directly in the
frequency domain (the layout the xc stage consumes: [window][channel][bin]
complex64), so the correlation stage can be benchmarked on its own.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class StationArray:
    nsta: int
    ncomp: int
    x_km: np.ndarray
    y_km: np.ndarray
    delay_s: np.ndarray  # coherent-source arrival delay per station

    @property
    def nchan(self) -> int:
        return self.nsta * self.ncomp


def station_array(nsta: int, seed: int = 0, ncomp: int = 3, extent_km: float = 80.0) -> StationArray:
    """Stations on a seeded random layout with pairwise separations of about
    10-80 km; the source sits 200 km away so delays differ per station."""
    rng = np.random.default_rng(seed)
    pts = []
    while len(pts) < nsta:
        p = rng.uniform(0, extent_km * 0.7, size=2)
        if all(np.hypot(*(p - q)) >= (10.0 if nsta <= 16 else 2.0) for q in pts):
            pts.append(p)
    pts = np.array(pts)
    src = np.array([-200.0, 35.0])
    dist = np.hypot(pts[:, 0] - src[0], pts[:, 1] - src[1])
    return StationArray(nsta, ncomp, pts[:, 0], pts[:, 1], dist / 3.0)


def cross_station_pairs(nsta: int, ncomp: int = 3, auto: bool = False):
    """All component pairs of all station pairs (s < t), src = lower station:
    the order of the reference's task list for one anchor block."""
    src, rec = [], []
    for s in range(nsta):
        for t in range(s if auto else s + 1, nsta):
            for i in range(ncomp):
                for j in range(ncomp):
                    src.append(s * ncomp + i)
                    rec.append(t * ncomp + j)
    return np.array(src, np.int32), np.array(rec, np.int32)


def band_taper(freqs: np.ndarray, lo: float, hi: float) -> np.ndarray:
    """Cosine band taper of the whitening step: zero below 0.667*lo and above
    1.333*hi, flat in [lo, hi]."""
    f1, f2, f3, f4 = 0.667 * lo, lo, hi, 1.333 * hi
    w = np.zeros_like(freqs)
    m = (freqs >= f1) & (freqs < f2)
    w[m] = 0.5 * (1 - np.cos(np.pi * (freqs[m] - f1) / (f2 - f1)))
    w[(freqs >= f2) & (freqs < f3)] = 1.0
    m = (freqs >= f3) & (freqs < f4)
    w[m] = 0.5 * (1 + np.cos(np.pi * (freqs[m] - f3) / (f4 - f3)))
    return w


def gap_mask(nwin: int, nchan: int, ncomp: int, frac: float, seed: int) -> np.ndarray:
    """[nwin][nchan] uint8, 0 = window zeroed as a gap (whole station)."""
    rng = np.random.default_rng(seed + 7919)
    nsta = nchan // ncomp
    sta = (rng.random((nwin, nsta)) >= frac).astype(np.uint8)
    return np.repeat(sta, ncomp, axis=1)


def spectra_device(torch, nwin: int, arr: StationArray, nspec: int, dt: float, seed: int = 0,
                   gap_frac: float = 0.05, band=(0.1, 2.0), device="cuda", out=None):
    """Whitened-like spectra [nwin][nchan][nspec] complex64 on the device.

    Y[w,c,f] = T(f) * (n[w,c,f] + g_c * C[w,f] * exp(-2 pi i f tau_s(c))),
    n, C complex Gaussian, T the whitening band taper, zero for gap windows.
    Returns (spectra, mask).
    """
    nfft = 2 * (nspec - 1)
    freqs = np.arange(nspec) / (nfft * dt)
    taper = torch.tensor(band_taper(freqs, *band), dtype=torch.float32, device=device)
    fr = torch.tensor(freqs, dtype=torch.float64, device=device)
    nchan = arr.nchan
    delays = torch.tensor(np.repeat(arr.delay_s, arr.ncomp), dtype=torch.float64, device=device)
    phase = torch.exp(-2j * np.pi * fr[None, :] * delays[:, None]).to(torch.complex64)  # [nchan][nspec]
    gains = torch.tensor(np.random.default_rng(seed + 1).uniform(0.5, 1.5, nchan), dtype=torch.float32,
                         device=device)[:, None]
    mask = gap_mask(nwin, nchan, arr.ncomp, gap_frac, seed)
    mask_d = torch.tensor(mask, dtype=torch.float32, device=device)
    if out is None:
        out = torch.empty((nwin, nchan, nspec), dtype=torch.complex64, device=device)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    for w in range(nwin):
        n = torch.randn((nchan, nspec), dtype=torch.complex64, device=device, generator=g)
        c = torch.randn((1, nspec), dtype=torch.complex64, device=device, generator=g)
        y = (n + 0.7 * gains * c * phase) * taper[None, :]
        out[w] = y * mask_d[w][:, None]
    return out, mask


def ricker(t: np.ndarray, f0: float) -> np.ndarray:
    a = (np.pi * f0 * t) ** 2
    return (1 - 2 * a) * np.exp(-a)


def ncf_traces(npairs: int, ntraces: int, nsamples: int = 2001, delta: float = 0.1, seed: int = 0,
               snr=(0.05, 0.5)) -> np.ndarray:
    """Stacking-configuration input: per pair `ntraces` NCF windows of
    `nsamples` lags holding a Ricker arrival (seeded f0 in 0.1-0.5 Hz) at a
    pair-specific lag plus Gaussian noise at an SNR drawn from `snr`.
    Returns float32 [npairs][ntraces][nsamples]."""
    rng = np.random.default_rng(seed)
    t = (np.arange(nsamples) - nsamples // 2) * delta
    out = np.empty((npairs, ntraces, nsamples), np.float32)
    for p in range(npairs):
        f0 = rng.uniform(0.1, 0.5)
        lag = rng.uniform(-0.6, 0.6) * t[-1]
        sig = ricker(t - lag, f0) + 0.6 * ricker(t + lag, f0)
        s = rng.uniform(*snr, size=ntraces)
        noise = rng.standard_normal((ntraces, nsamples))
        out[p] = (s[:, None] * sig[None, :] + noise).astype(np.float32)
    return out


def station_series(arr: StationArray, npts: int, delta: float, seed: int = 0, band=(0.1, 2.0),
                   source_amp: float = 3.0) -> np.ndarray:
    """Time series of the plain configurations: per channel N(0,1) noise plus
    a shared band-limited coherent source (4th-order zero-phase Butterworth
    over ``band``, its upper edge held below 0.9 of the Nyquist frequency)
    arriving at each station after its distance / 3 km/s delay, with a
    seeded gain per channel. Returns float32 [nchan][npts]."""
    from scipy.signal import butter, sosfiltfilt

    band = (band[0], min(band[1], 0.45 / delta))
    rng = np.random.default_rng(seed)
    shifts = np.round(arr.delay_s / delta).astype(np.int64)
    lead = int(shifts.max()) + 1
    sos = butter(4, list(band), "bandpass", fs=1.0 / delta, output="sos")
    src = sosfiltfilt(sos, rng.standard_normal(npts + lead))
    gains = rng.uniform(0.5, 1.5, arr.nchan)
    out = np.empty((arr.nchan, npts), np.float32)
    for s in range(arr.nsta):
        start = lead - int(shifts[s])
        sig = src[start: start + npts]
        for c in range(arr.ncomp):
            ch = s * arr.ncomp + c
            out[ch] = (rng.standard_normal(npts) + source_amp * gains[ch] * sig).astype(np.float32)
    return out
