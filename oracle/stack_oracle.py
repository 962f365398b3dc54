"""FP64 restatement of the stacking stages: cross-timestamp linear stack,
phase-weighted stack (ncf_pws) and S-transform time-frequency PWS
(ncf_tfpws).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

The linear stack is pinned against the reference's own Python
(tests/golden/linear_stack_golden.npz). PWS / TF-PWS restate the kernel
sequence of native/pws/worker/gpu.cu:87-282 + kernels/cuda.pws.cu and
native/tfpws/core/tfpws_compute.cu:19-366 + kernels/cuda.stransform.cu with
numpy's FFT in place of cuFFT; the reference ships no golden stacks, so
those float paths are "parity unpinned" beyond this restatement.
"""

from __future__ import annotations

import numpy as np


def linear_stack(traces: np.ndarray) -> np.ndarray:
    """_linear_stack_group (fastxc/operators/stacking/linear_stack.py:228-247):
    FP64 accumulation in record order, divide by the count, cast to float32."""
    acc = np.asarray(traces[0]).astype(np.float64)
    for t in traces[1:]:
        acc = acc + np.asarray(t).astype(np.float64)
    return (acc / float(len(traces))).astype(np.float32)


# ---------------------------------------------------------------------------
# Substack preparation (host side of the reference)
# ---------------------------------------------------------------------------


def pws_prestack(traces: np.ndarray, substack: int):
    """prepare_sourcepack_host_item (native/pws/io/sourcepack_io.cu:385-478):
    groups of `substack` consecutive traces (B < 2 -> 1), each group averaged,
    group weight = count / num_segments, linear = sum(mean * weight)."""
    n = traces.shape[0]
    b = substack if substack >= 2 else 1
    groups, weights = [], []
    for g0 in range(0, n, b):
        g = traces[g0:g0 + b].astype(np.float64)
        groups.append(g.mean(axis=0))
        weights.append(g.shape[0] / n)
    groups = np.array(groups)
    weights = np.array(weights)
    linear = (groups * weights[:, None]).sum(axis=0)
    return groups, weights, linear


def tfpws_prestack(traces: np.ndarray, substack: int):
    """TF-PWS prestack (native/tfpws/io/sourcepack_io.cu:440-490): group SUMS,
    weight = count / num_segments, linear = sum of sums / num_segments."""
    n = traces.shape[0]
    b = substack if substack >= 2 else 1
    groups, weights = [], []
    for g0 in range(0, n, b):
        g = traces[g0:g0 + b].astype(np.float64)
        groups.append(g.sum(axis=0))
        weights.append(g.shape[0] / n)
    groups = np.array(groups)
    linear = groups.sum(axis=0) / n
    return groups, np.array(weights), linear


def analytic(x: np.ndarray) -> np.ndarray:
    """R2C(N) into an N-point complex row, then hilbertTransformKernel
    (native/pws/kernels/cuda.pws.cu:3-26): bin 0 and bins >= (N+1)/2 -> 0,
    others x 2; C2C inverse (unnormalised)."""
    n = x.shape[-1]
    X = np.fft.fft(x, axis=-1)
    half = (n + 1) // 2
    k = np.arange(n)
    X = np.where((k == 0) | (k >= half), 0, 2 * X)
    return X


def pws(traces: np.ndarray, substack: int = 1, power: float = 1.0) -> np.ndarray:
    """compute_pws_host_batch (native/pws/worker/gpu.cu:87-282) for one pair:
    analytic signal of every group (unnormalised inverse / N), unit phasor
    with modulus floor 1e-7 (cudaNormalizeComplex), weighted mean
    (cudaWeightedMeanBatch), pws = linear * |mean|^power (cudaMultiplyBatch,
    power 1 in the reference)."""
    groups, w, linear = pws_prestack(traces, substack)
    n = groups.shape[-1]
    z = np.fft.ifft(analytic(groups), axis=-1) * n / n
    mod = np.maximum(np.abs(z), 1e-7)
    ph = z / mod
    mean = (w[:, None] * ph).sum(axis=0)
    return linear * np.abs(mean) ** power


def gaussian_window(n: int, f: int, scale: float = 0.1) -> np.ndarray:
    """gaussianModulateSub factor for centre bin f over shifts c in [0, n)
    (native/tfpws/kernels/cuda.stransform.cu:59-153): f = 0 -> 1; c = 0 -> 0;
    c < (n+1)/2 -> exp(-2 pi^2 c^2 scale / f^2); else mirrored c' = n - c."""
    c = np.arange(n)
    if f == 0:
        return np.ones(n)
    half = (n + 1) // 2
    cc = np.where(c < half, c, n - c).astype(np.float64)
    g = np.exp(-2.0 * np.pi ** 2 * cc * cc * scale / (float(f) * f))
    g[0] = 0.0
    mirror_bad = (c >= half) & ((n - c) >= half)
    g[mirror_bad] = 0.0
    return g


def tfpws(traces: np.ndarray, substack: int = 1, power: float = 1.0, band=None, taper_hz=None,
          delta: float = 0.1) -> np.ndarray:
    """compute_tfpws_from_prestack (native/tfpws/core/tfpws_compute.cu:19-366)
    for one pair: analytic spectra of the group sums and of the linear
    stack; for every frequency f < n/2+1 the S-transform voices (inverse FFT
    of the circularly shifted, Gaussian-modulated spectrum), the weight
    W = sum_g w_g v_g / (|v_g| N) (|v| <= 1e-7 -> 1), the stack voice times
    |W|^power summed over time into bin f; optional band blend; final C2C
    inverse, real part / N."""
    groups, w, linear = tfpws_prestack(traces, substack)
    n = groups.shape[-1]
    nfreq = n // 2 + 1
    Xg = analytic(groups)
    Xl = analytic(linear[None, :])[0]
    out = np.zeros(n, dtype=np.complex128)
    df = 1.0 / (n * delta)
    if band is not None:
        out[:] = Xl
        fmin, fmax = band
        nyq = 0.5 / delta
        fmax = min(fmax, nyq)
        if taper_hz is None or taper_hz < 0:
            taper_hz = 0.05 * (fmax - fmin)
    k = np.arange(n)
    for f in range(nfreq):
        if band is not None:
            freq = f * df
            # the reference skips whole chunks outside the band; bins with
            # alpha = 0 keep the linear spectrum either way
            if not (band[0] <= freq <= min(band[1], 0.5 / delta)):
                continue
        g = gaussian_window(n, f)
        idx = (f + k) % n
        vs = np.fft.ifft(Xl[idx] * g) * n
        vg = np.fft.ifft(Xg[:, idx] * g[None, :], axis=-1) * n
        a = np.abs(vg)
        a = np.where(a <= 1e-7, 1.0, a)
        W = (w[:, None] * vg / (a * n)).sum(axis=0)
        val = (vs * np.abs(W) ** power).sum()
        if band is not None:
            fmin, fmax = band[0], min(band[1], 0.5 / delta)
            freq = f * df
            bw = fmax - fmin
            tp = min(taper_hz, 0.5 * bw)
            if tp <= 0:
                alpha = 1.0
            elif freq < fmin + tp:
                alpha = 0.5 - 0.5 * np.cos(np.pi * (freq - fmin) / tp)
            elif freq > fmax - tp:
                alpha = 0.5 - 0.5 * np.cos(np.pi * (fmax - freq) / tp)
            else:
                alpha = 1.0
            out[f] = Xl[f] * (1 - alpha) + val * alpha
        else:
            out[f] = val
    return (np.fft.ifft(out) * n).real / n
