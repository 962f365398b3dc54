// sac2spec hot path: SAC windows -> preprocessed, normalised, whitened
// output spectra (the stepack payload [step][row][nspec] complex64).
//
// Reference: ComputeWorkerBatch (native/sac2spec/worker/compute.cu:8-272)
// and the kernels it launches (native/sac2spec/kernels/*.cu,
// native/sac2spec/core/{preprocess,normalization,spectrum}.cu); about 30
// launches and 5 cuFFT executions per batch there.
//
// GB300 design: one CTA (1024 threads) per (window, channel) row keeps the
// whole row and its transform in shared memory. A real transform of length
// 2M runs as a length-M complex FFT: forward DIF (natural in, digit-reversed
// out), a pointwise pass over the bin pairs (k, M-k) that does the real
// post-processing, the per-bin work (x dt, sanitize, |H|^2, whitening
// divide, band taper) and the inverse pre-processing in place, then an
// inverse DIT (digit-reversed in, natural out) -- no permutation pass and
// no HBM round trip between the forward and the inverse transform.
// Coupling across the num_ch components of a station (running-absolute-mean
// weights, whitening weights) goes through small HBM buffers between
// kernels:
//   k_s2s_front     load window, NaN->0, FP64 demean/detrend sums, Hann
//                   taper, prefilter (R2C, x dt, sanitize, x |H|^2, C2R,
//                   x 1/(N dt)), then one-bit or the smoothed |x| weight
//   k_s2s_mfband    (RUN-ABS-MF) per band: R2C, x |H_band|^2, C2R, weight
//   k_s2s_mfsum     (RUN-ABS-MF) sum of the normalised bands
//   k_s2s_whiten_a  [RAM divide] R2C(seg), x dt, sanitize, smoothed |X|
//   k_s2s_whiten_b  divide by the station weight, band taper, sanitize,
//                   C2R, then either the output transform or the time row
//   k_s2s_output    [RAM divide] zero-pad, R2C(output_nfft), x dt,
//                   sanitize, optional phase-only
//   k_s2s_station   the whole chain for the three components of a station
//                   window in one 3-CTA cluster, the weights exchanged
//                   through distributed shared memory (used where it
//                   applies; the kernels above otherwise)
// Each thread issues the global loads of 4-8 items before using any, and
// the pointwise passes read a batch of bin pairs before writing: one CTA per
// SM leaves no other CTA to hide load latency.
// Boxcar smoothing keeps the reference's window and divisor. The reference's
// FP64 sums and products (demean, detrend, normalisations) run as FP32 with
// Kahan-compensated sums, double-float block reductions and two-float
// constants (F2c below) formed on the host or by one thread: GB300's FP64
// pipe issues at 1/64 of its FP32 rate.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cooperative_groups.h>

// Every FFT stage of these row kernels runs inline: called through the ABI,
// each stage and transform call saved and restored live registers in local
// memory (about 3 MB of local traffic per row at the 64-register cap of
// 1024 threads); inline, the station kernel runs 6.50 -> 5.32 ms for 4608
// rows.
#define FXC_FFT_STAGE_ATTR __forceinline__
#define FXC_FFT_NL_ATTR __forceinline__
#include "context.cuh"
#include "fft.cuh"
#include "fft_launch.cuh"

namespace fxc {

#ifndef FXC_S2S_THREADS
#define FXC_S2S_THREADS 1024
#endif
constexpr int kS2sT = FXC_S2S_THREADS;
constexpr float kMaxVal = 20.0f;  // MAXVAL, native/sac2spec/include/config.h:13
constexpr float kMinValF = 1e-30f;  // MINVAL passed as a float (clampmin2DKernel)

// A double constant c as the unevaluated sum hi + lo of two floats.
struct F2c {
  float hi, lo;
};
__host__ __device__ inline F2c f2c(double c) {
  F2c r;
  r.hi = (float)c;
  r.lo = (float)(c - (double)r.hi);
  return r;
}

struct S2sDev {
  float delta;
  int seg, shift, filter_nfft, out_nfft, nspec;
  int taper;
  int f_idx1, f_idx2, f_idx3, f_idx4;
  int phase_only;
  int num_ch;
  int nrows;  // rows per step
  F2c inrm_f;  // 1 / (filter_nfft dt): prefilter round trip
  F2c inrm_s;  // 1 / (seg dt): whitening round trip
  F2c inv_rw;  // 1 / runabs_win
  F2c inv_ww;  // 1 / whiten_win
  // detrend least squares over i = 0 .. seg-1 (rtr2DKernel):
  double a11, a12, a22, inv_det;
};

// ---------------------------------------------------------------------------
// block helpers
// ---------------------------------------------------------------------------

// Sums over the CTA of N threads' compensated values (v_i = hi_i + lo_i),
// returned in double by thread 0 (0 elsewhere). Warps reduce in
// double-float FP32 arithmetic (error-free two-sums), so the only FP64
// operations are one warp's: GB300 issues FP64 at 1/64 of the FP32 rate.
__device__ __forceinline__ void df_add(float& ah, float& al, float bh, float bl) {
  const float s = ah + bh;
  const float v = s - ah;
  float e = (ah - (s - v)) + (bh - v);
  e += al + bl;
  ah = s + e;
  al = e - (ah - s);
}

template <int N>
__device__ __forceinline__ void block_sums_t0(const float (&hi)[N], const float (&lo)[N], double* sred,
                                              double (&out)[N]) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const int nw = (int)(blockDim.x >> 5);
#pragma unroll
  for (int q = 0; q < N; ++q) {
    float h = hi[q], e = lo[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, h, o);
      const float oe = __shfl_xor_sync(0xffffffffu, e, o);
      df_add(h, e, oh, oe);
    }
    if (l == 0) sred[q * 32 + w] = (double)h + (double)e;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < N; ++q) {
    double t = 0.0;
    if (w == 0) {
      t = l < nw ? sred[q * 32 + l] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    out[q] = threadIdx.x == 0 ? t : 0.0;
  }
  __syncthreads();  // sred free again
}

// GB300 runs FP64 at a small fraction of its FP32 rate, so per-sample work
// stays in FP32. A double constant c becomes the unevaluated sum hi + lo of
// two floats; x * c = fma(x, hi, x * lo) is within an ulp of the float of
// the double product. Sums over a row are Kahan-compensated FP32 per thread
// with the block reduction in double-float. Plan constants are formed on the
// host, per-row ones by one thread.
__device__ __forceinline__ float mul_f2c(float x, F2c c) { return fmaf(x, c.hi, x * c.lo); }
struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

__device__ __forceinline__ bool finite2(float2 v) { return isfinite(v.x) && isfinite(v.y); }
__device__ __forceinline__ float2 sanitize2(float2 v) {
  return finite2(v) ? v : make_float2(0.f, 0.f);
}

// Centred boxcar of width win over src[0, n) (reference smoothRowsRollingKernel:
// window [c - win/2, c - win/2 + win - 1] clipped to the row, divided by win)
// for the outputs c in [a, b), written to dst[c - a]. Each thread owns a
// contiguous run of outputs and slides a Kahan-compensated FP32 sum across
// it; the first window is summed in four interleaved compensated sums (four
// independent dependency chains) and combined. Out of line: the caller's
// live values stay out of the loop's registers. ABS takes |src|.
__device__ __forceinline__ void kahan_add(float& s, float& comp, float v) {
  const float y = v - comp;
  const float t = s + y;
  comp = (t - s) - y;
  s = t;
}

// Runs of an odd length: the 32 lanes of a warp then start 32 distinct
// shared-memory banks apart (an even run length folds them onto 16 or fewer
// banks, a 4-way conflict for a run of 36 on every window read).
__device__ __forceinline__ int odd_run(int n) { return ((n + kS2sT - 1) / kS2sT) | 1; }

template <bool ABS>
__device__ __noinline__ void boxcar_range(const float* src, int n, int win, F2c inv, int a, int b, float* dst) {
  const int per = odd_run(b - a);
  const int c0 = a + threadIdx.x * per;
  if (c0 >= b) return;
  const int c1 = min(b, c0 + per);
  const int half = win / 2;
  const int lo = max(0, c0 - half), hi = min(n - 1, c0 - half + win - 1);
  float s4[4] = {0.f, 0.f, 0.f, 0.f}, k4[4] = {0.f, 0.f, 0.f, 0.f};
  int j = lo;
  for (; j + 3 <= hi; j += 4) {
#pragma unroll
    for (int q = 0; q < 4; ++q) kahan_add(s4[q], k4[q], ABS ? fabsf(src[j + q]) : src[j + q]);
  }
  for (; j <= hi; ++j) kahan_add(s4[0], k4[0], ABS ? fabsf(src[j]) : src[j]);
  float s = 0.f, comp = 0.f;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    kahan_add(s, comp, s4[q]);
    kahan_add(s, comp, -k4[q]);
  }
  for (int c = c0; c < c1; ++c) {
    dst[c - a] = mul_f2c(s, inv);
    const int out = c - half;      // leaves the window
    const int in = c - half + win;  // enters the window
    if (out >= 0 && out < n) kahan_add(s, comp, -(ABS ? fabsf(src[out]) : src[out]));
    if (in >= 0 && in < n) kahan_add(s, comp, ABS ? fabsf(src[in]) : src[in]);
  }
}

// The boxcar of a[0, n) (no abs) written back over a (n <= RMAX x threads):
// each thread keeps its run of outputs in registers until every thread has
// read its window, then stores it. Ends with the CTA synchronised.
constexpr int kRunRegs = 21;  // boxcar_inplace run per thread (odd): n <= 21 x 1024

template <int RMAX>
__device__ __noinline__ void boxcar_inplace(float* a, int n, int win, F2c inv) {
  const int per = odd_run(n);
  const int c0 = threadIdx.x * per;
  const int c1 = min(n, c0 + per);
  float r[RMAX];
  if (c0 < n) {
    const int half = win / 2;
    const int lo = max(0, c0 - half), hi = min(n - 1, c0 - half + win - 1);
    float s4[4] = {0.f, 0.f, 0.f, 0.f}, k4[4] = {0.f, 0.f, 0.f, 0.f};
    int j = lo;
    for (; j + 3 <= hi; j += 4) {
#pragma unroll
      for (int q = 0; q < 4; ++q) kahan_add(s4[q], k4[q], a[j + q]);
    }
    for (; j <= hi; ++j) kahan_add(s4[0], k4[0], a[j]);
    float s = 0.f, comp = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      kahan_add(s, comp, s4[q]);
      kahan_add(s, comp, -k4[q]);
    }
#pragma unroll
    for (int jj = 0; jj < RMAX; ++jj) {
      const int c = c0 + jj;
      if (c < c1) {
        r[jj] = mul_f2c(s, inv);
        const int out = c - half, in = c - half + win;
        if (out >= 0 && out < n) kahan_add(s, comp, -a[out]);
        if (in >= 0 && in < n) kahan_add(s, comp, a[in]);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int jj = 0; jj < RMAX; ++jj)
    if (c0 + jj < c1) a[c0 + jj] = r[jj];
  __syncthreads();
}

// The boxcar (no abs) of a row of length n for the outputs c in [lo, hi),
// window [c - half, c - half + win - 1] clipped to [0, n), from
// u[j - u0] = the row at j for every j the windows reach (u0 = max(0,
// lo - half) .. min(n, hi - half + win)); each output overwrites u[c - u0]
// once every thread has read its windows (runs of odd length held in
// registers, hi - lo <= RMAX x threads). Ends with the CTA synchronised.
template <int RMAX>
__device__ __noinline__ void boxcar_sub_inplace(float* u, int u0, int n, int win, F2c inv, int lo, int hi) {
  const int per = odd_run(hi - lo);
  const int c0 = lo + threadIdx.x * per;
  const int c1 = min(hi, c0 + per);
  float r[RMAX];
  if (c0 < hi) {
    const int half = win / 2;
    const int wlo = max(0, c0 - half), whi = min(n - 1, c0 - half + win - 1);
    float s4[4] = {0.f, 0.f, 0.f, 0.f}, k4[4] = {0.f, 0.f, 0.f, 0.f};
    int j = wlo;
    for (; j + 3 <= whi; j += 4) {
#pragma unroll
      for (int q = 0; q < 4; ++q) kahan_add(s4[q], k4[q], u[j + q - u0]);
    }
    for (; j <= whi; ++j) kahan_add(s4[0], k4[0], u[j - u0]);
    float s = 0.f, comp = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      kahan_add(s, comp, s4[q]);
      kahan_add(s, comp, -k4[q]);
    }
#pragma unroll
    for (int jj = 0; jj < RMAX; ++jj) {
      const int c = c0 + jj;
      if (c < c1) {
        r[jj] = mul_f2c(s, inv);
        const int out = c - half, in = c - half + win;
        if (out >= 0 && out < n) kahan_add(s, comp, -u[out - u0]);
        if (in >= 0 && in < n) kahan_add(s, comp, u[in - u0]);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int jj = 0; jj < RMAX; ++jj)
    if (c0 + jj < c1) u[c0 + jj - u0] = r[jj];
  __syncthreads();
}

// RAM divide of one sample (runabsNormalizeSharedWeight) by the station
// weight s, the float sum of the component weights in component order:
// s clamped to MINVAL, x / s, NaN -> 0, clip to +-MAXVAL.
__device__ __forceinline__ float ram_divide_s(float x, float s) {
  if (!isfinite(s) || s < kMinValF) s = kMinValF;
  // (double)s < MINVAL in double is s < (float)MINVAL for a float s (no
  // float lies in [1e-30, (float)1e-30)), and never true after the clamp
  float y = (s < kMinValF) ? 0.f : x / s;
  if (!isfinite(y)) y = 0.f;
  return fminf(fmaxf(y, -kMaxVal), kMaxVal);
}

__device__ __forceinline__ float ram_divide(float x, const float* __restrict__ w, int64_t row0,
                                            int64_t pitch, int num_ch, int i) {
  float s = 0.f;
  for (int c = 0; c < num_ch; ++c) s += w[(row0 + c) * pitch + i];
  return ram_divide_s(x, s);
}

// Bins in flight per thread in the pointwise passes: the digit-reversal
// table and the row reads of kPw bins are issued before any of them is
// used, so their latencies overlap (one CTA per SM leaves no other CTA to
// hide them).
constexpr int kPw = 4;

// store(i, load(i)) for i in [0, n), each thread over i = tid, tid + T, ...
// in that order, with the loads of U consecutive items of a thread issued
// before the first store (global-memory latency overlapped U ways).
template <int U, typename Ld, typename St>
__device__ __forceinline__ void batched_rows(int n, Ld load, St store) {
  for (int i0 = threadIdx.x; i0 < n; i0 += U * kS2sT) {
    decltype(load(0)) v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) v[u] = load(min(i0 + u * kS2sT, n - 1));
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (i0 + u * kS2sT < n) store(i0 + u * kS2sT, v[u]);
  }
}

// Real-transform twiddle w_{2M}^k (k <= M) from the shared-memory copy of a
// real plan's table (tw_stride 2: the table is of the real length 2M).
__device__ __forceinline__ float2 real_tw(const float2* stw, int k, int M) {
  return k == M ? make_float2(-1.f, 0.f) : tw_lookup(stw, k);
}

// Forward post-processing (r2c_post) of the loaded pair za = Z[k],
// zb = Z[M-k] (Z[M] == Z[0]).
__device__ __forceinline__ float2 r2c_post_vals(float2 za, float2 zb, int k, int M, const float2* stw) {
  const float2 zc = conjf2(zb);
  const float2 xe = make_float2(0.5f * (za.x + zc.x), 0.5f * (za.y + zc.y));
  const float2 d = make_float2(0.5f * (za.x - zc.x), 0.5f * (za.y - zc.y));
  return cadd(xe, cmul(real_tw(stw, k, M), mul_mi(d)));
}

// g(k, X[k]) for the bins k in [0, kend) (kend <= M + 1) of the real
// forward transform whose length-M complex FFT Z sits digit-reversed in buf.
template <typename G>
__device__ __forceinline__ void r2c_post_bins(const float2* buf, const FftPlan& p, const float2* stw, int kend,
                                              G g) {
  const int M = p.n;
  for (int k0 = threadIdx.x; k0 < kend; k0 += kPw * kS2sT) {
    int pa[kPw], pb[kPw];
#pragma unroll
    for (int u = 0; u < kPw; ++u) {
      const int k = min(k0 + u * kS2sT, kend - 1);
      pa[u] = __ldg(p.perm + (k == M ? 0 : k));
      pb[u] = __ldg(p.perm + (k == 0 ? 0 : M - k));
    }
    float2 za[kPw], zb[kPw];
#pragma unroll
    for (int u = 0; u < kPw; ++u) {
      za[u] = buf[pa[u]];
      zb[u] = buf[pb[u]];
    }
#pragma unroll
    for (int u = 0; u < kPw; ++u) {
      const int k = k0 + u * kS2sT;
      if (k < kend) g(k, r2c_post_vals(za[u], zb[u], k, M, stw));
    }
  }
}

// Pointwise pass of a real round trip: Z is the DIF output of the length-M
// complex FFT of a real row of length 2M. For every bin pair (k, M-k) the
// thread forms the real-spectrum bins X[k], X[M-k] (X[M] for k = 0), maps
// them through f(k, X, pre(k)) and writes back the pre-processed inverse
// input Z' at the same digit-reversed points, ready for fft_dit(inverse).
// pre(k) is a per-bin value (a table entry, a weight) loaded with the
// batch's other reads. Each pair owns its two points, so a thread may read
// kPw pairs before writing any.
template <typename Pre, typename F>
__device__ __forceinline__ void real_roundtrip_pointwise_pre(float2* buf, const FftPlan& p, const float2* stw,
                                                             Pre pre, F f) {
  const int M = p.n;
  const int H = M / 2;
  for (int k0 = threadIdx.x; k0 <= H; k0 += kPw * kS2sT) {
    int pk[kPw], pk2[kPw];
    decltype(pre(0)) va[kPw], vb[kPw];
#pragma unroll
    for (int u = 0; u < kPw; ++u) {
      const int k = min(k0 + u * kS2sT, H);
      pk[u] = __ldg(p.perm + k);
      pk2[u] = __ldg(p.perm + (k == 0 ? 0 : M - k));  // k == 0: X[M] comes from Z[0] too
      va[u] = pre(k);
      vb[u] = pre(M - k);
    }
    float2 zk[kPw], zk2[kPw];
#pragma unroll
    for (int u = 0; u < kPw; ++u) {
      zk[u] = buf[pk[u]];
      zk2[u] = buf[pk2[u]];
    }
#pragma unroll
    for (int u = 0; u < kPw; ++u) {
      const int k = k0 + u * kS2sT;
      if (k > H) continue;
      const int k2 = M - k;  // == M for k == 0
      float2 Xk = r2c_post_vals(zk[u], zk2[u], k, M, stw);
      float2 Xk2 = (k == 0) ? r2c_post_vals(zk[u], zk[u], M, M, stw) : r2c_post_vals(zk2[u], zk[u], k2, M, stw);
      Xk = f(k, Xk, va[u]);
      Xk2 = f(k2, Xk2, vb[u]);
      if (k == 0) {
        // Z'[0] from Y[0], Y[M] (imaginary parts of DC / Nyquist ignored)
        buf[pk[u]] = c2r_pre_w(make_float2(Xk.x, 0.f), make_float2(Xk2.x, 0.f), real_tw(stw, 0, M));
      } else if (k == k2) {
        buf[pk[u]] = c2r_pre_w(Xk, Xk, real_tw(stw, k, M));
      } else {
        buf[pk[u]] = c2r_pre_w(Xk, Xk2, real_tw(stw, k, M));
        buf[pk2[u]] = c2r_pre_w(Xk2, Xk, real_tw(stw, k2, M));
      }
    }
  }
}

// The prefilter's pointwise map (x dt, sanitize, x |H|^2), |H|^2 from resp.
__device__ __forceinline__ void prefilter_pointwise(float2* buf, const FftPlan& p, const float2* stw, float dt,
                                                    const float* __restrict__ resp) {
  real_roundtrip_pointwise_pre(
      buf, p, stw, [&](int k) { return __ldg(resp + k); },
      [&](int, float2 X, float h) {
        X = sanitize2(make_float2(X.x * dt, X.y * dt));
        return make_float2(X.x * h, X.y * h);
      });
}

// InvNormalize2DKernel weight: 1 / (width * dt) with width*dt in float.
__host__ __device__ inline double inv_norm(int n, float dt) { return 1.0 / (double)((float)n * dt); }

// Row buffer of a transform CTA: shared memory, or -- for rows longer than
// shared memory holds (20 Hz data: 72 000-sample windows) -- this CTA's
// slice of an L2-resident global scratch (grows != null). The stage code is
// the same; __syncthreads orders the global accesses within the CTA. The
// twiddle table and small arrays stay in shared memory (from smraw on).
struct RowBuf {
  float2* grows;
  int64_t gelems;
};
__device__ __forceinline__ float2* row_buffer(float2* smraw, const RowBuf& rb) {
  return rb.grows ? rb.grows + (int64_t)blockIdx.x * rb.gelems : smraw;
}
__device__ __forceinline__ float2* after_row(float2* smraw, const RowBuf& rb, int row_elems) {
  return rb.grows ? smraw : smraw + row_elems;
}

// ---------------------------------------------------------------------------
// k_s2s_front: window load, preprocess, prefilter, one-bit / RAM weight
// ---------------------------------------------------------------------------

// Window load, NaN/Inf -> 0 (isnan2DKernel), demean (rdc2DKernel), detrend
// (rtr2DKernel), Hann end taper (timetaper2DKernel) and the prefilter round
// trip (R2C(filter_nfft), x dt, sanitize, x |H|^2, C2R) of one row: on
// return xs[0, seg) holds the unnormalised inverse (the caller applies
// 1 / (filter_nfft dt)); stw holds the prefilter plan's twiddles. Samples
// past the series are zero.
__device__ __forceinline__ void s2s_front_row(float2* sbuf, float2* stw, const float* __restrict__ src,
                                              int64_t start, int64_t series_len, const S2sDev& d,
                                              const FftPlan& pf, const float* __restrict__ resp) {
  __shared__ double sred[64];
  float* xs = reinterpret_cast<float*>(sbuf);
  const int Mf = pf.n;
  const int seg = d.seg;
  fft_twiddles_to_smem<kS2sT>(pf, stw);
  Kahan s1;
  batched_rows<8>(
      seg, [&](int i) { return start + i < series_len ? src[i] : 0.f; },
      [&](int i, float v) {
        if (!isfinite(v)) v = 0.f;
        xs[i] = v;
        s1.add(v);
      });
  for (int i = seg + threadIdx.x; i < 2 * Mf; i += kS2sT) xs[i] = 0.f;
  // demean: x -= sum/width
  __shared__ float srow[4];
  {
    const float hi[1] = {s1.s}, lo[1] = {-s1.c};
    double t[1];
    block_sums_t0<1>(hi, lo, sred, t);
    if (threadIdx.x == 0) {
      const F2c m = f2c(t[0] / (double)seg);
      srow[0] = m.hi;
      srow[1] = m.lo;
    }
    __syncthreads();
  }
  const F2c mean{srow[0], srow[1]};
  Kahan s2, si;
  for (int i = threadIdx.x; i < seg; i += kS2sT) {
    const float v = (xs[i] - mean.hi) - mean.lo;
    xs[i] = v;
    s2.add(v);
    si.add(v * (float)i);
  }
  // detrend: closed-form least squares (slope ca, intercept cb)
  {
    const float hi[2] = {s2.s, si.s}, lo[2] = {-s2.c, -si.c};
    double t[2];
    block_sums_t0<2>(hi, lo, sred, t);
    if (threadIdx.x == 0) {
      const double y2 = t[0], y1 = t[1];
      srow[2] = (float)((d.a22 * y1 - d.a12 * y2) * d.inv_det);
      srow[3] = (float)((d.a11 * y2 - d.a12 * y1) * d.inv_det);
    }
    __syncthreads();
  }
  const int tap = d.taper;
  const float caf = srow[2], cbf = srow[3], itap = 1.0f / (float)tap;
  for (int i = threadIdx.x; i < seg; i += kS2sT) {
    const float v = xs[i] - fmaf(caf, (float)i, cbf);
    // 0.5 (1 - cos(pi i / tap)) at both ends
    float fac = 1.0f;
    if (i < tap)
      fac = 0.5f * (1.0f - cospif((float)i * itap));
    else if (i >= seg - tap)
      fac = 0.5f * (1.0f - cospif((float)(seg - i) * itap));
    xs[i] = v * fac;
  }
  __syncthreads();
  fft_dif_nl<kS2sT>(sbuf, pf, stw, false);
  const float dt = d.delta;
  prefilter_pointwise(sbuf, pf, stw, dt, resp);
  __syncthreads();
  fft_dit_nl<kS2sT>(sbuf, pf, stw, true);
}

__global__ void __launch_bounds__(kS2sT, 1)
    k_s2s_front(const float* __restrict__ series, int64_t series_pitch, int64_t series_len,
                const int* __restrict__ steps, S2sDev d, FftPlan pf, const float* __restrict__ resp, int mode,
                int raw_win, float* __restrict__ xout, float* __restrict__ wout, RowBuf rb) {
  // mode: 0 = write x only, 1 = one-bit, 2 = x and smoothed |x| weight
  extern __shared__ float2 smraw[];
  const int Mf = pf.n;
  float2* sbuf = row_buffer(smraw, rb);
  float2* stw = after_row(smraw, rb, Mf);
  float* xs = reinterpret_cast<float*>(sbuf);
  const int r = blockIdx.x;
  const int sidx = r / d.nrows, row = r % d.nrows;
  const int64_t start = (int64_t)steps[sidx] * d.shift;
  const int seg = d.seg;
  s2s_front_row(sbuf, stw, series + (int64_t)row * series_pitch + start, start, series_len, d, pf, resp);
  const F2c inrm = d.inrm_f;
  float* xo = xout + (int64_t)r * seg;
  for (int i = threadIdx.x; i < seg; i += kS2sT) {
    float v = mul_f2c(xs[i], inrm);
    if (mode == 1) v = (v > 0.f) ? 1.f : ((v < 0.f) ? -1.f : 0.f);
    xs[i] = v;
    xo[i] = v;
  }
  if (mode == 2) {
    __syncthreads();
    float* wo = wout + (int64_t)r * seg;
    boxcar_range<true>(xs, seg, raw_win, d.inv_rw, 0, seg, wo);
  }
}

// ---------------------------------------------------------------------------
// RUN-ABS-MF: per band filter + weight, then the sum of normalised bands
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kS2sT, 1)
    k_s2s_mfband(const float* __restrict__ xin, S2sDev d, FftPlan pf, const float* __restrict__ resp, int raw_win,
                 F2c inv_win, float* __restrict__ xb,
                 float* __restrict__ wb, RowBuf rb) {
  extern __shared__ float2 smraw[];
  const int Mf = pf.n;
  float2* sbuf = row_buffer(smraw, rb);
  float2* stw = after_row(smraw, rb, Mf);
  float* xs = reinterpret_cast<float*>(sbuf);
  const int r = blockIdx.x;
  const int seg = d.seg;
  fft_twiddles_to_smem<kS2sT>(pf, stw);
  const float* xi = xin + (int64_t)r * seg;
  batched_rows<8>(seg, [&](int i) { return xi[i]; }, [&](int i, float v) { xs[i] = v; });
  for (int i = seg + threadIdx.x; i < 2 * Mf; i += kS2sT) xs[i] = 0.f;
  __syncthreads();
  fft_dif_nl<kS2sT>(sbuf, pf, stw, false);
  const float dt = d.delta;
  prefilter_pointwise(sbuf, pf, stw, dt, resp);
  __syncthreads();
  fft_dit_nl<kS2sT>(sbuf, pf, stw, true);
  const F2c inrm = d.inrm_f;
  float* xo = xb + (int64_t)r * seg;
  for (int i = threadIdx.x; i < seg; i += kS2sT) {
    const float v = mul_f2c(xs[i], inrm);
    xs[i] = v;
    xo[i] = v;
  }
  __syncthreads();
  float* wo = wb + (int64_t)r * seg;
  boxcar_range<true>(xs, seg, raw_win, inv_win, 0, seg, wo);
}

__global__ void k_s2s_mfsum(const float* __restrict__ xb, const float* __restrict__ wb, int nbands,
                            int64_t band_stride, S2sDev d, float* __restrict__ xout) {
  const int r = blockIdx.y;
  const int row = r % d.nrows;
  const int64_t row0 = (int64_t)(r - row) + (row / d.num_ch) * d.num_ch;  // first row of the station
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.seg; i += gridDim.x * blockDim.x) {
    float acc = 0.f;
    for (int b = 0; b < nbands; ++b) {
      const float* xbb = xb + b * band_stride;
      const float* wbb = wb + b * band_stride;
      acc += ram_divide(xbb[(int64_t)r * d.seg + i], wbb, row0, d.seg, d.num_ch, i);
    }
    xout[(int64_t)r * d.seg + i] = acc;
  }
}

// ---------------------------------------------------------------------------
// Whitening phase A: [RAM divide] R2C(seg), x dt, sanitize, smoothed |X|
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kS2sT, 1)
    k_s2s_whiten_a(const float* __restrict__ xin, const float* __restrict__ win_w, S2sDev d,
                   FftPlan ps, const float2* __restrict__ tws, int ww, float2* __restrict__ Xout,
                   float* __restrict__ Aout, int64_t fpitch, RowBuf rb) {
  extern __shared__ float2 smraw[];
  const int Ms = ps.n;
  float2* sbuf = row_buffer(smraw, rb);
  float2* stw = after_row(smraw, rb, Ms);
  float* amp = reinterpret_cast<float*>(stw + fft_tw_smem_elems(ps));
  float* xs = reinterpret_cast<float*>(sbuf);
  const int r = blockIdx.x;
  const int row = r % d.nrows;
  const int64_t row0 = (int64_t)(r - row) + (row / d.num_ch) * d.num_ch;
  const int seg = d.seg;
  fft_twiddles_to_smem<kS2sT>(ps, stw);
  const float* xi = xin + (int64_t)r * seg;
  batched_rows<4>(
      seg, [&](int i) { return win_w ? ram_divide(xi[i], win_w, row0, seg, d.num_ch, i) : xi[i]; },
      [&](int i, float v) { xs[i] = v; });
  __syncthreads();
  fft_dif_nl<kS2sT>(sbuf, ps, stw, false);
  const int fw = Ms + 1;
  const float dt = d.delta;
  float2* Xo = Xout + (int64_t)r * fpitch;
  r2c_post_bins(sbuf, ps, stw, fw, [&](int k, float2 X) {
    X = sanitize2(make_float2(X.x * dt, X.y * dt));
    Xo[k] = X;
    amp[k] = hypotf(X.x, X.y);
  });
  __syncthreads();
  float* Ao = Aout + (int64_t)r * fpitch;
  if (fw <= kRunRegs * kS2sT) {
    // smoothed in place, then stored coalesced
    boxcar_inplace<kRunRegs>(amp, fw, ww, d.inv_ww);
    for (int k = threadIdx.x; k < fw; k += kS2sT) Ao[k] = amp[k];
  } else {
    boxcar_range<false>(amp, fw, ww, d.inv_ww, 0, fw, Ao);
  }
}

// ---------------------------------------------------------------------------
// Whitening phase B (+ output transform, or back to the time row)
// ---------------------------------------------------------------------------

__device__ __forceinline__ float spec_taper_factor(int col, int width, const S2sDev& d) {
  // specTaper2DKernel, np = 1: cosine ramps up over [i1, i2), down over
  // [i3, i4)
  const int i1 = d.f_idx1, i2 = d.f_idx2, i3 = d.f_idx3;
  const int i4 = d.f_idx4 < width ? d.f_idx4 : width;
  if (col < i1) return 0.f;
  if (col >= i1 && col < i2) return 0.5f * (1.0f - cospif((float)(col - i1) / (float)(i2 - i1)));
  if (col >= i3 && col < i4) return 0.5f * (1.0f + cospif((float)(col - i3) / (float)(i4 - i3)));
  if (col >= i4 && col < width) return 0.f;
  return 1.f;
}

// One whitened bin (cdiv2DKernel after clampmin2DKernel, then the band
// taper and sanitize): X / s for the station weight s (the float sum of the
// components' smoothed amplitudes, clamped to MINVAL), times the taper.
__device__ __forceinline__ float2 whiten_bin(float2 X, float s, int k, int width, const S2sDev& d) {
  if (!isfinite(s) || s < kMinValF) s = kMinValF;  // clampmin2DKernel
  // cdiv2DKernel's double compare against MINVAL, as in ram_divide
  if (s < kMinValF) X = make_float2(0.f, 0.f);
  else X = make_float2(X.x / s, X.y / s);
  // (float)((double)x * f) of two floats is the correctly rounded float
  // product: the double product is exact
  const float f = spec_taper_factor(k, width, d);
  X = make_float2(X.x * f, X.y * f);
  return sanitize2(X);
}

__device__ __forceinline__ void output_transform(float2* sbuf, float* xs, int nvalid,
                                                 const FftPlan& po, const float2* twp,
                                                 float2* stw, const S2sDev& d,
                                                 float2* __restrict__ out) {
  // zero-pad to output_nfft, R2C x dt, sanitize, optional phase-only
  const int Mo = po.n;
  for (int i = nvalid + threadIdx.x; i < 2 * Mo; i += kS2sT) xs[i] = 0.f;
  __syncthreads();
  fft_twiddles_to_smem<kS2sT>(po, stw);
  __syncthreads();
  fft_dif_nl<kS2sT>(sbuf, po, stw, false);
  const float dt = d.delta;
  r2c_post_bins(sbuf, po, stw, d.nspec, [&](int k, float2 X) {
    X = sanitize2(make_float2(X.x * dt, X.y * dt));
    if (d.phase_only) {
      // spectralOnebit2DKernel (hypotf, amp <= MINVAL -> 0), then sanitize
      const float a = hypotf(X.x, X.y);
      if (!isfinite(a) || a <= kMinValF)
        X = make_float2(0.f, 0.f);
      else {
        const float ia = 1.0f / a;
        X = sanitize2(make_float2(X.x * ia, X.y * ia));
      }
    }
    out[k] = X;
  });
}

__global__ void __launch_bounds__(kS2sT, 1)
    k_s2s_whiten_b(const float2* __restrict__ Xin, const float* __restrict__ Ain, int64_t fpitch,
                   S2sDev d, FftPlan ps, const float2* __restrict__ tws, FftPlan po,
                   const float2* __restrict__ two, int to_time, int time_mode, int raw_win,
                   float* __restrict__ xout, float* __restrict__ wout, float2* __restrict__ out,
                   int64_t out_pitch, RowBuf rb) {
  extern __shared__ float2 smraw[];
  const int Mbuf = max(ps.n, po.n);
  float2* sbuf = row_buffer(smraw, rb);
  float2* stw = after_row(smraw, rb, Mbuf);
  float* xs = reinterpret_cast<float*>(sbuf);
  const int r = blockIdx.x;
  const int row = r % d.nrows;
  const int64_t row0 = (int64_t)(r - row) + (row / d.num_ch) * d.num_ch;
  const int Ms = ps.n;
  const int fw = Ms + 1;
  fft_twiddles_to_smem<kS2sT>(ps, stw);
  const float2* Xr = Xin + (int64_t)r * fpitch;
  // whitened, tapered, sanitised bins written as the C2R pre-processed input
  // at the digit-reversed points of the length-Ms transform; the reads of
  // kPw bin pairs are issued before any is used
  auto wsum = [&](int k) {
    float s = 0.f;
    for (int c = 0; c < d.num_ch; ++c) s += Ain[(row0 + c) * fpitch + k];
    return s;
  };
  for (int k0 = threadIdx.x; k0 < Ms; k0 += kPw * kS2sT) {
    int pos[kPw];
    float2 xa[kPw], xb[kPw];
    float sa[kPw], sb[kPw];
#pragma unroll
    for (int u = 0; u < kPw; ++u) {
      const int k = min(k0 + u * kS2sT, Ms - 1);
      pos[u] = __ldg(ps.perm + k);
      xa[u] = Xr[k];
      xb[u] = Xr[Ms - k];
      sa[u] = wsum(k);
      sb[u] = wsum(Ms - k);
    }
#pragma unroll
    for (int u = 0; u < kPw; ++u) {
      const int k = k0 + u * kS2sT;
      if (k >= Ms) continue;
      float2 a = whiten_bin(xa[u], sa[u], k, fw, d);
      float2 b = whiten_bin(xb[u], sb[u], Ms - k, fw, d);
      if (k == 0) {
        a.y = 0.f;
        b.y = 0.f;
      }
      sbuf[pos[u]] = c2r_pre_w(a, b, real_tw(stw, k, Ms));
    }
  }
  __syncthreads();
  fft_dit_nl<kS2sT>(sbuf, ps, stw, true);
  const int seg = d.seg;
  const F2c inrm = d.inrm_s;
  for (int i = threadIdx.x; i < seg; i += kS2sT) {
    float v = mul_f2c(xs[i], inrm);
    if (to_time && time_mode == 1) v = (v > 0.f) ? 1.f : ((v < 0.f) ? -1.f : 0.f);
    xs[i] = v;
  }
  __syncthreads();
  if (to_time) {
    float* xo = xout + (int64_t)r * seg;
    for (int i = threadIdx.x; i < seg; i += kS2sT) xo[i] = xs[i];
    if (time_mode == 2) {
      float* wo = wout + (int64_t)r * seg;
      boxcar_range<true>(xs, seg, raw_win, d.inv_rw, 0, seg, wo);
    }
    return;
  }
  output_transform(sbuf, xs, seg, po, two, stw, d, out + (int64_t)r * out_pitch);
}

__global__ void __launch_bounds__(kS2sT, 1)
    k_s2s_output(const float* __restrict__ xin, const float* __restrict__ win_w, S2sDev d,
                 FftPlan po, const float2* __restrict__ two, float2* __restrict__ out,
                 int64_t out_pitch, RowBuf rb) {
  extern __shared__ float2 smraw[];
  const int Mo = po.n;
  float2* sbuf = row_buffer(smraw, rb);
  float2* stw = after_row(smraw, rb, Mo);
  float* xs = reinterpret_cast<float*>(sbuf);
  const int r = blockIdx.x;
  const int row = r % d.nrows;
  const int64_t row0 = (int64_t)(r - row) + (row / d.num_ch) * d.num_ch;
  const int seg = d.seg;
  const float* xi = xin + (int64_t)r * seg;
  batched_rows<4>(
      seg, [&](int i) { return win_w ? ram_divide(xi[i], win_w, row0, seg, d.num_ch, i) : xi[i]; },
      [&](int i, float v) { xs[i] = v; });
  output_transform(sbuf, xs, seg, po, two, stw, d, out + (int64_t)r * out_pitch);
}

// ---------------------------------------------------------------------------
// k_s2s_station: the whole chain for the three components of a station
// window, one 3-CTA thread-block cluster per station window
// ---------------------------------------------------------------------------
//
// Used for three components with RAM / one-bit / no normalisation and
// whitening after normalisation (or none), when a row, the twiddles and the
// exchange buffer fit one CTA's shared memory. The components' coupling --
// the station RAM weight (the sum of the three smoothed |x|) and the
// station whitening weight (the sum of the three smoothed |X|) -- goes
// through distributed shared memory, and rows never leave shared memory
// between the window load and the spectrum store.
//
// RAM: a row of weights is more than `aux` holds next to the row, so CTA r
// forms the station weight only for its third of the samples, as the
// boxcar of |x_E| + |x_N| + |x_Z| (equal to the sum of the three smoothed
// |x|: the boxcar is linear), reading the peers' rows; every CTA then reads
// each sample's weight from the CTA that owns its third. Whitening: each
// CTA smooths its own amplitudes (seg/2 + 1 bins fit `aux` whole) and reads
// the two others' at the same bin, in component order. Smoothing runs hold
// their outputs in registers and write them back in place.
//
// Every cluster barrier below is reached unconditionally or under a
// condition uniform over the grid (the mode and plan), so the three CTAs
// always meet at the same barriers.

constexpr int kStationCtas = 3;

struct S2sFused {
  int mode;        // 0 = none, 1 = one-bit, 2 = RAM
  int whiten;      // 1: whitening after the normalisation
  int raw_win;     // RAM boxcar width
  int ww;          // whitening boxcar width
  int aux_floats;  // exchange buffer (floats): a third of the RAM row + halo, or the whitening bins
  int twmax;       // twiddle table elements (largest of the plans)
  int mbuf;        // row buffer (complex elements)
};

__global__ void __cluster_dims__(kStationCtas, 1, 1) __launch_bounds__(kS2sT, 1)
    k_s2s_station(const float* __restrict__ series, int64_t series_pitch, int64_t series_len,
                  const int* __restrict__ steps, S2sDev d, FftPlan pf, FftPlan ps, FftPlan po,
                  const float* __restrict__ resp, S2sFused fz, float2* __restrict__ out, int64_t out_pitch) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ float2 smraw[];
  float2* sbuf = smraw;
  float2* stw = smraw + fz.mbuf;
  float* aux = reinterpret_cast<float*>(stw + fz.twmax);
  float* xs = reinterpret_cast<float*>(sbuf);
  const int rank = (int)cl.block_rank();
  const float* peer[kStationCtas];
#pragma unroll
  for (int c = 0; c < kStationCtas; ++c) peer[c] = c == rank ? aux : cl.map_shared_rank(aux, c);
  const int r = blockIdx.x;
  const int sidx = r / d.nrows, row = r % d.nrows;
  const int64_t start = (int64_t)steps[sidx] * d.shift;
  const int seg = d.seg;
  const float dt = d.delta;

  // window load, preprocessing, prefilter
  s2s_front_row(sbuf, stw, series + (int64_t)row * series_pitch + start, start, series_len, d, pf, resp);
  {
    const F2c inrm = d.inrm_f;
    for (int i = threadIdx.x; i < seg; i += kS2sT) {
      float v = mul_f2c(xs[i], inrm);
      if (fz.mode == 1) v = (v > 0.f) ? 1.f : ((v < 0.f) ? -1.f : 0.f);
      xs[i] = v;
    }
    __syncthreads();
  }

  // RAM: station weight = the boxcar of |x_E| + |x_N| + |x_Z| (the sum of
  // the components' smoothed |x|: the boxcar is linear). CTA r forms it for
  // the outputs of its third of the row, from its peers' rows through
  // distributed shared memory, smoothed in place in `aux`; every CTA then
  // divides its row by the weight of the third that owns each sample.
  if (fz.mode == 2) {
    const int win = fz.raw_win, half = win / 2;
    const int L3 = (seg + kStationCtas - 1) / kStationCtas;
    const int lo = min(seg, rank * L3), hi = min(seg, lo + L3);
    const int u0 = max(0, lo - half), u1 = min(seg, hi - half + win);
    const float* px[kStationCtas];
#pragma unroll
    for (int c = 0; c < kStationCtas; ++c) px[c] = c == rank ? xs : cl.map_shared_rank(xs, c);
    cl.sync();  // every component's prefiltered row is final
    batched_rows<4>(
        max(0, u1 - u0), [&](int i) { return fabsf(px[0][u0 + i]) + fabsf(px[1][u0 + i]) + fabsf(px[2][u0 + i]); },
        [&](int i, float v) { aux[i] = v; });
    __syncthreads();
    // runs of 13 at one day of 0.1 s windows (L3 = 12 000): the shorter
    // register array keeps the loop free of spills
    if (L3 <= 13 * kS2sT)
      boxcar_sub_inplace<13>(aux, u0, seg, win, d.inv_rw, lo, hi);
    else
      boxcar_sub_inplace<kRunRegs>(aux, u0, seg, win, d.inv_rw, lo, hi);
    cl.sync();  // every third's weights are in place; no peer reads the rows any more
    const int b1 = L3, b2 = 2 * L3;
    const int s1 = max(0, b1 - half), s2 = max(0, b2 - half);  // u0 of thirds 1 and 2
    batched_rows<4>(
        seg,
        [&](int c) {
          const int q = (c >= b1) + (c >= b2);
          return peer[q][c - (q == 0 ? 0 : (q == 1 ? s1 : s2))];
        },
        [&](int c, float sw) { xs[c] = ram_divide_s(xs[c], sw); });
    cl.sync();  // every component done reading the weights
  }

  // whitening: X / (sum of the components' smoothed |X|), band taper
  if (fz.whiten) {
    fft_twiddles_to_smem<kS2sT>(ps, stw);
    __syncthreads();
    fft_dif_nl<kS2sT>(sbuf, ps, stw, false);
    const int fw = ps.n + 1;
    r2c_post_bins(sbuf, ps, stw, fw, [&](int k, float2 X) {
      X = sanitize2(make_float2(X.x * dt, X.y * dt));
      aux[k] = hypotf(X.x, X.y);
    });
    __syncthreads();
    boxcar_inplace<kRunRegs>(aux, fw, fz.ww, d.inv_ww);
    cl.sync();  // the three components' smoothed amplitudes are in place
    real_roundtrip_pointwise_pre(
        sbuf, ps, stw, [&](int k) { return peer[0][k] + peer[1][k] + peer[2][k]; },
        [&](int k, float2 X, float sw) {
          X = sanitize2(make_float2(X.x * dt, X.y * dt));
          return whiten_bin(X, sw, k, fw, d);
        });
    cl.sync();  // every component done reading the amplitudes
    fft_dit_nl<kS2sT>(sbuf, ps, stw, true);
    const F2c inrm = d.inrm_s;
    for (int i = threadIdx.x; i < seg; i += kS2sT) xs[i] = mul_f2c(xs[i], inrm);
  }
  output_transform(sbuf, xs, seg, po, nullptr, stw, d, out + (int64_t)r * out_pitch);
}

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------

// The fused chain (k_s2s_station) for this call, or FXC_ERR_UNSUPPORTED
// when it does not apply: other than three components, RUN-ABS-MF,
// whitening before the normalisation, rows or exchange buffers beyond one
// CTA's shared memory, or FXC_S2S_FUSED=0 in the environment (the kernel
// chain instead).
static int s2s_run_fused(fxc_ctx* ctx, const fxc_s2s_plan* plan, const S2sDev& d, const FftPlan& pf,
                         const FftPlan& ps, const FftPlan& po, const float* d_series, int64_t series_pitch,
                         int64_t series_len, const int32_t* h_steps, int32_t nsteps, int64_t nr, int32_t num_ch,
                         const float* d_responses, float* d_out, int64_t out_pitch) {
  const char* env = getenv("FXC_S2S_FUSED");
  if (env && env[0] == '0') return FXC_ERR_UNSUPPORTED;
  if (num_ch != kStationCtas) return FXC_ERR_UNSUPPORTED;
  S2sFused fz{};
  switch (plan->normalize) {
    case 0: fz.mode = 0; break;
    case 2: fz.mode = 1; break;
    case 3: fz.mode = 2; break;
    default: return FXC_ERR_UNSUPPORTED;
  }
  if (plan->whiten != 0 && plan->whiten != 2) return FXC_ERR_UNSUPPORTED;
  fz.whiten = plan->whiten == 2;
  fz.raw_win = std::max(plan->runabs_win, 1);
  fz.ww = std::max(plan->whiten_win, 1);
  fz.mbuf = std::max(pf.n, po.n);
  fz.twmax = std::max(fft_tw_smem_elems(pf), fft_tw_smem_elems(po));
  if (fz.whiten) {
    fz.mbuf = std::max(fz.mbuf, ps.n);
    fz.twmax = std::max(fz.twmax, fft_tw_smem_elems(ps));
  }
  cudaFuncAttributes attr;
  FXC_CUDA_TRY(cudaFuncGetAttributes(&attr, k_s2s_station));
  const int64_t budget = 227 * 1024 - (int64_t)attr.sharedSizeBytes;
  const int64_t fixed = 8 * (int64_t)fz.mbuf + 8 * (int64_t)fz.twmax;
  const int64_t aux = (budget - fixed) / 16 * 4;
  if (aux < 4) return FXC_ERR_UNSUPPORTED;
  fz.aux_floats = (int)aux;
  if (fz.whiten && (ps.n + 1 > fz.aux_floats || ps.n + 1 > kRunRegs * kS2sT)) return FXC_ERR_UNSUPPORTED;
  if (fz.mode == 2) {
    // a third of the row plus a window of halo, smoothed in registers
    const int l3 = (d.seg + kStationCtas - 1) / kStationCtas;
    if (l3 + fz.raw_win > fz.aux_floats || l3 > kRunRegs * kS2sT) return FXC_ERR_UNSUPPORTED;
  }
  const size_t smem = (size_t)(fixed + 4 * aux);
  FXC_CUDA_TRY(cudaFuncSetAttribute(k_s2s_station, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)kStationCtas);
    cfg.blockDim = dim3((unsigned)kS2sT);
    cfg.dynamicSmemBytes = smem;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_s2s_station, &cfg) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      return FXC_ERR_UNSUPPORTED;
    }
  }
  FXC_TRY(ctx->scratch4.reserve(sizeof(int) * (size_t)nsteps));
  int* d_steps = reinterpret_cast<int*>(ctx->scratch4.ptr);
  FXC_CUDA_TRY(cudaMemcpyAsync(d_steps, h_steps, sizeof(int) * nsteps, cudaMemcpyHostToDevice, ctx->stream));
  k_s2s_station<<<(unsigned)nr, kS2sT, smem, ctx->stream>>>(d_series, series_pitch, series_len, d_steps, d, pf, ps,
                                                            po, d_responses, fz, reinterpret_cast<float2*>(d_out),
                                                            out_pitch);
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

// Composite radices up to 10 for the station cluster kernel's transforms:
// at 64 registers a thread (1024 threads) the radix-12/14/15/21 butterflies
// spill, and next to 232 KB of shared memory the L1 holds little of the
// spill. Measured on 4608 rows: 7.62 ms with composites up to 21, 7.24
// (15), 7.07 (12), 7.00 ms (10). The kernel chain keeps the default plans.
constexpr int kStationMaxComposite = 10;

static int make_real_plan(int n, FftPlan* p, const float2** tw, int max_composite = -1) {
  FXC_CHECK_ARG(n % 2 == 0 && n / 2 <= 65536, "real transform length %d not supported (must be even and "
                "at most 131072)", n);
  FXC_TRY(fft_twiddles(n, tw));
  return fft_make_plan_limited(n / 2, *tw, 2, p, max_composite);
}

}  // namespace fxc

using namespace fxc;

static int64_t llround_d(double x) { return (int64_t)llround(x); }

static bool smooth2357(int v) {
  if (v < 1) return false;
  const int ps[4] = {2, 3, 5, 7};
  for (int p : ps)
    while (v > 1 && v % p == 0) v /= p;
  return v == 1;
}
static int next_smooth(int n) {
  if (n < 1) n = 1;
  while (!smooth2357(n)) ++n;
  return n;
}
static int next_even_smooth(int n) {
  int l = next_smooth(n);
  while (l % 2 != 0) l = next_smooth(l + 1);
  return l;
}
static int prev_smooth(int maxlen) {
  if (maxlen <= 1) return 0;
  for (int l = maxlen - 1; l > 0; --l)
    if (smooth2357(l)) return l;
  return 0;
}

// estimateSinglePassImpulseLength (native/sac2spec/core/filter_response.c:11-72)
static int impulse_len(const double* b, const double* a, int max_samples) {
  const double a0 = a[0];
  if (fabs(a0) < 1e-30) return max_samples;
  std::vector<double> resp((size_t)max_samples);
  double xh[5] = {0}, yh[5] = {0}, total = 0.0;
  for (int n = 0; n < max_samples; ++n) {
    for (int j = 4; j > 0; --j) {
      xh[j] = xh[j - 1];
      yh[j] = yh[j - 1];
    }
    xh[0] = (n == 0) ? 1.0 : 0.0;
    double y = 0.0;
    for (int j = 0; j < 5; ++j) y += b[j] * xh[j];
    for (int j = 1; j < 5; ++j) y -= a[j] * yh[j];
    y /= a0;
    yh[0] = y;
    resp[n] = y;
    total += y * y;
  }
  if (total <= 0.0) return 1;
  double tail = 0.0;
  for (int n = max_samples - 1; n >= 0; --n) {
    tail += resp[n] * resp[n];
    if (tail > total * 1.0e-6) return n + 1;
  }
  return 1;
}

extern "C" {

int fxc_s2s_plan_init(float sac_len, float win_len, float shift_len, float xcorr_lag, float delta,
                      const double* h_b, const double* h_a, const float* h_freq_low,
                      const float* h_freq_high, int32_t nfilters, int32_t whiten, int32_t normalize,
                      int32_t phase_only, fxc_s2s_plan* out) {
  clear_error();
  FXC_CHECK_ARG(out != nullptr, "out is null");
  FXC_CHECK_ARG(delta > 0.0f && sac_len > 0.0f && win_len > 0.0f, "invalid lengths");
  FXC_CHECK_ARG(nfilters >= 1 && h_b && h_a && h_freq_low && h_freq_high, "need >= 1 filter");
  FXC_CHECK_ARG(nfilters <= FXC_S2S_MAX_BANDS, "at most %d filters", FXC_S2S_MAX_BANDS);
  FXC_CHECK_ARG(whiten >= 0 && whiten <= 3 && normalize >= 0 && normalize <= 3,
                "whiten %d / normalize %d out of range", whiten, normalize);
  fxc_s2s_plan p;
  memset(&p, 0, sizeof(p));
  p.delta = delta;
  const double ts = (double)sac_len / (double)delta;
  FXC_CHECK_ARG(std::isfinite(ts) && ts >= 1.0 && ts <= 2147483647.0, "invalid sac_len");
  p.npts = (int32_t)llround_d(ts);
  // segment_length_from_seconds (native/sac2spec/fft_length.c:90-108)
  int req = 0;
  {
    const double s = (double)win_len / (double)delta;
    req = (!std::isfinite(s) || s > 2147483647.0) ? 2147483647 : (int)llround_d(s);
  }
  int seg = next_smooth(req);
  if (seg > p.npts) seg = prev_smooth(p.npts);
  FXC_CHECK_ARG(seg > 0, "no 2-3-5-7-smooth segment length below %d", p.npts);
  p.segment_pts = seg;
  int shift = (int)llround_d((double)shift_len / (double)delta);
  if (shift < 1) shift = seg;
  p.shift_pts = shift;
  p.nstep = (seg <= p.npts) ? std::max((p.npts - seg) / shift + 1, 1) : 1;
  const int max_out = seg * 2;
  int keep = (int)llround_d((double)xcorr_lag / (double)delta);
  if (keep > seg) keep = seg;
  p.output_nfft = std::min(next_even_smooth(seg + keep), max_out);
  p.nspec = p.output_nfft / 2 + 1;
  const float seg_df = 1.0f / ((float)seg * delta);
  p.freq_low = h_freq_low[0];
  p.freq_high = h_freq_high[0];
  FXC_CHECK_ARG(p.freq_low > 0.0f && p.freq_high > p.freq_low, "invalid broad band");
  p.f_idx1 = (int32_t)(p.freq_low * 0.667f / seg_df);
  p.f_idx2 = (int32_t)(p.freq_low / seg_df);
  p.f_idx3 = (int32_t)(p.freq_high / seg_df);
  p.f_idx4 = (int32_t)(p.freq_high * 1.333f / seg_df);
  int maxi = 1;
  for (int i = 0; i < nfilters; ++i) maxi = std::max(maxi, impulse_len(h_b + 5 * i, h_a + 5 * i, seg));
  int pad = std::min(std::max(2 * maxi, 1), seg);
  p.filter_padding = pad;
  p.filter_nfft = std::min(next_even_smooth(seg + pad), max_out);
  p.taper_pts = (int32_t)(2.0f * (1.0f / p.freq_low) / delta);
  {
    const float fl = p.freq_low * 0.667f;
    int w = 2 * (int)(1.0 / (double)(fl * delta)) + 1;
    p.runabs_win = w < 1 ? 1 : w;
  }
  {
    int w = (int)(0.02 * (double)seg * (double)delta);
    p.whiten_win = w < 1 ? 1 : w;
  }
  p.whiten = whiten;
  p.normalize = normalize;
  p.phase_only = phase_only;
  p.nfilters = nfilters;
  for (int i = 0; i < nfilters; ++i) p.band_freq_low[i] = h_freq_low[i];
  *out = p;
  return FXC_OK;
}

int fxc_s2s_filter_response(const fxc_s2s_plan* plan, const double* h_b, const double* h_a,
                            int32_t nfilters, float* h_out) {
  clear_error();
  FXC_CHECK_ARG(plan && h_b && h_a && h_out && nfilters >= 1, "null argument");
  const int nfft = plan->filter_nfft;
  const int half = nfft / 2;
  const double pi = 3.14159265358979323846;
  for (int f = 0; f < nfilters; ++f) {
    const double* b = h_b + 5 * f;
    const double* a = h_a + 5 * f;
    float* o = h_out + (size_t)f * (half + 1);
    // calFilterPowerResp (native/sac2spec/core/filter_response.c:186-233)
    for (int i = 0; i < half + 1; ++i) {
      const double nf = (double)i / (double)half;
      double Bx = 0, By = 0, Ax = 0, Ay = 0;
      for (int j = 0; j < 5; ++j) {
        const double ang = -1.0 * pi * nf * (double)j;
        const double c = cos(ang), s = sin(ang);
        Bx += b[j] * c;
        By += b[j] * s;
        Ax += a[j] * c;
        Ay += a[j] * s;
      }
      const double num = Bx * Bx + By * By, den = Ax * Ax + Ay * Ay;
      double rp = (den <= 2.2250738585072014e-308) ? 0.0 : (num / den);
      if (!std::isfinite(rp)) rp = 0.0;
      else if (rp > 3.402823466e38) rp = 3.402823466e38;
      o[i] = (float)rp;
    }
  }
  return FXC_OK;
}

int fxc_s2s_run(fxc_ctx* ctx, const fxc_s2s_plan* plan, const float* d_series, int64_t series_pitch,
                int64_t series_len, int32_t nrows, int32_t num_ch, const int32_t* h_steps,
                int32_t nsteps, const float* d_responses, float* d_out, int64_t out_pitch) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(plan && d_series && h_steps && d_responses && d_out, "null argument");
  FXC_CHECK_ARG(nrows > 0 && num_ch > 0 && nrows % num_ch == 0, "nrows %d must be a multiple of "
                "num_ch %d", nrows, num_ch);
  FXC_CHECK_ARG(nsteps > 0, "no steps");
  FXC_CHECK_ARG(out_pitch >= plan->nspec, "out_pitch < nspec");
  const int seg = plan->segment_pts;
  const bool wh_before = plan->whiten == 1 || plan->whiten == 3;
  const bool wh_after = plan->whiten == 2 || plan->whiten == 3;
  if (wh_before || wh_after) FXC_CHECK_ARG(seg % 2 == 0, "whitening needs an even segment length (got %d)", seg);
  for (int i = 0; i < nsteps; ++i)
    FXC_CHECK_ARG(h_steps[i] >= 0 && h_steps[i] < plan->nstep, "step %d out of range", h_steps[i]);
  const int64_t nr = (int64_t)nsteps * nrows;
  FXC_CHECK_ARG(nr <= 0x7fffffff, "too many rows");

  FftPlan pf, ps, po;
  const float2 *twf = nullptr, *tws = nullptr, *two = nullptr;
  FXC_TRY(make_real_plan(plan->filter_nfft, &pf, &twf));
  FXC_TRY(make_real_plan(plan->output_nfft, &po, &two));
  if (wh_before || wh_after) FXC_TRY(make_real_plan(seg, &ps, &tws));

  S2sDev d;
  d.delta = plan->delta;
  d.seg = seg;
  d.shift = plan->shift_pts;
  d.filter_nfft = plan->filter_nfft;
  d.out_nfft = plan->output_nfft;
  d.nspec = plan->nspec;
  d.taper = plan->taper_pts;
  d.f_idx1 = plan->f_idx1;
  d.f_idx2 = plan->f_idx2;
  d.f_idx3 = plan->f_idx3;
  d.f_idx4 = plan->f_idx4;
  d.phase_only = plan->phase_only;
  d.num_ch = num_ch;
  d.nrows = nrows;
  d.inrm_f = f2c(inv_norm(plan->filter_nfft, plan->delta));
  d.inrm_s = f2c(inv_norm(seg, plan->delta));
  d.inv_rw = f2c(1.0 / (double)std::max(plan->runabs_win, 1));
  d.inv_ww = f2c(1.0 / (double)std::max(plan->whiten_win, 1));
  d.a12 = 0.5 * seg * (seg - 1.0);
  d.a11 = d.a12 * (2.0 * seg - 1.0) / 3.0;
  d.a22 = seg;
  d.inv_det = 1.0 / (d.a11 * d.a22 - d.a12 * d.a12);

  // one 3-CTA cluster per station window where the plan allows it
  {
    FftPlan qf, qs{}, qo;
    const float2* tw_unused = nullptr;
    FXC_TRY(make_real_plan(plan->filter_nfft, &qf, &tw_unused, kStationMaxComposite));
    FXC_TRY(make_real_plan(plan->output_nfft, &qo, &tw_unused, kStationMaxComposite));
    if (wh_before || wh_after) FXC_TRY(make_real_plan(seg, &qs, &tw_unused, kStationMaxComposite));
    int rc = s2s_run_fused(ctx, plan, d, qf, qs, qo, d_series, series_pitch, series_len, h_steps, nsteps, nr,
                           num_ch, d_responses, d_out, out_pitch);
    if (rc != FXC_ERR_UNSUPPORTED) return rc;
    clear_error();
  }

  const int nbands = plan->normalize == 1 ? plan->nfilters - 1 : 0;
  const int64_t fpitch = (int64_t)(seg / 2 + 1 + 3) / 4 * 4;
  const size_t xbytes = sizeof(float) * (size_t)nr * seg;
  const size_t a256 = 256;
  auto al = [&](size_t x) { return (x + a256 - 1) / a256 * a256; };
  size_t off = 0;
  const size_t o_steps = off;
  off = al(off + sizeof(int) * nsteps);
  const size_t o_x = off;
  off = al(off + xbytes);
  const size_t o_w = off;
  off = al(off + xbytes);
  const size_t o_X = off;
  off = al(off + ((wh_before || wh_after) ? sizeof(float2) * (size_t)nr * fpitch : 0));
  const size_t o_A = off;
  off = al(off + ((wh_before || wh_after) ? sizeof(float) * (size_t)nr * fpitch : 0));
  const size_t o_xb = off;
  off = al(off + (size_t)nbands * xbytes);
  const size_t o_wb = off;
  off = al(off + (size_t)nbands * xbytes);
  FXC_TRY(ctx->scratch4.reserve(off));
  char* base = reinterpret_cast<char*>(ctx->scratch4.ptr);
  int* d_steps = reinterpret_cast<int*>(base + o_steps);
  float* x = reinterpret_cast<float*>(base + o_x);
  float* w = reinterpret_cast<float*>(base + o_w);
  float2* X = reinterpret_cast<float2*>(base + o_X);
  float* A = reinterpret_cast<float*>(base + o_A);
  float* xb = reinterpret_cast<float*>(base + o_xb);
  float* wb = reinterpret_cast<float*>(base + o_wb);
  FXC_CUDA_TRY(cudaMemcpyAsync(d_steps, h_steps, sizeof(int) * nsteps, cudaMemcpyHostToDevice,
                               ctx->stream));
  const size_t rpitch = (size_t)plan->filter_nfft / 2 + 1;
  const float* resp0 = d_responses;

  // shared memory of each transform kernel: [row buffer] + twiddles (+ the
  // whitening amplitude row); a kernel whose total exceeds one CTA's shared
  // memory keeps its row buffer in the L2-resident global scratch instead
  const int Mbuf = (wh_before || wh_after) ? std::max(ps.n, po.n) : po.n;
  const size_t twf_b = sizeof(float2) * fft_tw_smem_elems(pf), two_b = sizeof(float2) * fft_tw_smem_elems(po);
  const size_t tws_b = (wh_before || wh_after) ? sizeof(float2) * fft_tw_smem_elems(ps) : 0;
  const size_t amp_b = (wh_before || wh_after) ? sizeof(float) * (size_t)(ps.n + 1) : 0;
  const size_t kSmemMax = 227 * 1024;
  struct Sm {
    size_t row, rest;
    bool global() const { return row + rest > 227 * 1024; }
    size_t bytes() const { return global() ? rest : row + rest; }
  };
  const Sm smf_{sizeof(float2) * (size_t)pf.n, twf_b};
  const Sm smo_{sizeof(float2) * (size_t)po.n, two_b};
  const Sm smb_{sizeof(float2) * (size_t)Mbuf, std::max(two_b, tws_b)};
  const Sm sma_{sizeof(float2) * (size_t)((wh_before || wh_after) ? ps.n : 0), tws_b + amp_b};
  FXC_CHECK_ARG(smf_.rest <= kSmemMax && smo_.rest <= kSmemMax && smb_.rest <= kSmemMax && sma_.rest <= kSmemMax,
                "transform tables too large for one CTA's shared memory");
  int64_t gelems = 0;
  for (const Sm* k : {&smf_, &smo_, &smb_, &sma_})
    if (k->global()) gelems = std::max<int64_t>(gelems, (int64_t)(k->row / sizeof(float2)));
  float2* grows = nullptr;
  if (gelems > 0) {
    gelems = (gelems + 31) / 32 * 32;
    FXC_TRY(ctx->scratch.reserve(sizeof(float2) * (size_t)nr * (size_t)gelems));
    grows = reinterpret_cast<float2*>(ctx->scratch.ptr);
  }
  auto rb_of = [&](const Sm& k) { return RowBuf{k.global() ? grows : nullptr, gelems}; };
  const size_t smf = smf_.bytes(), smo = smo_.bytes(), smb = smb_.bytes(), sma = sma_.bytes();

  // front: preprocess + prefilter (+ one-bit / RAM weight unless whitening comes first)
  int mode = 0;
  if (!wh_before) {
    if (plan->normalize == 2) mode = 1;
    if (plan->normalize == 3) mode = 2;
  }
  FXC_TRY(set_smem_limit(k_s2s_front, smf));
  k_s2s_front<<<(unsigned)nr, kS2sT, smf, ctx->stream>>>(d_series, series_pitch, series_len,
                                                         d_steps, d, pf, resp0, mode,
                                                         plan->runabs_win, x, w, rb_of(smf_));
  count_launch();
  FXC_LAUNCH_CHECK();
  const float* wgt = (mode == 2) ? w : nullptr;

  if (wh_before) {
    FXC_TRY(set_smem_limit(k_s2s_whiten_a, sma));
    k_s2s_whiten_a<<<(unsigned)nr, kS2sT, sma, ctx->stream>>>(x, nullptr, d, ps, tws,
                                                              plan->whiten_win, X, A, fpitch, rb_of(sma_));
    count_launch();
    FXC_LAUNCH_CHECK();
    int tmode = 0;
    if (plan->normalize == 2) tmode = 1;
    if (plan->normalize == 3) tmode = 2;
    FXC_TRY(set_smem_limit(k_s2s_whiten_b, smb));
    k_s2s_whiten_b<<<(unsigned)nr, kS2sT, smb, ctx->stream>>>(X, A, fpitch, d, ps, tws, po, two, 1,
                                                              tmode, plan->runabs_win, x, w,
                                                              nullptr, 0, rb_of(smb_));
    count_launch();
    FXC_LAUNCH_CHECK();
    wgt = (tmode == 2) ? w : nullptr;
  }

  if (plan->normalize == 1 && nbands > 0) {
    // RUN-ABS-MF: filter each band from the broad-band row, weight, sum
    FXC_TRY(set_smem_limit(k_s2s_mfband, smf));
    for (int b = 0; b < nbands; ++b) {
      const float fl = plan->band_freq_low[b + 1];
      int win = 2 * (int)(1.0 / (double)(fl * plan->delta)) + 1;
      if (win < 1) win = 1;
      k_s2s_mfband<<<(unsigned)nr, kS2sT, smf, ctx->stream>>>(
          x, d, pf, resp0 + (size_t)(b + 1) * rpitch, win, f2c(1.0 / (double)win), xb + (size_t)b * nr * seg,
          wb + (size_t)b * nr * seg, rb_of(smf_));
      count_launch();
      FXC_LAUNCH_CHECK();
    }
    dim3 g((unsigned)((seg + 255) / 256), (unsigned)nr);
    k_s2s_mfsum<<<g, 256, 0, ctx->stream>>>(xb, wb, nbands, (int64_t)nr * seg, d, x);
    count_launch();
    FXC_LAUNCH_CHECK();
    wgt = nullptr;
  }

  float2* out = reinterpret_cast<float2*>(d_out);
  if (wh_after) {
    FXC_TRY(set_smem_limit(k_s2s_whiten_a, sma));
    k_s2s_whiten_a<<<(unsigned)nr, kS2sT, sma, ctx->stream>>>(x, wgt, d, ps, tws, plan->whiten_win,
                                                              X, A, fpitch, rb_of(sma_));
    count_launch();
    FXC_LAUNCH_CHECK();
    FXC_TRY(set_smem_limit(k_s2s_whiten_b, smb));
    k_s2s_whiten_b<<<(unsigned)nr, kS2sT, smb, ctx->stream>>>(X, A, fpitch, d, ps, tws, po, two, 0,
                                                              0, 0, nullptr, nullptr, out,
                                                              out_pitch, rb_of(smb_));
    count_launch();
    FXC_LAUNCH_CHECK();
  } else {
    FXC_TRY(set_smem_limit(k_s2s_output, smo));
    k_s2s_output<<<(unsigned)nr, kS2sT, smo, ctx->stream>>>(x, wgt, d, po, two, out, out_pitch,
                                                            rb_of(smo_));
    count_launch();
    FXC_LAUNCH_CHECK();
  }
  return FXC_OK;
}

}  // extern "C"
