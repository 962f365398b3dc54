// Stacking stages: cross-timestamp linear stack, substack prestacking,
// phase-weighted stack (ncf_pws) and S-transform time-frequency PWS
// (ncf_tfpws).
//
// Reference behaviour reproduced here:
//   _linear_stack_group        fastxc/operators/stacking/linear_stack.py:228-247
//   prepare_sourcepack_host_item (PWS prestack = group means)
//                              native/pws/io/sourcepack_io.cu:385-478
//   TF-PWS prestack (group sums) native/tfpws/io/sourcepack_io.cu:440-490
//   compute_pws_host_batch + hilbertTransformKernel, cudaNormalizeComplex,
//   cudaWeightedMeanBatch, cudaMultiplyBatch
//                              native/pws/worker/gpu.cu:87-282, kernels/cuda.pws.cu
//   compute_tfpws_from_prestack + gaussianModulateSub, calculateWeightSub,
//   applyWeight, sumOverTimeAxisKernel, blendBandLimitedSpectrum, extractReal
//                              native/tfpws/core/tfpws_compute.cu:19-366,
//                              kernels/cuda.stransform.cu
//
// GB300 design: every row transform (N = 2001 = 3*23*29 lags for +-100 s at
// 10 Hz) stays in shared memory. PWS runs one CTA per pair that streams its
// groups (forward FFT, analytic mask in the digit-reversed layout, inverse
// DIT back to natural order, unit phasor, weighted sum) without writing any
// group row back. TF-PWS runs one CTA per (pair, frequency): the group
// voices of that frequency are produced and reduced into the weight in
// shared memory; the Gaussian window is evaluated in FP64. The weight power
// (1 in the reference) is a parameter.
#include <algorithm>
#include <cmath>
#include <vector>

// The row kernels' FFT stages run inline (no ABI save/restore of live
// registers around each stage; k_tfpws_freq then fits 128 registers):
// PWS 8.10 -> 7.66 ms on 512 pairs x 720 traces, TF-PWS 70.7 -> 68.2 ms on
// 64 pairs, same results.
#define FXC_FFT_STAGE_ATTR __forceinline__
// and so do k_pws's first forward stage (reading the group rows) and last
// inverse stage (accumulating the phasors): 6.73 -> 6.37 ms on 512 pairs x
// 720 traces, same bits (6.95 with those two out of line)
#define FXC_FFT_EDGE_ATTR __forceinline__
// k_pws's resident CTAs per SM: 5 caps it at 128 registers (8 bytes of
// spill) against the 168 ptxas picks unbounded, 12 -> 15 warps per SM:
// PWS 7.66 -> 6.94 ms on 512 pairs x 720 traces, same bits
#ifndef FXC_PWS_MIN_BLOCKS
#define FXC_PWS_MIN_BLOCKS 5
#endif
#include "context.cuh"
#include "exact_sum.cuh"
#include "fft.cuh"
#include "fft_any.cuh"
#include "fft_launch.cuh"

namespace fxc {

constexpr int kStT = 96;           // threads per row transform CTA
constexpr int kStNmax = 8192;      // longest directly transformed trace
constexpr int kStBluestein = 16384;  // longest Bluestein length (any other trace length)

// ---------------------------------------------------------------------------
// linear stack and prestack
// ---------------------------------------------------------------------------

// Cross-timestamp linear stack: exact int64 fixed-point column sums that
// reproduce _linear_stack_group's FP64 accumulation bit for bit
// (exact_sum.cuh). One sample column per thread, an 8-row register ring, one
// window branch per 2 rows (the fastest of the shapes timed on GB300).
constexpr int kLsT = 256, kLsV = 1;

__global__ void __launch_bounds__(kLsT)
    k_linear_stack(const float* __restrict__ traces, const int64_t* __restrict__ offs,
                   const int32_t* __restrict__ counts, int n, float* __restrict__ out) {
  linear_stack_cta<kLsT, kLsV, 8, 2>(traces, offs, counts, n, out);
}

// Group rows of `substack` consecutive traces (B < 2 -> 1): mode 0 mean
// (PWS), mode 1 sum (TF-PWS). weight[g] = count_g / count_p. linear: mode 0
// sum_g mean_g * weight_g, mode 1 sum_g sum_g / count_p.
__global__ void k_prestack(const float* __restrict__ traces, const int64_t* __restrict__ toffs,
                           const int32_t* __restrict__ tcounts, const int64_t* __restrict__ goffs,
                           int n, int substack, int mode, float* __restrict__ groups,
                           float* __restrict__ weights, float* __restrict__ linear) {
  const int p = blockIdx.y;
  const int64_t toff = toffs[p];
  const int cnt = tcounts[p];
  const int64_t goff = goffs[p];
  const int b = substack >= 2 ? substack : 1;
  const int ng = (cnt + b - 1) / b;
  const float inv_total = 1.0f / (float)cnt;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    float lin = 0.f;
    for (int g = 0; g < ng; ++g) {
      const int k0 = g * b, k1 = min(cnt, k0 + b);
      float s = 0.f;
      for (int k = k0; k < k1; ++k) s += traces[(toff + k) * n + t];
      const int gc = k1 - k0;
      float v, wgt;
      if (mode == 0) {
        // group mean, weight count/num_segments, linear += mean * weight
        v = s * (1.0f / (float)gc);
        wgt = (float)gc / (float)cnt;
        lin += v * wgt;
      } else {
        // group sum, weight count * (1/num_segments), linear += sum / num_segments
        v = s;
        wgt = (float)gc * inv_total;
        lin += s * inv_total;
      }
      groups[(goff + g) * n + t] = v;
      if (t == 0) weights[goff + g] = wgt;
    }
    linear[(int64_t)p * n + t] = lin;
  }
}

// ---------------------------------------------------------------------------
// shared pieces of the row transforms
// ---------------------------------------------------------------------------

// Analytic-signal mask of hilbertTransformKernel: bin 0 and bins >= (N+1)/2
// -> 0, the others x 2. buf holds the any_forward layout.
__device__ __forceinline__ void analytic_mask(float2* buf, const AnyPlan& a) {
  const int n = a.n;
  const int half = (n + 1) / 2;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int pos = any_pos(a, k);
    float2 v = buf[pos];
    if (k == 0 || k >= half)
      v = make_float2(0.f, 0.f);
    else
      v = make_float2(v.x * 2.0f, v.y * 2.0f);
    buf[pos] = v;
  }
}

__device__ __forceinline__ float weight_pow(float mag2, float power) {
  // |W|^power from |W|^2 (applyWeight: powf(rw*rw + iw*iw, 0.5*order))
  return power == 1.0f ? sqrtf(mag2) : powf(mag2, 0.5f * power);
}

// ---------------------------------------------------------------------------
// PWS: one CTA per (pair, chunk of groups)
// ---------------------------------------------------------------------------

// 1 / max(|z|, 1e-7) for |z|^2 = m2 (cudaNormalizeComplex's floored
// modulus) by one reciprocal square root: within a few ulp of the division
// by the square root, and two IEEE divisions and a square root per sample
// fewer in the phase loops.
__device__ __forceinline__ float inv_mod_floor(float m2) { return m2 > 1e-14f ? rsqrtf(m2) : 1e7f; }

// Asks L2 for floats [0, count) of row x, one request per 32-byte sector,
// spread over the CTA's threads: issued an iteration ahead, the group rows
// a CTA reads next are in L2 by the time its loads ask for them.
__device__ __forceinline__ void prefetch_rows_l2(const float* x, int count) {
  for (int i = threadIdx.x * 8; i < count; i += kStT * 8)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(x + i));
}

// Two group rows as the real and imaginary parts of one transform input
// (the second zero when there is none), read from global memory by the
// first DIF stage itself.
struct GroupPairLoad {
  const float* __restrict__ x1;
  const float* __restrict__ x2;
  bool two;
  __device__ __forceinline__ float2 operator()(int k) const { return make_float2(x1[k], two ? x2[k] : 0.f); }
};

// The phasor accumulation of two groups at lag t, fed by the last DIT stage
// with h = N (H(x1) + i H(x2)) at t: the cudaNormalizeComplex (modulus
// floored at 1e-7) + cudaWeightedMeanBatch of k_pws below.
struct GroupPairAccumulate {
  const float* __restrict__ x1;
  const float* __restrict__ x2;
  float2* acc;
  float m1, m2, w1, w2, invn;
  bool two;
  __device__ __forceinline__ void operator()(int t, float2 h) const {
    float re = x1[t] - m1, im = h.x * invn;
    float s = inv_mod_floor(re * re + im * im) * w1;
    float2 ac = acc[t];
    ac.x += re * s;
    ac.y += im * s;
    if (two) {
      re = x2[t] - m2;
      im = h.y * invn;
      s = inv_mod_floor(re * re + im * im) * w2;
      ac.x += re * s;
      ac.y += im * s;
    }
    acc[t] = ac;
  }
};

// CTA (pair p, chunk c) sums the weighted unit phasors of groups
// [c * cg, (c + 1) * cg) of pair p into partial row (p, c); k_pws_combine
// adds a pair's partial rows in chunk order. Chunks keep the grid many
// waves deep (one CTA per pair left the last of 2.5 waves half empty).
__global__ void __launch_bounds__(kStT, FXC_PWS_MIN_BLOCKS)
    k_pws(const float* __restrict__ groups, const float* __restrict__ weights,
          const int64_t* __restrict__ goffs, const int32_t* __restrict__ gcounts, int cg, AnyPlan a,
          float2* __restrict__ partial) {
  extern __shared__ float2 sm[];
  const int n = a.n;
  float2* buf = sm;
  float2* acc = sm + any_buf_elems(a);
  float2* stw = acc + n;
  const int pair = blockIdx.x;
  const int g0 = blockIdx.y * cg;
  const int64_t goff = goffs[pair] + g0;
  const int ng = max(0, min(cg, gcounts[pair] - g0));
  fft_twiddles_to_smem<kStT>(a.p, stw);
  for (int t = threadIdx.x; t < n; t += kStT) acc[t] = make_float2(0.f, 0.f);
  const float invn = 1.0f / (float)n;
  __shared__ float2 dc;
  if (n & 1) {
    // Odd N (every NCF: N = 2 half_cc + 1). The masked inverse z/N of the
    // reference is x - mean(x) + i H(x): its real part needs no transform,
    // and the Hilbert transform H is real-to-real, so two groups share one
    // forward transform of x1 + i x2 and one inverse of -i sign(k) Z(k),
    // which returns N (H(x1) + i H(x2)). One transform per group instead of
    // two; the group rows are read again (from L2) for the real parts.
    const int half = (n + 1) / 2;
    // direct transforms of two or more stages: the first forward stage
    // reads the group rows itself and the last inverse stage accumulates the
    // phasors, two passes over shared memory and two barriers fewer per pair
    // of groups than the row copy in and the accumulation pass out
    const bool fused = a.chirp == nullptr && a.p.nstages >= 2;
    for (int g = 0; g < ng; g += 2) {
      const bool two = g + 1 < ng;
      const float* x1 = groups + (goff + g) * n;
      const float* x2 = two ? x1 + n : x1;
      const float w1 = weights[goff + g];
      const float w2 = two ? weights[goff + g + 1] : 0.f;
      if (g + 2 < ng) prefetch_rows_l2(x1 + 2 * n, (g + 3 < ng ? 2 : 1) * n);  // the next two groups
      __syncthreads();
      if (fused) {
        fft_dif_stage0_load<kStT, false>(buf, a.p, stw, GroupPairLoad{x1, x2, two});
        fft_dif_inner<kStT, false>(buf, a.p, stw, 1, a.p.nstages);
      } else {
        for (int t = threadIdx.x; t < n; t += kStT) buf[t] = make_float2(x1[t], two ? x2[t] : 0.f);
        __syncthreads();
        any_forward<kStT>(buf, a, stw);
      }
      for (int k = threadIdx.x; k < n; k += kStT) {
        const int pos = any_pos(a, k);
        const float2 z = buf[pos];
        if (k == 0) dc = z;  // (sum x1, sum x2)
        // -i z for 0 < k < N/2, +i z above, 0 at DC
        buf[pos] = k == 0 ? make_float2(0.f, 0.f) : (k < half ? mul_mi(z) : mul_pi(z));
      }
      __syncthreads();
      if (fused) {
        fft_dit_head<kStT, false>(buf, a.p, stw, true);
        fft_dit_last_store<kStT, false>(
            buf, a.p, stw, true, GroupPairAccumulate{x1, x2, acc, dc.x * invn, dc.y * invn, w1, w2, invn, two});
        continue;
      }
      any_inverse<kStT>(buf, a, stw);
      const float m1 = dc.x * invn, m2 = dc.y * invn;
      for (int t = threadIdx.x; t < n; t += kStT) {
        const float2 h = buf[t];
        // cudaNormalizeComplex (modulus floored at 1e-7) + cudaWeightedMeanBatch
        float re = x1[t] - m1, im = h.x * invn;
        float s = inv_mod_floor(re * re + im * im) * w1;
        float2 ac = acc[t];
        ac.x += re * s;
        ac.y += im * s;
        if (two) {
          re = x2[t] - m2;
          im = h.y * invn;
          s = inv_mod_floor(re * re + im * im) * w2;
          ac.x += re * s;
          ac.y += im * s;
        }
        acc[t] = ac;
      }
    }
  } else {
    for (int g = 0; g < ng; ++g) {
      const float* x = groups + (goff + g) * n;
      const float wg = weights[goff + g];
      if (g + 1 < ng) prefetch_rows_l2(x + n, n);  // the next group
      __syncthreads();
      for (int t = threadIdx.x; t < n; t += kStT) buf[t] = make_float2(x[t], 0.f);
      __syncthreads();
      any_forward<kStT>(buf, a, stw);  // R2C into an N-point row (full spectrum)
      analytic_mask(buf, a);
      __syncthreads();
      any_inverse<kStT>(buf, a, stw);  // C2C inverse, unnormalised, natural order
      for (int t = threadIdx.x; t < n; t += kStT) {
        // cudaNormalizeComplex: z / nfft, modulus floored at 1e-7
        const float2 z = buf[t];
        const float re = z.x * invn, im = z.y * invn;
        // cudaWeightedMeanBatch
        const float sc = inv_mod_floor(re * re + im * im) * wg;
        acc[t].x += re * sc;
        acc[t].y += im * sc;
      }
    }
  }
  __syncthreads();
  float2* o = partial + ((int64_t)pair * gridDim.y + blockIdx.y) * n;
  for (int t = threadIdx.x; t < n; t += kStT) o[t] = acc[t];
}

// out[p] = lin[p] * |sum_c partial[p][c]|^power, chunks added in order.
__global__ void k_pws_combine(const float2* __restrict__ partial, int nchunks, const float* __restrict__ linear,
                              int n, int64_t total, float power, float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = i / n, t = i - p * n;
    const float2* row = partial + p * nchunks * n + t;
    float2 s = row[0];
    for (int c = 1; c < nchunks; ++c) {
      const float2 v = row[(int64_t)c * n];
      s.x += v.x;
      s.y += v.y;
    }
    out[i] = linear[i] * weight_pow(s.x * s.x + s.y * s.y, power);
  }
}

// Streaming PWS: one group (e.g. one day's NCF of every pair) per call.
// acc[p] += w * unit analytic phasor of row p, lin[p] += w * row p; the
// same per-sample arithmetic as k_pws, summed call by call. Odd lengths
// take rows two at a time through one forward and one inverse transform
// (the Hilbert parts of both; the real parts are x - mean), as k_pws does.
__global__ void __launch_bounds__(kStT)
    k_pws_stream_add(const float* __restrict__ rows, int64_t rows_pitch, int nrows, AnyPlan a, float w,
                     float2* __restrict__ acc, float* __restrict__ lin) {
  extern __shared__ float2 sm[];
  const int n = a.n;
  float2* buf = sm;
  float2* stw = sm + any_buf_elems(a);
  fft_twiddles_to_smem<kStT>(a.p, stw);
  if (n & 1) {
    __shared__ float2 dc;
    const int64_t r1 = 2 * (int64_t)blockIdx.x;
    const bool two = r1 + 1 < nrows;
    const float* x1 = rows + r1 * rows_pitch;
    const float* x2 = two ? x1 + rows_pitch : x1;
    for (int t = threadIdx.x; t < n; t += kStT) buf[t] = make_float2(x1[t], two ? x2[t] : 0.f);
    __syncthreads();
    any_forward<kStT>(buf, a, stw);
    const int half = (n + 1) / 2;
    for (int k = threadIdx.x; k < n; k += kStT) {
      const int pos = any_pos(a, k);
      const float2 z = buf[pos];
      if (k == 0) dc = z;  // (sum x1, sum x2)
      // -i z for 0 < k < N/2, +i z above, 0 at DC
      buf[pos] = k == 0 ? make_float2(0.f, 0.f) : (k < half ? mul_mi(z) : mul_pi(z));
    }
    __syncthreads();
    any_inverse<kStT>(buf, a, stw);
    const float invn = 1.0f / (float)n;
    const float m1 = dc.x * invn, m2 = dc.y * invn;
    float2* ac1 = acc + r1 * n;
    float* li1 = lin + r1 * n;
    for (int t = threadIdx.x; t < n; t += kStT) {
      const float2 h = buf[t];
      float re = x1[t] - m1, im = h.x * invn;
      float sc = inv_mod_floor(re * re + im * im) * w;
      float2 v = ac1[t];
      v.x += re * sc;
      v.y += im * sc;
      ac1[t] = v;
      li1[t] += x1[t] * w;
      if (two) {
        re = x2[t] - m2;
        im = h.y * invn;
        sc = inv_mod_floor(re * re + im * im) * w;
        v = ac1[n + t];
        v.x += re * sc;
        v.y += im * sc;
        ac1[n + t] = v;
        li1[n + t] += x2[t] * w;
      }
    }
    return;
  }
  const float* x = rows + (int64_t)blockIdx.x * rows_pitch;
  for (int t = threadIdx.x; t < n; t += kStT) buf[t] = make_float2(x[t], 0.f);
  __syncthreads();
  any_forward<kStT>(buf, a, stw);
  analytic_mask(buf, a);
  __syncthreads();
  any_inverse<kStT>(buf, a, stw);
  const float invn = 1.0f / (float)n;
  float2* ac = acc + (int64_t)blockIdx.x * n;
  float* li = lin + (int64_t)blockIdx.x * n;
  for (int t = threadIdx.x; t < n; t += kStT) {
    const float2 z = buf[t];
    const float re = z.x * invn, im = z.y * invn;
    const float sc = inv_mod_floor(re * re + im * im) * w;
    float2 v = ac[t];
    v.x += re * sc;
    v.y += im * sc;
    ac[t] = v;
    li[t] += x[t] * w;
  }
}

__global__ void k_pws_stream_finish(const float2* __restrict__ acc, const float* __restrict__ lin, int64_t total,
                                    float power, float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = acc[i];
    out[i] = lin[i] * weight_pow(a.x * a.x + a.y * a.y, power);
  }
}

// ---------------------------------------------------------------------------
// TF-PWS
// ---------------------------------------------------------------------------

// Analytic spectrum (natural order) of every row: groups of all pairs, then
// the linear stack of every pair.
__global__ void __launch_bounds__(kStT)
    k_analytic_spectrum(const float* __restrict__ rows, AnyPlan a, float2* __restrict__ out) {
  extern __shared__ float2 sm[];
  const int n = a.n;
  float2* buf = sm;
  float2* stw = sm + any_buf_elems(a);
  fft_twiddles_to_smem<kStT>(a.p, stw);
  const float* x = rows + (int64_t)blockIdx.x * n;
  for (int t = threadIdx.x; t < n; t += kStT) buf[t] = make_float2(x[t], 0.f);
  __syncthreads();
  any_forward<kStT>(buf, a, stw);
  analytic_mask(buf, a);
  __syncthreads();
  float2* o = out + (int64_t)blockIdx.x * n;
  for (int k = threadIdx.x; k < n; k += kStT) o[k] = buf[any_pos(a, k)];
}

struct TfBand {
  int limited;
  float df, fmin, fmax, taper;
};

// gaussianModulateSub factor (FP64): f = 0 -> 1; c = 0 -> 0; c < (N+1)/2 ->
// exp(-2 pi^2 c^2 scale / f^2); otherwise the mirror c' = N - c under the
// same rules.
__device__ __forceinline__ float gauss_factor(int c, int f, int n, double scale) {
  if (f == 0) return 1.0f;
  if (c == 0) return 0.0f;
  const int half = (n + 1) / 2;
  int cc = c;
  if (c >= half) {
    cc = n - c;
    if (!(cc < half && cc != 0)) return 0.0f;
  }
  const double pi = 3.14159265358979323846;
  return (float)exp(-2.0 * pi * pi * (double)cc * (double)cc * scale / ((double)f * (double)f));
}

// The factors of every (frequency, shift) once per call: they do not depend
// on the pair, and FP64 exp per CTA would load GB300's slow FP64 pipe.
__global__ void k_tfpws_gauss(float* __restrict__ gtab, int n, int nfreq) {
  const int64_t total = (int64_t)nfreq * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    gtab[i] = gauss_factor((int)(i % n), (int)(i / n), n, 0.1);
}

// calculateWeightSub for one lag t of a group's voice z: W[t] += wg z /
// (|z| N), a modulus <= 1e-7 taken as 1; 1/|z| by one reciprocal square
// root (within a few ulp of the two divisions by |z| N).
// Group spectrum X shifted by f and Gaussian-windowed at frequency c
// (gaussianModulateSub): the voice transform's input at c.
struct VoiceLoad {
  const float2* __restrict__ X;
  const float* gs;
  int f, n;
  __device__ __forceinline__ float2 operator()(int c) const {
    int k = f + c;
    if (k >= n) k -= n;
    const float2 v = X[k];
    const float gf = gs[c];
    return make_float2(v.x * gf, v.y * gf);
  }
};

struct VoiceWeightAdd {
  float2* W;
  float wg, invnf;
  __device__ __forceinline__ void operator()(int t, float2 z) const {
    const float m2 = z.x * z.x + z.y * z.y;
    const float sc = wg * (m2 <= 1e-14f ? 1.0f : rsqrtf(m2)) * invnf;
    W[t].x += z.x * sc;
    W[t].y += z.y * sc;
  }
};

// One CTA per (frequency f, pair): voices of every group and of the linear
// stack at f, the time-frequency weight, the weighted stack voice summed
// over time -> bin f of the output spectrum (band blend applied).
__global__ void __launch_bounds__(kStT)
    k_tfpws_freq(const float2* __restrict__ Xg, const float2* __restrict__ Xl,
                 const float* __restrict__ weights, const int64_t* __restrict__ goffs,
                 const int32_t* __restrict__ gcounts, AnyPlan a, int f0, TfBand band, float power,
                 const float* __restrict__ gtab, float2* __restrict__ spec_out) {
  extern __shared__ float2 sm[];
  __shared__ float sred[kStT / 32];
  __shared__ float sredi[kStT / 32];
  const int n = a.n;
  float2* buf = sm;
  float2* W = sm + any_buf_elems(a);
  float* gs = reinterpret_cast<float*>(W + n);
  float2* stw = reinterpret_cast<float2*>(gs + ((n + 1) & ~1));
  const int f = f0 + blockIdx.x;
  const int pair = blockIdx.y;
  const int nfreq = n / 2 + 1;
  if (f >= nfreq) return;
  float alpha = 1.0f;
  if (band.limited) {
    const float freq = (float)f * band.df;
    if (!(freq >= band.fmin && freq <= band.fmax)) return;  // bin keeps the linear spectrum
    const float bw = band.fmax - band.fmin;
    const float tp = fminf(band.taper, 0.5f * bw);
    const float pi = 3.14159265358979323846f;
    if (tp <= 0.0f) {
      alpha = 1.0f;
    } else if (freq < band.fmin + tp) {
      alpha = 0.5f - 0.5f * cosf(pi * ((freq - band.fmin) / tp));
    } else if (freq > band.fmax - tp) {
      alpha = 0.5f - 0.5f * cosf(pi * ((band.fmax - freq) / tp));
    }
  }
  fft_twiddles_to_smem<kStT>(a.p, stw);
  for (int c = threadIdx.x; c < n; c += kStT) {
    gs[c] = gtab[(int64_t)f * n + c];
    W[c] = make_float2(0.f, 0.f);
  }
  const int64_t goff = goffs[pair];
  const int ng = gcounts[pair];
  const float invnf = 1.0f / (float)n;
  const bool fused = a.chirp == nullptr && a.p.nstages >= 2;
  for (int g = 0; g < ng; ++g) {
    const float2* X = Xg + (goff + g) * n;
    const float wg = weights[goff + g];
    __syncthreads();
    // voice of group g (unnormalised C2C inverse): for direct plans of two
    // or more stages the first DIT stage reads the windowed spectrum itself
    // and the last adds each lag's weight term
    if (fused) {
      fft_dit_first_load<kStT, false>(buf, a.p, a.iperm, true, VoiceLoad{X, gs, f, n});
      fft_dit_head<kStT, false>(buf, a.p, stw, true, a.p.nstages - 2);
      fft_dit_last_store<kStT, false>(buf, a.p, stw, true, VoiceWeightAdd{W, wg, invnf});
      continue;
    }
    for (int c = threadIdx.x; c < n; c += kStT) buf[any_pos(a, c)] = VoiceLoad{X, gs, f, n}(c);
    __syncthreads();
    any_inverse<kStT, false>(buf, a, stw);
    for (int t = threadIdx.x; t < n; t += kStT) {
      const float2 z = buf[t];
      VoiceWeightAdd{W, wg, invnf}(t, z);
    }
  }
  __syncthreads();
  const float2* XL = Xl + (int64_t)pair * n;
  for (int c = threadIdx.x; c < n; c += kStT) {
    int k = f + c;
    if (k >= n) k -= n;
    const float2 v = XL[k];
    const float gf = gs[c];
    buf[any_pos(a, c)] = make_float2(v.x * gf, v.y * gf);
  }
  __syncthreads();
  any_inverse<kStT, false>(buf, a, stw);  // stack voice (full dispatch: 128 registers without spills here)
  // applyWeight + sumOverTimeAxisKernel
  float sr = 0.f, si = 0.f;
  for (int t = threadIdx.x; t < n; t += kStT) {
    const float mag = weight_pow(W[t].x * W[t].x + W[t].y * W[t].y, power);
    sr += buf[t].x * mag;
    si += buf[t].y * mag;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    si += __shfl_xor_sync(0xffffffffu, si, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sred[threadIdx.x >> 5] = sr;
    sredi[threadIdx.x >> 5] = si;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float tr = 0.f, ti = 0.f;
    for (int w = 0; w < kStT / 32; ++w) {
      tr += sred[w];
      ti += sredi[w];
    }
    float2 val = make_float2(tr, ti);
    if (band.limited) {
      // blendBandLimitedSpectrum
      const float2 lin = XL[f];
      val = make_float2(lin.x * (1.0f - alpha) + val.x * alpha, lin.y * (1.0f - alpha) + val.y * alpha);
    }
    spec_out[(int64_t)pair * n + f] = val;
  }
}

// Final C2C inverse of the output spectrum, real part / N (extractReal).
__global__ void __launch_bounds__(kStT)
    k_tfpws_final(const float2* __restrict__ spec, AnyPlan a, float* __restrict__ out) {
  extern __shared__ float2 sm[];
  const int n = a.n;
  float2* buf = sm;
  float2* stw = sm + any_buf_elems(a);
  fft_twiddles_to_smem<kStT>(a.p, stw);
  const float2* S = spec + (int64_t)blockIdx.x * n;
  for (int k = threadIdx.x; k < n; k += kStT) buf[any_pos(a, k)] = S[k];
  __syncthreads();
  any_inverse<kStT>(buf, a, stw);
  float* o = out + (int64_t)blockIdx.x * n;
  for (int t = threadIdx.x; t < n; t += kStT) o[t] = buf[t].x / (float)n;
}

// output spectrum initialisation: band-limited -> the linear analytic
// spectrum everywhere (bins outside the band keep it), else zeros.
__global__ void k_tfpws_init(const float2* __restrict__ Xl, int64_t total, int limited,
                             float2* __restrict__ spec) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    spec[i] = limited ? Xl[i] : make_float2(0.f, 0.f);
}

static int stack_plan(int n, AnyPlan* a) {
  FXC_CHECK_ARG(n >= 2, "trace length %d below 2", n);
  return any_plan(n, kStNmax, kStBluestein, a);
}

struct PairGroups {
  std::vector<int64_t> offs;
  std::vector<int32_t> counts;
};

}  // namespace fxc

using namespace fxc;

extern "C" {

int fxc_linear_stack(fxc_ctx* ctx, const float* d_traces, const int64_t* h_offsets,
                     const int32_t* h_counts, int32_t npairs, int32_t nsamples, float* d_out) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(npairs >= 0 && nsamples > 0, "invalid shape");
  if (npairs == 0) return FXC_OK;
  FXC_CHECK_ARG(d_traces && h_offsets && h_counts && d_out, "null pointer");
  FXC_CHECK_ARG(npairs <= 65535, "at most 65535 pairs per call");
  const size_t ob = sizeof(int64_t) * npairs, cb = sizeof(int32_t) * npairs;
  FXC_TRY(ctx->scratch2.reserve(ob + cb + 256));
  int64_t* d_off = reinterpret_cast<int64_t*>(ctx->scratch2.ptr);
  int32_t* d_cnt = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(ctx->scratch2.ptr) + ((ob + 255) & ~size_t(255)));
  FXC_CUDA_TRY(cudaMemcpyAsync(d_off, h_offsets, ob, cudaMemcpyHostToDevice, ctx->stream));
  FXC_CUDA_TRY(cudaMemcpyAsync(d_cnt, h_counts, cb, cudaMemcpyHostToDevice, ctx->stream));
  dim3 g((unsigned)((nsamples + kLsT * kLsV - 1) / (kLsT * kLsV)), (unsigned)npairs);
  k_linear_stack<<<g, kLsT, 0, ctx->stream>>>(d_traces, d_off, d_cnt, nsamples, d_out);
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

int fxc_stack_prestack(fxc_ctx* ctx, const float* d_traces, const int64_t* h_trace_offsets,
                       const int32_t* h_trace_counts, int32_t npairs, int32_t nsamples,
                       int32_t substack, int32_t mode, float* d_groups, float* d_weights,
                       float* d_linear, int64_t* h_group_offsets, int32_t* h_group_counts) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(npairs >= 0 && nsamples > 0 && (mode == 0 || mode == 1), "invalid arguments");
  if (npairs == 0) return FXC_OK;
  FXC_CHECK_ARG(npairs <= 65535, "at most 65535 pairs per call");
  FXC_CHECK_ARG(d_traces && h_trace_offsets && h_trace_counts && d_groups && d_weights && d_linear &&
                    h_group_offsets && h_group_counts, "null pointer");
  const int b = substack >= 2 ? substack : 1;
  int64_t goff = 0;
  for (int p = 0; p < npairs; ++p) {
    FXC_CHECK_ARG(h_trace_counts[p] >= 1, "pair %d has no traces", p);
    h_group_offsets[p] = goff;
    h_group_counts[p] = (h_trace_counts[p] + b - 1) / b;
    goff += h_group_counts[p];
  }
  const size_t n8 = sizeof(int64_t) * npairs, n4 = sizeof(int32_t) * npairs;
  const size_t o2 = (n8 + 255) & ~size_t(255), o3 = o2 + ((n4 + 255) & ~size_t(255));
  FXC_TRY(ctx->scratch2.reserve(o3 + n8 + 256));
  char* base = reinterpret_cast<char*>(ctx->scratch2.ptr);
  int64_t* d_toff = reinterpret_cast<int64_t*>(base);
  int32_t* d_tcnt = reinterpret_cast<int32_t*>(base + o2);
  int64_t* d_goff = reinterpret_cast<int64_t*>(base + o3);
  FXC_CUDA_TRY(cudaMemcpyAsync(d_toff, h_trace_offsets, n8, cudaMemcpyHostToDevice, ctx->stream));
  FXC_CUDA_TRY(cudaMemcpyAsync(d_tcnt, h_trace_counts, n4, cudaMemcpyHostToDevice, ctx->stream));
  FXC_CUDA_TRY(cudaMemcpyAsync(d_goff, h_group_offsets, n8, cudaMemcpyHostToDevice, ctx->stream));
  dim3 g((unsigned)((nsamples + 255) / 256), (unsigned)npairs);
  k_prestack<<<g, 256, 0, ctx->stream>>>(d_traces, d_toff, d_tcnt, d_goff, nsamples, substack, mode,
                                         d_groups, d_weights, d_linear);
  count_launch();
  FXC_LAUNCH_CHECK();
  // the host arrays outlive the call; keep the copies ordered before return
  FXC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FXC_OK;
}

int fxc_pws_stream_add(fxc_ctx* ctx, const float* d_rows, int64_t rows_pitch, int32_t npairs, int32_t nsamples,
                       float weight, float* d_acc, float* d_lin) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(npairs >= 0 && nsamples >= 2 && rows_pitch >= nsamples, "invalid shape");
  if (npairs == 0) return FXC_OK;
  FXC_CHECK_ARG(d_rows && d_acc && d_lin, "null pointer");
  AnyPlan a;
  FXC_TRY(stack_plan(nsamples, &a));
  const size_t smem = sizeof(float2) * ((size_t)any_buf_elems(a) + fft_tw_smem_elems(a.p));
  FXC_TRY(set_smem_limit(k_pws_stream_add, smem));
  const unsigned grid = (nsamples & 1) ? (unsigned)((npairs + 1) / 2) : (unsigned)npairs;
  k_pws_stream_add<<<grid, kStT, smem, ctx->stream>>>(d_rows, rows_pitch, npairs, a, weight,
                                                      reinterpret_cast<float2*>(d_acc), d_lin);
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

int fxc_pws_stream_finish(fxc_ctx* ctx, const float* d_acc, const float* d_lin, int32_t npairs, int32_t nsamples,
                          float power, float* d_out) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(npairs >= 0 && nsamples >= 1, "invalid shape");
  if (npairs == 0) return FXC_OK;
  FXC_CHECK_ARG(d_acc && d_lin && d_out, "null pointer");
  k_pws_stream_finish<<<1024, 256, 0, ctx->stream>>>(reinterpret_cast<const float2*>(d_acc), d_lin,
                                                     (int64_t)npairs * nsamples, power, d_out);
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

int fxc_pws_run(fxc_ctx* ctx, const float* d_groups, const float* d_weights,
                const int64_t* h_group_offsets, const int32_t* h_group_counts, int32_t npairs,
                const float* d_linear, int32_t nsamples, float power, float* d_out) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(npairs >= 0, "invalid npairs");
  if (npairs == 0) return FXC_OK;
  FXC_CHECK_ARG(d_groups && d_weights && h_group_offsets && h_group_counts && d_linear && d_out,
                "null pointer");
  AnyPlan a;
  FXC_TRY(stack_plan(nsamples, &a));
  const size_t n8 = sizeof(int64_t) * npairs, n4 = sizeof(int32_t) * npairs;
  const size_t o2 = (n8 + 255) & ~size_t(255);
  FXC_TRY(ctx->scratch2.reserve(o2 + n4 + 256));
  char* base = reinterpret_cast<char*>(ctx->scratch2.ptr);
  int64_t* d_goff = reinterpret_cast<int64_t*>(base);
  int32_t* d_gcnt = reinterpret_cast<int32_t*>(base + o2);
  FXC_CUDA_TRY(cudaMemcpyAsync(d_goff, h_group_offsets, n8, cudaMemcpyHostToDevice, ctx->stream));
  FXC_CUDA_TRY(cudaMemcpyAsync(d_gcnt, h_group_counts, n4, cudaMemcpyHostToDevice, ctx->stream));
  const size_t smem =
      sizeof(float2) * ((size_t)any_buf_elems(a) + (size_t)nsamples + fft_tw_smem_elems(a.p));
  FXC_TRY(set_smem_limit(k_pws, smem));
  // chunks of an even number of groups, enough CTAs for ~8 waves of the
  // resident ones (register-bound at about 6 per SM)
  int ngmax = 1, nsm = 0;
  for (int p = 0; p < npairs; ++p) ngmax = std::max(ngmax, (int)h_group_counts[p]);
  FXC_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
  const int64_t want = std::max<int64_t>(1, (8LL * 6 * std::max(nsm, 1) + npairs - 1) / npairs);
  int nchunks = (int)std::min<int64_t>(want, (ngmax + 1) / 2);
  int cg = (ngmax + nchunks - 1) / nchunks;
  cg += cg & 1;
  nchunks = (ngmax + cg - 1) / cg;
  FXC_CHECK_ARG(nchunks <= 65535, "too many group chunks");
  FXC_TRY(ctx->scratch4.reserve(sizeof(float2) * (size_t)npairs * (size_t)nchunks * (size_t)nsamples));
  float2* d_part = reinterpret_cast<float2*>(ctx->scratch4.ptr);
  k_pws<<<dim3((unsigned)npairs, (unsigned)nchunks), kStT, smem, ctx->stream>>>(d_groups, d_weights, d_goff,
                                                                               d_gcnt, cg, a, d_part);
  count_launch();
  FXC_LAUNCH_CHECK();
  const int64_t total = (int64_t)npairs * nsamples;
  k_pws_combine<<<(unsigned)std::min<int64_t>((total + 255) / 256, 152 * 32), 256, 0, ctx->stream>>>(
      d_part, nchunks, d_linear, nsamples, total, power, d_out);
  count_launch();
  FXC_LAUNCH_CHECK();
  FXC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FXC_OK;
}

int fxc_tfpws_run(fxc_ctx* ctx, const float* d_groups, const float* d_weights,
                  const int64_t* h_group_offsets, const int32_t* h_group_counts, int32_t npairs,
                  const float* d_linear, int32_t nsamples, float delta, int32_t band_limited,
                  float fmin, float fmax, float taper_hz, float power, float* d_out) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(npairs >= 0, "invalid npairs");
  if (npairs == 0) return FXC_OK;
  FXC_CHECK_ARG(d_groups && d_weights && h_group_offsets && h_group_counts && d_linear && d_out,
                "null pointer");
  FXC_CHECK_ARG(npairs <= 65535, "at most 65535 pairs per call");
  AnyPlan a;
  FXC_TRY(stack_plan(nsamples, &a));
  const int n = nsamples;
  int64_t total_groups = 0;
  for (int i = 0; i < npairs; ++i) total_groups = std::max<int64_t>(total_groups, h_group_offsets[i] + h_group_counts[i]);
  TfBand band{0, 0.f, 0.f, 0.f, 0.f};
  if (band_limited) {
    // compute_tfpws_from_prestack (tfpws_compute.cu:112-153)
    FXC_CHECK_ARG(delta > 0.0f, "band limit needs delta > 0");
    const double df_hz = 1.0 / ((double)n * (double)delta);
    const double nyq = 0.5 / (double)delta;
    FXC_CHECK_ARG((double)fmin < nyq, "band lower bound %g above Nyquist %g", fmin, nyq);
    double fm = fmax;
    if (fm > nyq) fm = nyq;
    double tp = taper_hz;
    if (tp < 0.0) tp = 0.05 * (fm - (double)fmin);
    band = TfBand{1, (float)df_hz, fmin, (float)fm, (float)tp};
  }
  const size_t n8 = sizeof(int64_t) * npairs, n4 = sizeof(int32_t) * npairs;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t o_gcnt = al(n8);
  const size_t o_xg = o_gcnt + al(n4);
  const size_t o_xl = o_xg + al(sizeof(float2) * (size_t)total_groups * n);
  const size_t o_sp = o_xl + al(sizeof(float2) * (size_t)npairs * n);
  const int nfreq = n / 2 + 1;
  const size_t o_gt = o_sp + al(sizeof(float2) * (size_t)npairs * n);
  const size_t total = o_gt + al(sizeof(float) * (size_t)nfreq * n);
  FXC_TRY(ctx->scratch4.reserve(total));
  char* base = reinterpret_cast<char*>(ctx->scratch4.ptr);
  int64_t* d_goff = reinterpret_cast<int64_t*>(base);
  int32_t* d_gcnt = reinterpret_cast<int32_t*>(base + o_gcnt);
  float2* Xg = reinterpret_cast<float2*>(base + o_xg);
  float2* Xl = reinterpret_cast<float2*>(base + o_xl);
  float2* spec = reinterpret_cast<float2*>(base + o_sp);
  float* gtab = reinterpret_cast<float*>(base + o_gt);
  FXC_CUDA_TRY(cudaMemcpyAsync(d_goff, h_group_offsets, n8, cudaMemcpyHostToDevice, ctx->stream));
  FXC_CUDA_TRY(cudaMemcpyAsync(d_gcnt, h_group_counts, n4, cudaMemcpyHostToDevice, ctx->stream));
  const size_t sm1 = sizeof(float2) * ((size_t)any_buf_elems(a) + fft_tw_smem_elems(a.p));
  FXC_TRY(set_smem_limit(k_analytic_spectrum, sm1));
  FXC_CHECK_ARG(total_groups <= 0x7fffffff, "too many groups");
  if (total_groups > 0) {
    k_analytic_spectrum<<<(unsigned)total_groups, kStT, sm1, ctx->stream>>>(d_groups, a, Xg);
    count_launch();
    FXC_LAUNCH_CHECK();
  }
  k_analytic_spectrum<<<(unsigned)npairs, kStT, sm1, ctx->stream>>>(d_linear, a, Xl);
  count_launch();
  FXC_LAUNCH_CHECK();
  k_tfpws_init<<<1024, 256, 0, ctx->stream>>>(Xl, (int64_t)npairs * n, band_limited, spec);
  count_launch();
  FXC_LAUNCH_CHECK();
  k_tfpws_gauss<<<1024, 256, 0, ctx->stream>>>(gtab, n, nfreq);
  count_launch();
  FXC_LAUNCH_CHECK();
  const size_t sm2 = sizeof(float2) * ((size_t)any_buf_elems(a) + (size_t)n + fft_tw_smem_elems(a.p)) +
                     sizeof(float) * (size_t)((n + 1) & ~1);
  FXC_TRY(set_smem_limit(k_tfpws_freq, sm2));
  for (int f0 = 0; f0 < nfreq; f0 += 65535) {
    dim3 g((unsigned)std::min(65535, nfreq - f0), (unsigned)npairs);
    k_tfpws_freq<<<g, kStT, sm2, ctx->stream>>>(Xg, Xl, d_weights, d_goff, d_gcnt, a, f0, band, power,
                                                gtab, spec);
    count_launch();
    FXC_LAUNCH_CHECK();
  }
  FXC_TRY(set_smem_limit(k_tfpws_final, sm1));
  k_tfpws_final<<<(unsigned)npairs, kStT, sm1, ctx->stream>>>(spec, a, d_out);
  count_launch();
  FXC_LAUNCH_CHECK();
  FXC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FXC_OK;
}

}  // extern "C"
