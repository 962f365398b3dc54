// Launch-shape constants and the real-transform pre/post twiddle steps shared
// by every kernel that embeds a real FFT.
#pragma once

#include "fft.cuh"

namespace fxc {

// Small rows (NCF lengths such as 2001, 4001 after Bluestein): 256 threads.
constexpr int kFftSmallT = 256;
constexpr int kFftSmallNmax = 4096;
// Long rows (the 36 000 .. 38 400-point real transforms of sac2spec / xc):
// one CTA per SM holding the complex half-length row.
#ifndef FXC_FFT_LARGE_THREADS
#define FXC_FFT_LARGE_THREADS 1024
#endif
constexpr int kFftLargeT = FXC_FFT_LARGE_THREADS;
constexpr int kFftLargeNmax = 20480;

template <typename K>
inline int set_smem_limit(K kernel, size_t smem) {
  if (smem > 48 * 1024) {
    FXC_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  return FXC_OK;
}

// Post-processing of a length-2M real forward transform computed as the
// length-M complex FFT Z of z[m] = x[2m] + i x[2m+1]:
//   X[k] = (Z[k] + conj Z[M-k]) / 2 + w^k (Z[k] - conj Z[M-k]) / (2i),
// w = exp(-2 pi i / 2M), k in [0, M].
// Z is in the digit-reversed layout of fft_dif (perm maps frequency -> point).
__device__ __forceinline__ float2 r2c_post(const float2* Z, const int* __restrict__ perm, int M,
                                           int k, const float2* __restrict__ twn) {
  const float2 zk = Z[__ldg(perm + (k == M ? 0 : k))];
  const float2 zc = conjf2(Z[__ldg(perm + (k == 0 ? 0 : M - k))]);
  const float2 xe = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
  const float2 d = make_float2(0.5f * (zk.x - zc.x), 0.5f * (zk.y - zc.y));
  const float2 xo = mul_mi(d);
  const float2 w = (k == M) ? make_float2(-1.f, 0.f) : __ldg(twn + k);
  return cadd(xe, cmul(w, xo));
}

// Pre-processing of a length-2M real inverse transform from bins X[0..M]:
//   Z[k] = (X[k] + conj X[M-k]) + i w^-k (X[k] - conj X[M-k]),  k in [0, M)
// so that the unnormalised inverse complex FFT of Z gives
// z[m] = x[2m] + i x[2m+1] of the unnormalised real inverse. The imaginary
// parts of the DC and Nyquist bins are ignored (cufftExecC2R / numpy irfft).
// c2r_pre_w takes a = X[k], b = X[M-k] and the table value twn[k] as loaded.
__device__ __forceinline__ float2 c2r_pre_w(float2 a, float2 b, float2 twk) {
  const float2 bc = conjf2(b);
  const float2 e = cadd(a, bc);
  const float2 d = csub(a, bc);
  return cadd(e, mul_pi(cmul(conjf2(twk), d)));
}

__device__ __forceinline__ float2 c2r_pre_vals(float2 a, float2 b, int k,
                                               const float2* __restrict__ twn) {
  return c2r_pre_w(a, b, __ldg(twn + k));
}

__device__ __forceinline__ float2 c2r_pre(const float2* __restrict__ X, int M, int k,
                                          const float2* __restrict__ twn) {
  float2 a = X[k];
  float2 b = X[M - k];
  if (k == 0) {
    a.y = 0.f;
    b.y = 0.f;
  }
  return c2r_pre_vals(a, b, k, twn);
}

}  // namespace fxc
