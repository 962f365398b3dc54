// Row transforms of any length inside one CTA.
//
// Lengths that factor into the radices of fft.cuh (2, 4, 8 and odd primes up
// to 31) run directly: the forward transform leaves the spectrum in the
// digit-reversed DIF layout and the inverse (DIT) reads it from there.
// Other lengths -- NCF lengths 2*half_cc+1 are often prime, e.g. 4001 for a
// 200 s lag at 10 Hz -- run as Bluestein's chirp-z transform: with
// w_k = exp(-i pi k^2 / n) the DFT is X_k = w_k * sum_j (x_j w_j) conj(w_{k-j}),
// a circular convolution evaluated with two transforms of a smooth length
// m >= 2n - 1 (a forward DIF, a pointwise product with the precomputed,
// digit-reversed spectrum of the chirp kernel, an inverse DIT). Bluestein
// spectra are in natural order. The inverse is the forward transform of the
// conjugate, conjugated.
#pragma once

#include "fft.cuh"

namespace fxc {

struct AnyPlan {
  FftPlan p;            // transform of length m (m == n when direct)
  int n;                // logical length
  const float2* chirp;  // Bluestein: w_k, k < n; null when direct
  const float2* khat;   // Bluestein: DFT_m(conj chirp kernel) / m at the DIF positions of p
  const int* iperm;     // direct: iperm[pos] = frequency held at point pos after fft_dif; null for Bluestein
};

// Complex elements of the row buffer the transforms need.
__host__ __device__ inline int any_buf_elems(const AnyPlan& a) { return a.p.n; }

// Position of frequency k in the layout any_forward leaves.
__device__ __forceinline__ int any_pos(const AnyPlan& a, int k) {
  return a.chirp ? k : __ldg(a.p.perm + k);
}

// SMOOTH: dispatch only the 7-smooth radices any_plan gives a Bluestein
// plan (less code per kernel; a kernel may keep the full dispatch where its
// register allocation came out better with it).
template <int T, bool SMOOTH = true>
__device__ void bluestein(float2* buf, const AnyPlan& a, const float2* stw, bool inverse) {
  const int n = a.n, m = a.p.n;
  for (int j = threadIdx.x; j < m; j += T) {
    float2 v = make_float2(0.f, 0.f);
    if (j < n) {
      float2 x = buf[j];
      if (inverse) x = conjf2(x);
      v = cmul(x, __ldg(a.chirp + j));
    }
    buf[j] = v;
  }
  __syncthreads();
  fft_dif<T, false, SMOOTH>(buf, a.p, stw, false);
  for (int j = threadIdx.x; j < m; j += T) buf[j] = cmul(buf[j], __ldg(a.khat + j));
  __syncthreads();
  fft_dit<T, false, SMOOTH>(buf, a.p, stw, true);
  for (int k = threadIdx.x; k < n; k += T) {
    const float2 y = cmul(buf[k], __ldg(a.chirp + k));
    buf[k] = inverse ? conjf2(y) : y;
  }
  __syncthreads();
}

// Forward DFT of buf[0, n) (natural order, CTA-synchronised); the result is
// at buf[any_pos(k)] and visible to the CTA on return.
template <int T, bool SMOOTH = true>
__device__ __forceinline__ void any_forward(float2* buf, const AnyPlan& a, const float2* stw) {
  if (a.chirp)
    bluestein<T, SMOOTH>(buf, a, stw, false);
  else
    fft_dif<T, false>(buf, a.p, stw, false);
}

// Unnormalised inverse from the any_forward layout to natural order.
template <int T, bool SMOOTH = true>
__device__ __forceinline__ void any_inverse(float2* buf, const AnyPlan& a, const float2* stw) {
  if (a.chirp)
    bluestein<T, SMOOTH>(buf, a, stw, true);
  else
    fft_dit<T, false>(buf, a.p, stw, true);
}

// Host: plans without composite radices (the row kernels dispatch only the
// prime radices and 2, 4, 8). Direct plan when n factors into them and
// n <= direct_max, else Bluestein over the smallest 2-3-5-7-smooth m >= 2n-1
// (m <= bluestein_max). Tables are cached per device and length.
int any_plan(int n, int direct_max, int bluestein_max, AnyPlan* out);

}  // namespace fxc
