// Batched FFT entry points (one CTA per row, whole row in shared memory).
// They replace the cuFFT plans of the reference (cufftExecR2C / C2R / C2C)
// and are also the unit under test for the FFT library.
#include "context.cuh"
#include "fft.cuh"
#include "fft_launch.cuh"

namespace fxc {

template <int T, int NMAX>
__global__ void __launch_bounds__(T, 1)
    k_fft_c2c(const float2* __restrict__ in, float2* __restrict__ out, FftPlan p, int64_t in_pitch,
              int64_t out_pitch, int inverse) {
  extern __shared__ float2 buf[];
  const int n = p.n;
  float2* stw = buf + n;
  fft_twiddles_to_smem<T>(p, stw);
  const float2* x = in + (int64_t)blockIdx.x * in_pitch;
  for (int i = threadIdx.x; i < n; i += T) buf[i] = x[i];
  __syncthreads();
  fft_dif<T>(buf, p, stw, inverse != 0);
  float2* y = out + (int64_t)blockIdx.x * out_pitch;
  for (int i = threadIdx.x; i < n; i += T) y[i] = buf[__ldg(p.perm + i)];
}

// Real forward transform of even length 2M through a length-M complex FFT.
template <int T, int NMAX>
__global__ void __launch_bounds__(T, 1)
    k_fft_r2c_even(const float* __restrict__ in, float2* __restrict__ out, FftPlan p,
                   const float2* __restrict__ twn, int64_t in_pitch, int64_t out_pitch) {
  extern __shared__ float2 buf[];
  const int M = p.n;
  float2* stw = buf + M;
  fft_twiddles_to_smem<T>(p, stw);
  const float* x = in + (int64_t)blockIdx.x * in_pitch;
  for (int m = threadIdx.x; m < M; m += T) buf[m] = make_float2(x[2 * m], x[2 * m + 1]);
  __syncthreads();
  fft_dif<T>(buf, p, stw, false);
  float2* y = out + (int64_t)blockIdx.x * out_pitch;
  for (int k = threadIdx.x; k <= M; k += T) y[k] = r2c_post(buf, p.perm, M, k, twn);
}

// Real forward transform of odd length: complex FFT of the zero-imaginary row.
template <int T, int NMAX>
__global__ void __launch_bounds__(T, 1)
    k_fft_r2c_odd(const float* __restrict__ in, float2* __restrict__ out, FftPlan p,
                  int64_t in_pitch, int64_t out_pitch) {
  extern __shared__ float2 buf[];
  const int n = p.n;
  float2* stw = buf + n;
  fft_twiddles_to_smem<T>(p, stw);
  const float* x = in + (int64_t)blockIdx.x * in_pitch;
  for (int i = threadIdx.x; i < n; i += T) buf[i] = make_float2(x[i], 0.f);
  __syncthreads();
  fft_dif<T>(buf, p, stw, false);
  float2* y = out + (int64_t)blockIdx.x * out_pitch;
  for (int k = threadIdx.x; k <= n / 2; k += T) y[k] = buf[__ldg(p.perm + k)];
}

// Real inverse transform of even length 2M (unnormalised).
template <int T, int NMAX>
__global__ void __launch_bounds__(T, 1)
    k_fft_c2r_even(const float2* __restrict__ in, float* __restrict__ out, FftPlan p,
                   const float2* __restrict__ twn, int64_t in_pitch, int64_t out_pitch) {
  extern __shared__ float2 buf[];
  const int M = p.n;
  float2* stw = buf + M;
  fft_twiddles_to_smem<T>(p, stw);
  const float2* X = in + (int64_t)blockIdx.x * in_pitch;
  for (int k = threadIdx.x; k < M; k += T) buf[k] = c2r_pre(X, M, k, twn);
  __syncthreads();
  fft_dif<T>(buf, p, stw, true);
  float* y = out + (int64_t)blockIdx.x * out_pitch;
  for (int m = threadIdx.x; m < M; m += T) {
    float2 v = buf[__ldg(p.perm + m)];
    y[2 * m] = v.x;
    y[2 * m + 1] = v.y;
  }
}

static int check_common(fxc_ctx* ctx, const void* in, const void* out, int n, int batch) {
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(in != nullptr && out != nullptr, "null data pointer");
  FXC_CHECK_ARG(n >= 1, "transform length %d < 1", n);
  FXC_CHECK_ARG(batch >= 0 && batch <= (1 << 30), "batch %d out of range", batch);
  return FXC_OK;
}

}  // namespace fxc

using namespace fxc;

extern "C" {

int fxc_fft_supported(int n, int real_transform) {
  if (n < 1) return 0;
  int m = n;
  if (real_transform && n % 2 == 0) m = n / 2;
  if (m > kFftLargeNmax) return 0;
  return fft_length_supported(m) ? 1 : 0;
}

int fxc_fft_c2c(fxc_ctx* ctx, const float* d_in, float* d_out, int n, int batch, int64_t in_pitch,
                int64_t out_pitch, int inverse) {
  clear_error();
  FXC_TRY(check_common(ctx, d_in, d_out, n, batch));
  FXC_CHECK_ARG(in_pitch >= n && out_pitch >= n, "pitch smaller than n");
  FXC_CHECK_ARG(n <= kFftLargeNmax, "c2c length %d above the in-CTA limit %d", n, kFftLargeNmax);
  if (batch == 0) return FXC_OK;
  const float2* tw = nullptr;
  FXC_TRY(fft_twiddles(n, &tw));
  FftPlan p;
  FXC_TRY(fft_make_plan(n, tw, 1, &p));
  const size_t smem = sizeof(float2) * ((size_t)n + fft_tw_smem_elems(p));
  const float2* in = reinterpret_cast<const float2*>(d_in);
  float2* out = reinterpret_cast<float2*>(d_out);
  if (n <= kFftSmallNmax) {
    k_fft_c2c<kFftSmallT, kFftSmallNmax><<<batch, kFftSmallT, smem, ctx->stream>>>(
        in, out, p, in_pitch, out_pitch, inverse);
  } else {
    FXC_TRY(set_smem_limit(k_fft_c2c<kFftLargeT, kFftLargeNmax>, smem));
    k_fft_c2c<kFftLargeT, kFftLargeNmax><<<batch, kFftLargeT, smem, ctx->stream>>>(
        in, out, p, in_pitch, out_pitch, inverse);
  }
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

int fxc_fft_r2c(fxc_ctx* ctx, const float* d_in, float* d_out, int n, int batch, int64_t in_pitch,
                int64_t out_pitch) {
  clear_error();
  FXC_TRY(check_common(ctx, d_in, d_out, n, batch));
  FXC_CHECK_ARG(in_pitch >= n && out_pitch >= n / 2 + 1, "pitch too small");
  if (batch == 0) return FXC_OK;
  float2* out = reinterpret_cast<float2*>(d_out);
  const float2* twn = nullptr;
  FXC_TRY(fft_twiddles(n, &twn));
  if (n % 2 == 0) {
    const int M = n / 2;
    FXC_CHECK_ARG(M <= kFftLargeNmax, "r2c length %d above the in-CTA limit", n);
    FftPlan p;
    FXC_TRY(fft_make_plan(M, twn, 2, &p));
    const size_t smem = sizeof(float2) * ((size_t)M + fft_tw_smem_elems(p));
    if (M <= kFftSmallNmax) {
      k_fft_r2c_even<kFftSmallT, kFftSmallNmax><<<batch, kFftSmallT, smem, ctx->stream>>>(
          d_in, out, p, twn, in_pitch, out_pitch);
    } else {
      FXC_TRY(set_smem_limit(k_fft_r2c_even<kFftLargeT, kFftLargeNmax>, smem));
      k_fft_r2c_even<kFftLargeT, kFftLargeNmax><<<batch, kFftLargeT, smem, ctx->stream>>>(
          d_in, out, p, twn, in_pitch, out_pitch);
    }
  } else {
    FXC_CHECK_ARG(n <= kFftLargeNmax, "r2c odd length %d above the in-CTA limit", n);
    FftPlan p;
    FXC_TRY(fft_make_plan(n, twn, 1, &p));
    const size_t smem = sizeof(float2) * ((size_t)n + fft_tw_smem_elems(p));
    if (n <= kFftSmallNmax) {
      k_fft_r2c_odd<kFftSmallT, kFftSmallNmax><<<batch, kFftSmallT, smem, ctx->stream>>>(
          d_in, out, p, in_pitch, out_pitch);
    } else {
      FXC_TRY(set_smem_limit(k_fft_r2c_odd<kFftLargeT, kFftLargeNmax>, smem));
      k_fft_r2c_odd<kFftLargeT, kFftLargeNmax><<<batch, kFftLargeT, smem, ctx->stream>>>(
          d_in, out, p, in_pitch, out_pitch);
    }
  }
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

int fxc_fft_c2r(fxc_ctx* ctx, const float* d_in, float* d_out, int n, int batch, int64_t in_pitch,
                int64_t out_pitch) {
  clear_error();
  FXC_TRY(check_common(ctx, d_in, d_out, n, batch));
  FXC_CHECK_ARG(n % 2 == 0, "c2r length must be even (got %d)", n);
  FXC_CHECK_ARG(in_pitch >= n / 2 + 1 && out_pitch >= n, "pitch too small");
  if (batch == 0) return FXC_OK;
  const int M = n / 2;
  FXC_CHECK_ARG(M <= kFftLargeNmax, "c2r length %d above the in-CTA limit", n);
  const float2* twn = nullptr;
  FXC_TRY(fft_twiddles(n, &twn));
  FftPlan p;
  FXC_TRY(fft_make_plan(M, twn, 2, &p));
  const size_t smem = sizeof(float2) * ((size_t)M + fft_tw_smem_elems(p));
  const float2* in = reinterpret_cast<const float2*>(d_in);
  if (M <= kFftSmallNmax) {
    k_fft_c2r_even<kFftSmallT, kFftSmallNmax><<<batch, kFftSmallT, smem, ctx->stream>>>(
        in, d_out, p, twn, in_pitch, out_pitch);
  } else {
    FXC_TRY(set_smem_limit(k_fft_c2r_even<kFftLargeT, kFftLargeNmax>, smem));
    k_fft_c2r_even<kFftLargeT, kFftLargeNmax><<<batch, kFftLargeT, smem, ctx->stream>>>(
        in, d_out, p, twn, in_pitch, out_pitch);
  }
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

}  // extern "C"
