// ENZ -> RTZ rotation of nine-component NCF tensors.
//
// Reference: build_rotate_matrix / rotate_enz_to_rtz
// (fastxc/operators/rotation/python_rotate.py:33-105). A station pair's nine
// component NCFs (source E,N,Z x receiver E,N,Z, rows in the order E-E, E-N,
// E-Z, N-E, ..., Z-Z) become R-R, R-T, R-Z, T-R, ..., Z-Z through one 9 x 9
// matrix built from the pair's azimuth and back azimuth; per sample
// rtz[r] = sum_c M[r][c] * enz[c].
//
// GB300 design: the operation is a per-sample 9 x 9 mat-vec, 72 bytes of
// DRAM traffic per sample against 81 FMAs, so it is HBM-bound. One CTA
// column per pair chunk keeps the pair's matrix in shared memory; each
// thread rotates one sample of all nine components (nine coalesced loads,
// nine coalesced stores). Many pairs per launch amortise the launch.
#include <algorithm>
#include <cmath>

#include "context.cuh"

namespace fxc {
namespace {

constexpr int kRotT = 256;

__global__ void __launch_bounds__(kRotT)
    k_rotate_enz_rtz(const float* __restrict__ enz, int64_t npairs, int npts, int64_t pitch,
                     const float* __restrict__ mats, float* __restrict__ rtz) {
  __shared__ float m[81];
  for (int64_t p = blockIdx.y; p < npairs; p += gridDim.y) {
    __syncthreads();  // the previous pair's matrix is no longer read
    if (threadIdx.x < 81) m[threadIdx.x] = mats[p * 81 + threadIdx.x];
    __syncthreads();
    const float* in = enz + p * 9 * pitch;
    float* out = rtz + p * 9 * pitch;
    for (int t = blockIdx.x * kRotT + threadIdx.x; t < npts; t += gridDim.x * kRotT) {
      float x[9];
#pragma unroll
      for (int c = 0; c < 9; ++c) x[c] = __ldcs(in + c * pitch + t);
#pragma unroll
      for (int r = 0; r < 9; ++r) {
        float acc = 0.f;
#pragma unroll
        for (int c = 0; c < 9; ++c) acc = fmaf(m[r * 9 + c], x[c], acc);
        __stcs(out + r * pitch + t, acc);
      }
    }
  }
}

}  // namespace
}  // namespace fxc

using namespace fxc;

extern "C" {

int fxc_rotate_matrix(double azimuth_deg, double back_azimuth_deg, float* out81) {
  clear_error();
  FXC_CHECK_ARG(out81 != nullptr, "null output");
  // angles to float32 radians, then float32 sines/cosines and products, as
  // the reference does with numpy float32 scalars
  const float az = (float)(azimuth_deg * (M_PI / 180.0));
  const float baz = (float)(back_azimuth_deg * (M_PI / 180.0));
  const float sa = sinf(az), ca = cosf(az), sb = sinf(baz), cb = cosf(baz);
  for (int i = 0; i < 81; ++i) out81[i] = 0.f;
  float(*M)[9] = reinterpret_cast<float(*)[9]>(out81);
  // source side: R = E sin(az) + N cos(az), T = E cos(az) - N sin(az);
  // receiver side (radial from receiver back to source):
  // R = -E sin(baz) - N cos(baz), T = -E cos(baz) + N sin(baz); Z unchanged
  const float src[3][3] = {{sa, ca, 0.f}, {ca, -sa, 0.f}, {0.f, 0.f, 1.f}};
  const float rec[3][3] = {{-sb, -cb, 0.f}, {-cb, sb, 0.f}, {0.f, 0.f, 1.f}};
  // horizontal factors couple only horizontal components and Z only Z; a Z
  // factor (1) leaves the other factor unrounded
  auto linked = [](int i, int a) { return (i < 2 && a < 2) || (i == 2 && a == 2); };
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          if (!linked(i, a) || !linked(j, b)) continue;
          const float s = src[i][a], r = rec[j][b];
          M[i * 3 + j][a * 3 + b] = (i == 2) ? r : (j == 2) ? s : s * r;
        }
  return FXC_OK;
}

int fxc_rotate_enz_rtz(fxc_ctx* ctx, const float* d_enz, int64_t npairs, int32_t npts, int64_t pitch,
                       const float* d_mats, float* d_rtz) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(npairs >= 0 && npts > 0 && pitch >= npts, "invalid shape npairs=%lld npts=%d pitch=%lld",
                (long long)npairs, npts, (long long)pitch);
  if (npairs == 0) return FXC_OK;
  FXC_CHECK_ARG(d_enz && d_mats && d_rtz, "null pointer");
  const int gx = (npts + kRotT - 1) / kRotT;
  const unsigned gy = (unsigned)std::min<int64_t>(npairs, 65535);
  k_rotate_enz_rtz<<<dim3((unsigned)std::min(gx, 64), gy), kRotT, 0, ctx->stream>>>(d_enz, npairs, npts, pitch,
                                                                                     d_mats, d_rtz);
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

}  // extern "C"
