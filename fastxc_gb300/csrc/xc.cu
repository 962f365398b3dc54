// xc_fast hot path: per-pair conjugate spectral product stacked over windows,
// then the inverse real FFT and the +-max_lag cut.
//
// Reference behaviour reproduced here:
//   accumulateStepXc2DKernel    native/xc/kernels/cuda.kernels.cu:16-36
//   per-step launch loop        native/xc/worker/async_workers.cu:61-83
//   finalize_xc_batch           native/xc/worker/executor.cu:6-55
//   finalize_shape              native/xc/io/input.cu:1033-1054
//
// GB300 design:
//   * the reference launches one kernel per window and read-modify-writes the
//     whole [pair][freq] stack in HBM each time; here one launch keeps the
//     stack of a register tile of 8 x 8 pairs in registers across all windows
//     and writes each stacked bin once;
//   * pairs are grouped into 16 x 16 channel tiles so every loaded spectrum
//     value feeds 8 pairs from registers (2 flop per loaded byte);
//   * the finalize kernel fuses the (-1)^f phase shift (folded into the lag
//     index), the C2R transform, the 1/(nfft*dt) scaling and the lag cut:
//     one CTA per pair, the half-length complex row in shared memory, only
//     cc_size samples written back.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

// The finalize's FFT stages run inline (no ABI save/restore of live
// registers around each stage: 2.20 -> 2.09 ms for 18 144 pairs).
#define FXC_FFT_STAGE_ATTR __forceinline__
#include "context.cuh"
#include "fft.cuh"
#include "fft_launch.cuh"
#include "xc.cuh"

namespace fxc {

// ---------------------------------------------------------------------------
// Pair plan
// ---------------------------------------------------------------------------

int pairplan_build(const int32_t* src, const int32_t* rec, int64_t npairs, int32_t nchan,
                   std::vector<XcTile>* tiles, std::vector<int32_t>* maps) {
  tiles->clear();
  maps->clear();
  // (src_block, rec_block) -> tile index; a slot collision (a duplicate pair)
  // spills the pair into a further layer of tiles.
  std::vector<std::map<std::pair<int32_t, int32_t>, int32_t>> layers(1);
  for (int64_t p = 0; p < npairs; ++p) {
    const int32_t s = src[p], r = rec[p];
    if (s < 0 || s >= nchan || r < 0 || r >= nchan) {
      set_error("pair %lld has channel (%d,%d) outside [0,%d)", (long long)p, s, r, nchan);
      return FXC_ERR_INVALID;
    }
    const int32_t sb = s / kXcTile, rb = r / kXcTile;
    const int slot = (s % kXcTile) * kXcTile + (r % kXcTile);
    for (size_t layer = 0;; ++layer) {
      if (layer == layers.size()) layers.emplace_back();
      auto key = std::make_pair(sb, rb);
      auto it = layers[layer].find(key);
      int32_t t;
      if (it == layers[layer].end()) {
        t = (int32_t)tiles->size();
        layers[layer][key] = t;
        XcTile tile;
        tile.a_base = sb * kXcTile;
        tile.b_base = rb * kXcTile;
        tile.map_offset = t * kXcTile * kXcTile;
        tile.npairs = 0;
        tiles->push_back(tile);
        maps->insert(maps->end(), kXcTile * kXcTile, -1);
      } else {
        t = it->second;
      }
      int32_t& cell = (*maps)[(size_t)(*tiles)[t].map_offset + slot];
      if (cell < 0) {
        cell = (int32_t)p;
        (*tiles)[t].npairs++;
        break;
      }
    }
  }
  // Order tiles by (a_base, b_base) so consecutive CTAs share channels in L2.
  std::vector<int32_t> order(tiles->size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int32_t)i;
  std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
    const XcTile &a = (*tiles)[x], &b = (*tiles)[y];
    if (a.a_base != b.a_base) return a.a_base < b.a_base;
    return a.b_base < b.b_base;
  });
  std::vector<XcTile> t2(tiles->size());
  std::vector<int32_t> m2(maps->size());
  for (size_t i = 0; i < order.size(); ++i) {
    XcTile t = (*tiles)[order[i]];
    std::copy(maps->begin() + t.map_offset, maps->begin() + t.map_offset + kXcTile * kXcTile,
              m2.begin() + i * kXcTile * kXcTile);
    t.map_offset = (int32_t)(i * kXcTile * kXcTile);
    t2[i] = t;
  }
  tiles->swap(t2);
  maps->swap(m2);
  return FXC_OK;
}

// ---------------------------------------------------------------------------
// Plain FP32 stack kernel
// ---------------------------------------------------------------------------
// CTA = one 16x16 channel tile x kXcFreqChunk (64) consecutive bins.
// Windows stream through a ring of kXcSlots shared-memory window slots filled
// with cp.async (8-byte copies: any spectrum pitch works; invalid channels
// and bins past nspec are zero-filled by the copy itself). A slot is 32 rows
// (16 src channels, then 16 rec channels) x 64 bins of float2 (16 KB).
// Windows move in pairs: one barrier per pair, two pairs in flight.
// Thread (col = tid % 64, quadrant q = tid / 64) accumulates 8 src x 8 rec
// pairs of bin f0+col in registers: 512 FFMA per 32 shared loads per window
// pair.
// Window masks (when given) are staged as 32 bytes per slot, loaded one
// iteration before they are stored so the load latency is hidden.

constexpr int kXcSlots = 6;                                 // window slots (3 pairs)
constexpr int kXcSlotElems = 2 * kXcTile * kXcFreqChunk;    // 2048 float2 = 16 KB

__device__ __forceinline__ void cp_async8(uint32_t dst, const void* src, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src),
               "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// acc[i][j] += conj(a[i]) * b[j] = (ar*br + ai*bi) + i (ar*bi - ai*br).
// (Packed fma.rn.f32x2 was measured slower here than scalar FFMA.)
__device__ __forceinline__ void xc_cmac8x8(float2 (&acc)[8][8], const float2 (&a)[8],
                                           const float2 (&b)[8]) {
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      acc[i][j].x = fmaf(a[i].x, b[j].x, acc[i][j].x);
      acc[i][j].x = fmaf(a[i].y, b[j].y, acc[i][j].x);
      acc[i][j].y = fmaf(a[i].x, b[j].y, acc[i][j].y);
      acc[i][j].y = fmaf(-a[i].y, b[j].x, acc[i][j].y);
    }
}

template <bool MASK>
__global__ void __launch_bounds__(256, 1)
    k_xc_stack_plain(const float2* __restrict__ spec, int64_t nwin, int nchan, int nspec,
                     int64_t spec_pitch, const uint8_t* __restrict__ mask,
                     const XcTile* __restrict__ tiles, const int32_t* __restrict__ maps,
                     float scale, float2* __restrict__ stack, int64_t stack_pitch, int accumulate) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float2* sm = reinterpret_cast<float2*>(smraw);
  uint8_t* smask = smraw + sizeof(float2) * kXcSlots * kXcSlotElems;

  const XcTile tile = tiles[blockIdx.x];
  const int tid = threadIdx.x;
  const int col = tid & (kXcFreqChunk - 1);
  const int f0 = blockIdx.y * kXcFreqChunk;
  const bool colok = f0 + col < nspec;

  // copy rows of this thread: r = (tid >> 6) + 4k, k < 8
  const int r0 = tid >> 6;
  int chs[8];
  unsigned okbits = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int r = r0 + 4 * k;
    const int ch = (r < kXcTile) ? tile.a_base + r : tile.b_base + (r - kXcTile);
    chs[k] = ch;
    if (colok && ch < nchan) okbits |= 1u << k;
  }
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sm) + (uint32_t)(col * sizeof(float2));

  // Copy window w (zero-filled when w >= nwin) into its slot.
  auto issue = [&](int64_t w) {
    const int slot = (int)(w % kXcSlots);
    const uint32_t dst = sbase + (uint32_t)(slot * kXcSlotElems * sizeof(float2));
    const int64_t wrow = w * nchan;
    const bool wok = w < nwin;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int r = r0 + 4 * k;
      const bool ok = wok && ((okbits >> k) & 1u);
      const float2* src = ok ? spec + (wrow + chs[k]) * spec_pitch + f0 + col : spec;
      cp_async8(dst + (uint32_t)(r * kXcFreqChunk * sizeof(float2)), src, ok ? 8 : 0);
    }
  };

  // mask bytes: thread tid < 32 owns row tid of every slot
  const int mrow_ch = (tid < kXcTile) ? tile.a_base + tid : tile.b_base + (tid - kXcTile);
  const bool mown = MASK && tid < 2 * kXcTile;
  auto mask_at = [&](int64_t w) -> uint8_t {
    return (w < nwin && mrow_ch < nchan) ? __ldg(mask + w * nchan + mrow_ch) : (uint8_t)0;
  };

  const int64_t npair = (nwin + 1) / 2;
  // prologue: window pairs 0 and 1
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    issue(2 * p);
    issue(2 * p + 1);
    cp_async_commit();
  }
  uint8_t mp0 = 0, mp1 = 0;
  if (mown) {
    for (int w = 0; w < 4; ++w) smask[w * 2 * kXcTile + tid] = mask_at(w);
    mp0 = mask_at(4);
    mp1 = mask_at(5);
  }

  const int q = tid >> 6;
  const int qa = q & 1, qb = q >> 1;
  float2 acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = make_float2(0.f, 0.f);

  for (int64_t p = 0; p < npair; ++p) {
    const int64_t w = 2 * p;
    cp_async_wait<1>();  // pair p has landed (pair p+1 may be in flight)
    __syncthreads();     // ... for every thread; pair p-1's slots are free
    issue(w + 4);
    issue(w + 5);
    cp_async_commit();
    if (mown) {
      smask[(int)((w + 4) % kXcSlots) * 2 * kXcTile + tid] = mp0;
      smask[(int)((w + 5) % kXcSlots) * 2 * kXcTile + tid] = mp1;
      mp0 = mask_at(w + 6);
      mp1 = mask_at(w + 7);
    }
    const int s0 = (int)(w % kXcSlots);
    const int s1 = (int)((w + 1) % kXcSlots);
    const float2* st0 = sm + s0 * kXcSlotElems + col;
    const float2* st1 = sm + s1 * kXcSlotElems + col;
    float2 ya0[8], yb0[8], ya1[8], yb1[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      ya0[i] = st0[(qa * 8 + i) * kXcFreqChunk];
      yb0[i] = st0[(kXcTile + qb * 8 + i) * kXcFreqChunk];
      ya1[i] = st1[(qa * 8 + i) * kXcFreqChunk];
      yb1[i] = st1[(kXcTile + qb * 8 + i) * kXcFreqChunk];
    }
    if (MASK) {
      const uint8_t* mk0 = smask + s0 * 2 * kXcTile;
      const uint8_t* mk1 = smask + s1 * 2 * kXcTile;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if (mk0[qa * 8 + i] == 0) ya0[i] = make_float2(0.f, 0.f);
        if (mk0[kXcTile + qb * 8 + i] == 0) yb0[i] = make_float2(0.f, 0.f);
        if (mk1[qa * 8 + i] == 0) ya1[i] = make_float2(0.f, 0.f);
        if (mk1[kXcTile + qb * 8 + i] == 0) yb1[i] = make_float2(0.f, 0.f);
      }
    }
    xc_cmac8x8(acc, ya0, yb0);
    xc_cmac8x8(acc, ya1, yb1);
  }
  cp_async_wait<0>();

  if (!colok) return;
  const int f = f0 + col;
  const int32_t* map = maps + tile.map_offset;
  // per row of 8 pairs: the previous values (accumulate) are loaded together
  // before any store -- the pairs are distinct -- so a row costs one DRAM
  // round trip rather than eight
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int64_t off[8];
    float2 v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int32_t p = __ldg(map + (qa * 8 + i) * kXcTile + qb * 8 + j);
      off[j] = p >= 0 ? (int64_t)p * stack_pitch + f : -1;
      v[j] = make_float2(acc[i][j].x * scale, acc[i][j].y * scale);
    }
    if (accumulate) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float2 o = off[j] >= 0 ? __ldcg(stack + off[j]) : make_float2(0.f, 0.f);
        v[j].x += o.x;
        v[j].y += o.y;
      }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (off[j] >= 0) stack[off[j]] = v[j];
  }
}

// ---------------------------------------------------------------------------
// Finalize: (-1)^f shift, C2R(nfft), 1/(nfft*dt), lag cut
// ---------------------------------------------------------------------------
// out[j] = x[(nfft - half_cc + j) mod nfft] * inv_norm, where x is the
// unshifted C2R result; multiplying bin f by (-1)^f shifts the series by
// nfft/2, so the reference's cut start nfft/2 - half_cc lands here.
//
// The C2R runs as an M = nfft/2 point inverse complex DIF transform z[m] =
// x[2m] + i x[2m+1] of the pre-processed bins, without two of its passes
// over shared memory:
//   * the pre-processing (and the inverse transform's input conjugation) is
//     done on the loads of the first stage, which reads the bins from global
//     memory itself;
//   * the last stage is formed only at the complex points that hold kept
//     lags (cc_size/2 + 1 of M: 1 001 of 18 522 at nfft 37 044), each as one
//     R-term sum over its butterfly's inputs (fft_dif_last_point).
// The plan's radices run in ascending order, so the pruned stage is the
// largest.

// bin k of the C2R input: Z[k] from X[k], X[M-k] (imaginary parts of the
// DC and Nyquist bins ignored), conjugated for the inverse transform
struct C2rBinLoad {
  const float2* __restrict__ X;
  const float2* __restrict__ twn;
  int M;
  __device__ __forceinline__ float2 operator()(int k) const {
    float2 a = X[k], b = X[M - k];
    const float2 w = __ldg(twn + k);
    if (k == 0) {
      a.y = 0.f;
      b.y = 0.f;
    }
    return conjf2(c2r_pre_w(a, b, w));
  }
};

template <int T, int NMAX>
__global__ void __launch_bounds__(T, 1)
    k_xc_finalize(const float2* __restrict__ stack, int64_t stack_pitch, FftPlan p,
                  const float2* __restrict__ twn, int half_cc, int cc_size, float inv_norm_f,
                  double inv_norm, float* __restrict__ ncf) {
  extern __shared__ float2 buf[];
  const int M = p.n;
  const int N = 2 * M;
  float2* stw = buf + M;
  fft_twiddles_to_smem<T>(p, stw);
  const C2rBinLoad load{stack + (int64_t)blockIdx.x * stack_pitch, twn, M};
  const int S = p.nstages;
  if (S >= 2) {
    __syncthreads();  // the twiddle table
    fft_dif_stage0_load<T>(buf, p, stw, load);
    fft_dif_inner<T>(buf, p, stw, 1, S - 1);
  } else {
    for (int k = threadIdx.x; k < M; k += T) buf[k] = load(k);
    __syncthreads();
  }
  // complex points k0 .. k0 + nq - 1 (mod M) hold the kept lags: point k
  // carries reals m = 2k (real part) and 2k + 1 (imaginary part)
  int m0 = N - half_cc;
  if (m0 >= N) m0 -= N;
  const int k0 = m0 >> 1;
  const int nq = ((m0 + cc_size - 1) >> 1) - k0 + 1;
  float* out = ncf + (int64_t)blockIdx.x * cc_size;
  for (int q = threadIdx.x; q < nq; q += T) {
    int k = k0 + q;
    if (k >= M) k -= M;
    // the inverse transform's output conjugation
    const float2 v = conjf2(fft_dif_last_point(buf, p, stw, k));
    const int j = 2 * (k0 + q) - m0;
    // InvNormalize2DKernel: float data times a double weight
    if (j >= 0 && j < cc_size) out[j] = (float)((double)v.x * inv_norm);
    if (j + 1 < cc_size) out[j + 1] = (float)((double)v.y * inv_norm);
  }
  (void)inv_norm_f;
}

// Finalize for nfft = N = 2M with M above the in-CTA limit and M/2 within
// it (e.g. nfft 74 088 at 20 Hz): the C2R runs, as in k_xc_finalize, as the
// M-point inverse of the folded spectrum Z (c2r_pre), x[2n] = Re z[n],
// x[2n+1] = Im z[n]; z is pruned to the lags kept. With k = k1 + 2 k2 and
// Q = M/2,
//   z[n] = Y_0[n mod Q] + exp(2 pi i n / M) Y_1[n mod Q],
//   Y_k1 = inverse DFT_Q of Z[k1 + 2 k2],
// two Q-point transforms in shared memory per pair (against P transforms of
// a full complex N-point split in k_xc_finalize_pruned: a quarter of the
// transform work).
template <int T>
__global__ void __launch_bounds__(T, 1)
    k_xc_finalize_half(const float2* __restrict__ stack, int64_t stack_pitch, FftPlan pq,
                       const float2* __restrict__ twn, int M, int half_cc, int cc_size, double inv_norm,
                       float* __restrict__ ncf) {
  extern __shared__ float2 buf[];
  const int Q = pq.n;
  const int N = 2 * M;
  // pq's twiddle table has stride N/Q = 4 over the N-point table, so stw
  // also serves exp(-2 pi i m / N) for the twiddle of Y_1
  float2* stw = buf + Q;
  float* acc = reinterpret_cast<float*>(stw + fft_tw_smem_elems(pq));
  fft_twiddles_to_smem<T>(pq, stw);
  const float2* X = stack + (int64_t)blockIdx.x * stack_pitch;
  for (int k1 = 0; k1 < 2; ++k1) {
    __syncthreads();
    for (int k2 = threadIdx.x; k2 < Q; k2 += T) buf[k2] = c2r_pre(X, M, k1 + 2 * k2, twn);
    __syncthreads();
    fft_dif<T>(buf, pq, stw, true);  // inverse DFT_Q, digit-reversed positions
    for (int j = threadIdx.x; j < cc_size; j += T) {
      int m = N - half_cc + j;
      if (m >= N) m -= N;
      const int n = m >> 1;
      float2 v = buf[__ldg(pq.perm + (n >= Q ? n - Q : n))];
      if (k1) v = cmul(v, conjf2(tw_lookup(stw, 2 * n)));  // exp(+2 pi i n / M)
      const float x = (m & 1) ? v.y : v.x;
      acc[j] = k1 ? acc[j] + x : x;
    }
  }
  float* out = ncf + (int64_t)blockIdx.x * cc_size;
  for (int j = threadIdx.x; j < cc_size; j += T) out[j] = (float)((double)acc[j] * inv_norm);
}

// Output-pruned finalize for any even nfft (also above the in-CTA FFT
// limit, e.g. nfft 74 088 at 20 Hz): only the cc_size lags of the cut are
// formed. With nfft = N = P*Q and k = k1 + P*k2,
//   x[n] = sum_k1 exp(2 pi i n k1 / N) * Y_k1[n mod Q],
//   Y_k1 = inverse DFT_Q of the decimated Hermitian spectrum S[k1 + P*k2],
// so a pair costs P length-Q transforms in shared memory plus P complex
// multiply-adds per kept lag; the real part is kept (C2R drops the
// imaginary parts of bins 0 and N/2 the same way). The lag sums live in
// shared memory (nothing is held in registers across the transforms).
template <int T>
__global__ void __launch_bounds__(T, 4)
    k_xc_finalize_pruned(const float2* __restrict__ stack, int64_t stack_pitch, FftPlan pq, int N,
                         int half_cc, int cc_size, double inv_norm, float* __restrict__ ncf) {
  extern __shared__ float2 sm[];
  const int Q = pq.n;
  const int P = N / Q;
  const int nspec = N / 2 + 1;
  // pq's twiddle table has stride N/Q over the N-point table, so stw also
  // serves exp(-2 pi i m / N) for the lag phases (tw_lookup(stw, m)).
  float2* buf = sm;
  float2* stw = buf + Q;
  float* acc = reinterpret_cast<float*>(stw + fft_tw_smem_elems(pq));
  fft_twiddles_to_smem<T>(pq, stw);
  for (int t = threadIdx.x; t < cc_size; t += T) acc[t] = 0.f;
  const float2* X = stack + (int64_t)blockIdx.x * stack_pitch;
  for (int k1 = 0; k1 < P; ++k1) {
    __syncthreads();
    for (int k2 = threadIdx.x; k2 < Q; k2 += T) {
      const int k = k1 + P * k2;
      float2 v;
      if (k < nspec) {
        v = X[k];
      } else {
        v = X[N - k];
        v.y = -v.y;
      }
      buf[k2] = v;
    }
    __syncthreads();
    fft_dif<T>(buf, pq, stw, true);  // inverse DFT_Q, digit-reversed positions
    // lag n = (N - half_cc + t) mod N of this thread's first t; from one t
    // to the next (t += T) n mod Q advances by T mod Q and n k1 mod N by
    // T k1 mod N, so no division is left in the loop
    int n = N - half_cc + (int)threadIdx.x;
    if (n >= N) n -= N;
    int m = (int)(((long long)n * k1) % N);
    int idx = n % Q;
    const int dm = (int)(((long long)T * k1) % N);
    const int di = T % Q;
    for (int t = threadIdx.x; t < cc_size; t += T) {
      const float2 y = buf[__ldg(pq.perm + idx)];
      const float2 w = tw_lookup(stw, m);
      acc[t] += y.x * w.x + y.y * w.y;  // Re(y * conj(w)), w = exp(-2 pi i m / N)
      m += dm;
      if (m >= N) m -= N;
      idx += di;
      if (idx >= Q) idx -= Q;
    }
  }
  __syncthreads();
  float* out = ncf + (int64_t)blockIdx.x * cc_size;
  for (int t = threadIdx.x; t < cc_size; t += T) out[t] = (float)((double)acc[t] * inv_norm);
}

// Divisor Q of N for the pruned finalize: minimises N log2 Q + cc_size N / Q
// (transform work + lag sums) over lengths the in-CTA FFT supports, with
// Q <= 8192 (64 KB of row buffer).
static int pruned_q(int N, int cc_size) {
  int best = 0;
  double best_cost = 0.0;
  for (int q = 2; q <= 8192 && q <= N; ++q) {
    if (N % q || !fft_length_supported(q)) continue;
    const double cost = (double)N * std::log2((double)q) + (double)cc_size * (double)(N / q) * 4.0;
    if (best == 0 || cost < best_cost) {
      best = q;
      best_cost = cost;
    }
  }
  return best;
}

static int xc_finalize_pruned_launch(fxc_ctx* ctx, const float2* stack, int64_t npairs,
                                     int64_t stack_pitch, const fxc_xc_shape* s, float* ncf) {
  constexpr int T = 256;
  const int N = s->nfft;
  const int Q = pruned_q(N, s->cc_size);
  FXC_CHECK_ARG(Q > 0, "nfft %d has no supported divisor for the pruned finalize", N);
  FXC_CHECK_ARG(s->cc_size <= 16384, "cc_size %d above 16384", s->cc_size);
  const float2* twn = nullptr;
  FXC_TRY(fft_twiddles(N, &twn));
  FftPlan pq;
  FXC_TRY(fft_make_plan(Q, twn, N / Q, &pq));
  const double inv_norm = 1.0 / (double)((float)N * s->dt);
  const size_t smem =
      sizeof(float2) * ((size_t)Q + fft_tw_smem_elems(pq)) + sizeof(float) * (size_t)s->cc_size;
  FXC_TRY(set_smem_limit(k_xc_finalize_pruned<T>, smem));
  k_xc_finalize_pruned<T><<<(unsigned)npairs, T, smem, ctx->stream>>>(stack, stack_pitch, pq, N, s->half_cc,
                                                                       s->cc_size, inv_norm, ncf);
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

int xc_stack_launch(fxc_ctx* ctx, const fxc_pairplan* plan, const float2* spec, int64_t nwin,
                    int nchan, int nspec, int64_t spec_pitch, const uint8_t* mask, float scale,
                    float2* stack, int64_t stack_pitch, int method, int accumulate) {
  if (plan->npairs == 0 || nspec == 0) return FXC_OK;
  if (method == FXC_XC_TENSOR) return xc_stack_tensor_launch(ctx, plan, spec, nwin, nchan, nspec,
                                                             spec_pitch, mask, scale, stack,
                                                             stack_pitch, accumulate);
  FXC_CHECK_ARG(method == FXC_XC_PLAIN, "unknown xc method %d", method);
  const int64_t nchunks = ceil_div(nspec, kXcFreqChunk);
  FXC_CHECK_ARG(nchunks <= 65535, "nspec %d too large for the grid", nspec);
  dim3 grid((unsigned)plan->ntiles, (unsigned)nchunks);
  const size_t smem = sizeof(float2) * kXcSlots * kXcSlotElems + kXcSlots * 2 * kXcTile;
  if (mask) {
    FXC_TRY(set_smem_limit(k_xc_stack_plain<true>, smem));
    k_xc_stack_plain<true><<<grid, 256, smem, ctx->stream>>>(spec, nwin, nchan, nspec, spec_pitch,
                                                             mask, plan->d_tiles, plan->d_maps,
                                                             scale, stack, stack_pitch, accumulate);
  } else {
    FXC_TRY(set_smem_limit(k_xc_stack_plain<false>, smem));
    k_xc_stack_plain<false><<<grid, 256, smem, ctx->stream>>>(spec, nwin, nchan, nspec, spec_pitch,
                                                              mask, plan->d_tiles, plan->d_maps,
                                                              scale, stack, stack_pitch, accumulate);
  }
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

// Lengths the one-CTA FFT also covers use the full transform unless
// FXC_FINALIZE=pruned selects the pruned form.
static bool xc_finalize_prefers_pruned(int N) {
  (void)N;
  const char* e = getenv("FXC_FINALIZE");
  return e && !strcmp(e, "pruned");
}

int xc_finalize_launch(fxc_ctx* ctx, const float2* stack, int64_t npairs, int64_t stack_pitch,
                       const fxc_xc_shape* s, float* ncf) {
  if (npairs == 0) return FXC_OK;
  const int N = s->nfft;
  FXC_CHECK_ARG(N % 2 == 0 && N >= 2, "nfft %d must be even", N);
  const int M = N / 2;
  FXC_CHECK_ARG(npairs <= 0x7fffffff, "too many pairs for one launch");
  if (M > kFftLargeNmax && !xc_finalize_prefers_pruned(N) && M % 2 == 0 && M / 2 <= kFftLargeNmax &&
      fft_length_supported(M / 2) && s->cc_size <= 16384) {
    const float2* twn = nullptr;
    FXC_TRY(fft_twiddles(N, &twn));
    FftPlan pq;
    FXC_TRY(fft_make_plan(M / 2, twn, 4, &pq));
    const double inv_norm = 1.0 / (double)((float)N * s->dt);
    const size_t smem = sizeof(float2) * ((size_t)(M / 2) + fft_tw_smem_elems(pq)) + sizeof(float) * (size_t)s->cc_size;
    FXC_TRY(set_smem_limit(k_xc_finalize_half<kFftLargeT>, smem));
    k_xc_finalize_half<kFftLargeT><<<(unsigned)npairs, kFftLargeT, smem, ctx->stream>>>(
        stack, stack_pitch, pq, twn, M, s->half_cc, s->cc_size, inv_norm, ncf);
    count_launch();
    FXC_LAUNCH_CHECK();
    return FXC_OK;
  }
  if (M > kFftLargeNmax || xc_finalize_prefers_pruned(N))
    return xc_finalize_pruned_launch(ctx, stack, npairs, stack_pitch, s, ncf);
  const float2* twn = nullptr;
  FXC_TRY(fft_twiddles(N, &twn));
  FftPlan p;
  FXC_TRY(fft_make_plan_ascending(M, twn, 2, &p));
  // 1/(width*dt) with width*dt in float, as InvNormalize2DKernel computes it
  const float wdt = (float)N * s->dt;
  const double inv_norm = 1.0 / (double)wdt;
  const size_t smem = sizeof(float2) * ((size_t)M + fft_tw_smem_elems(p));
  if (M <= kFftSmallNmax) {
    k_xc_finalize<kFftSmallT, kFftSmallNmax><<<(unsigned)npairs, kFftSmallT, smem, ctx->stream>>>(
        stack, stack_pitch, p, twn, s->half_cc, s->cc_size, (float)inv_norm, inv_norm, ncf);
  } else {
    FXC_TRY(set_smem_limit(k_xc_finalize<kFftLargeT, kFftLargeNmax>, smem));
    k_xc_finalize<kFftLargeT, kFftLargeNmax><<<(unsigned)npairs, kFftLargeT, smem, ctx->stream>>>(
        stack, stack_pitch, p, twn, s->half_cc, s->cc_size, (float)inv_norm, inv_norm, ncf);
  }
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

// Same launch as xc_finalize_launch, with the twiddle and digit-reversal
// tables supplied by the caller instead of the per-device table cache.
int xc_finalize_launch_tables(fxc_ctx* ctx, const float2* stack, int64_t npairs,
                              int64_t stack_pitch, const fxc_xc_shape* s, const float2* twn,
                              const int* perm, float* ncf) {
  if (npairs == 0) return FXC_OK;
  const int N = s->nfft;
  FXC_CHECK_ARG(N % 2 == 0 && N >= 2, "nfft %d must be even", N);
  const int M = N / 2;
  FXC_CHECK_ARG(M <= kFftLargeNmax, "nfft %d above the in-CTA FFT limit %d", N, 2 * kFftLargeNmax);
  FXC_CHECK_ARG(npairs <= 0x7fffffff, "too many pairs for one launch");
  FftPlan p;
  FXC_TRY(fft_make_plan_with(M, twn, 2, perm, &p));
  const float wdt = (float)N * s->dt;
  const double inv_norm = 1.0 / (double)wdt;
  const size_t smem = sizeof(float2) * ((size_t)M + fft_tw_smem_elems(p));
  if (M <= kFftSmallNmax) {
    k_xc_finalize<kFftSmallT, kFftSmallNmax><<<(unsigned)npairs, kFftSmallT, smem, ctx->stream>>>(
        stack, stack_pitch, p, twn, s->half_cc, s->cc_size, (float)inv_norm, inv_norm, ncf);
  } else {
    FXC_TRY(set_smem_limit(k_xc_finalize<kFftLargeT, kFftLargeNmax>, smem));
    k_xc_finalize<kFftLargeT, kFftLargeNmax><<<(unsigned)npairs, kFftLargeT, smem, ctx->stream>>>(
        stack, stack_pitch, p, twn, s->half_cc, s->cc_size, (float)inv_norm, inv_norm, ncf);
  }
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

int64_t xc_stack_pitch(int nspec) { return (int64_t)((nspec + 3) / 4) * 4; }

// dst[dst_rows[r]][c] (+)= src[src_rows[r]][c] for c < ncols float2 columns:
// folds one day's stack rows into the cross-day stack rows of their
// (path, component) groups
__global__ void __launch_bounds__(256)
    k_xc_rows_accumulate(const float2* __restrict__ src, int64_t src_pitch, const int64_t* __restrict__ src_rows,
                         const int64_t* __restrict__ dst_rows, int64_t nrows, float2* __restrict__ dst,
                         int64_t dst_pitch, int ncols, int assign) {
  for (int64_t r = blockIdx.y; r < nrows; r += gridDim.y) {
    const float2* s = src + src_rows[r] * src_pitch;
    float2* d = dst + dst_rows[r] * dst_pitch;
    for (int c = blockIdx.x * 256 + threadIdx.x; c < ncols; c += gridDim.x * 256) {
      const float2 a = __ldcs(s + c);
      if (assign) {
        d[c] = a;
      } else {
        float2 b = d[c];
        b.x += a.x;
        b.y += a.y;
        d[c] = b;
      }
    }
  }
}

}  // namespace fxc

using namespace fxc;

extern "C" {

int fxc_xc_shape_init(int32_t nspec, int32_t nstep, float dt, float cc_length, fxc_xc_shape* out) {
  clear_error();
  FXC_CHECK_ARG(out != nullptr, "out is null");
  FXC_CHECK_ARG(nspec >= 2 && nstep > 0 && dt > 0.0f && cc_length > 0.0f,
                "invalid shape nspec=%d nstep=%d dt=%g cc_length=%g", nspec, nstep, dt, cc_length);
  fxc_xc_shape s;
  s.nspec = nspec;
  s.nstep = nstep;
  s.dt = dt;
  s.nfft = 2 * (nspec - 1);
  s.half_cc = (int32_t)llround((double)cc_length / (double)dt);
  if (s.half_cc >= nspec) s.half_cc = nspec - 1;
  s.cc_size = 2 * s.half_cc + 1;
  FXC_CHECK_ARG(s.cc_size > 0 && s.cc_size <= s.nfft, "cc_size %d invalid for nfft %d", s.cc_size,
                s.nfft);
  *out = s;
  return FXC_OK;
}

int fxc_pairplan_create(fxc_ctx* ctx, const int32_t* h_src, const int32_t* h_rec, int64_t npairs,
                        int32_t nchan, fxc_pairplan** out) {
  clear_error();
  FXC_CHECK_ARG(out != nullptr, "out is null");
  *out = nullptr;
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(npairs >= 0 && nchan > 0, "npairs=%lld nchan=%d", (long long)npairs, nchan);
  FXC_CHECK_ARG(npairs == 0 || (h_src && h_rec), "null pair arrays");
  FXC_CHECK_ARG(npairs < 0x7fffffff, "npairs exceeds int32 range");
  std::vector<XcTile> tiles;
  std::vector<int32_t> maps;
  FXC_TRY(pairplan_build(h_src, h_rec, npairs, nchan, &tiles, &maps));
  fxc_pairplan* p = new (std::nothrow) fxc_pairplan();
  if (!p) {
    set_error("host allocation failed");
    return FXC_ERR_NOMEM;
  }
  p->device = ctx->device;
  p->npairs = npairs;
  p->nchan = nchan;
  p->ntiles = (int64_t)tiles.size();
  p->h_src.assign(h_src, h_src + npairs);
  p->h_rec.assign(h_rec, h_rec + npairs);
  if (!tiles.empty()) {
    cudaError_t e1 = cudaMalloc(&p->d_tiles, sizeof(XcTile) * tiles.size());
    cudaError_t e2 = cudaMalloc(&p->d_maps, sizeof(int32_t) * maps.size());
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
      (void)cudaGetLastError();
      fxc_pairplan_destroy(p);
      set_error("cudaMalloc of pair plan failed");
      return FXC_ERR_NOMEM;
    }
    cudaError_t e3 = cudaMemcpy(p->d_tiles, tiles.data(), sizeof(XcTile) * tiles.size(),
                                cudaMemcpyHostToDevice);
    cudaError_t e4 = cudaMemcpy(p->d_maps, maps.data(), sizeof(int32_t) * maps.size(),
                                cudaMemcpyHostToDevice);
    if (e3 != cudaSuccess || e4 != cudaSuccess) {
      fxc_pairplan_destroy(p);
      set_error("upload of pair plan failed: %s", cudaGetErrorString(e3 != cudaSuccess ? e3 : e4));
      return FXC_ERR_CUDA;
    }
  }
  FXC_TRY(xc_tensor_plan_init(ctx, p));
  *out = p;
  return FXC_OK;
}

int fxc_pairplan_destroy(fxc_pairplan* plan) {
  if (!plan) return FXC_OK;
  cudaSetDevice(plan->device);
  if (plan->d_tiles) cudaFree(plan->d_tiles);
  if (plan->d_maps) cudaFree(plan->d_maps);
  xc_tensor_plan_free(plan);
  delete plan;
  return FXC_OK;
}

int64_t fxc_pairplan_npairs(const fxc_pairplan* plan) { return plan ? plan->npairs : -1; }
int64_t fxc_pairplan_ntiles(const fxc_pairplan* plan) { return plan ? plan->ntiles : -1; }

int fxc_xc_stack(fxc_ctx* ctx, const fxc_pairplan* plan, const float* d_spec, int64_t nwin,
                 int32_t nchan, int32_t nspec, int64_t spec_pitch, const uint8_t* d_mask,
                 float scale, float* d_stack, int64_t stack_pitch, int method) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(plan != nullptr, "null pair plan");
  FXC_CHECK_ARG(nchan == plan->nchan, "nchan %d differs from the plan's %d", nchan, plan->nchan);
  FXC_CHECK_ARG(nwin >= 0 && nspec >= 1 && spec_pitch >= nspec && stack_pitch >= nspec,
                "invalid shape nwin=%lld nspec=%d spec_pitch=%lld stack_pitch=%lld",
                (long long)nwin, nspec, (long long)spec_pitch, (long long)stack_pitch);
  FXC_CHECK_ARG(plan->npairs == 0 || (d_spec && d_stack), "null data pointer");
  return xc_stack_launch(ctx, plan, reinterpret_cast<const float2*>(d_spec), nwin, nchan, nspec,
                         spec_pitch, d_mask, scale, reinterpret_cast<float2*>(d_stack), stack_pitch,
                         method);
}

int fxc_xc_finalize(fxc_ctx* ctx, const float* d_stack, int64_t npairs, int64_t stack_pitch,
                    const fxc_xc_shape* shape, float* d_ncf) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(shape != nullptr, "null shape");
  FXC_CHECK_ARG(npairs >= 0 && stack_pitch >= shape->nspec, "invalid npairs/pitch");
  FXC_CHECK_ARG(npairs == 0 || (d_stack && d_ncf), "null data pointer");
  FXC_CHECK_ARG(shape->nfft == 2 * (shape->nspec - 1) && shape->cc_size == 2 * shape->half_cc + 1,
                "inconsistent shape");
  return xc_finalize_launch(ctx, reinterpret_cast<const float2*>(d_stack), npairs, stack_pitch,
                            shape, d_ncf);
}

int fxc_xc_run(fxc_ctx* ctx, const fxc_pairplan* plan, const float* d_spec, int64_t nwin,
               int32_t nchan, int64_t spec_pitch, const uint8_t* d_mask, float scale,
               const fxc_xc_shape* shape, float* d_ncf, int method) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(plan != nullptr && shape != nullptr, "null plan or shape");
  if (plan->npairs == 0) return FXC_OK;
  if (method == FXC_XC_TENSOR && plan->tensor) {
    FXC_CHECK_ARG(nchan == plan->nchan && nwin >= 0 && spec_pitch >= shape->nspec && d_spec && d_ncf,
                  "invalid arguments");
    {
      // the fused pack + whole-bin contraction where the plan takes it
      const int64_t pitch = xc_stack_pitch(shape->nspec);
      FXC_TRY(ctx->scratch.reserve(sizeof(float2) * (size_t)pitch * (size_t)plan->npairs));
      float2* stack = reinterpret_cast<float2*>(ctx->scratch.ptr);
      const int rc = xc_gemm_f32_launch(ctx, plan, reinterpret_cast<const float2*>(d_spec), nwin, nchan,
                                        shape->nspec, spec_pitch, d_mask, 0, scale, stack, pitch, 0);
      if (rc == FXC_OK) return xc_finalize_launch(ctx, stack, plan->npairs, pitch, shape, d_ncf);
      if (rc != FXC_ERR_UNSUPPORTED) return rc;
      clear_error();
    }
    // pack, then contraction + finalize without a [pair][bin] stack
    const int64_t chunks = xc_packed_chunks(nchan, nwin, shape->nspec);
    if (chunks > 0) FXC_TRY(ctx->scratch3.reserve((size_t)chunks * 16));
    uint4* packed = reinterpret_cast<uint4*>(ctx->scratch3.ptr);
    FXC_TRY(xc_pack_launch(ctx, reinterpret_cast<const float2*>(d_spec), nwin, nchan, shape->nspec, spec_pitch,
                           d_mask, packed));
    return fxc_xc_stack_finalize_packed(ctx, plan, packed, nwin, shape->nspec, scale, shape, d_ncf);
  }
  const int64_t pitch = xc_stack_pitch(shape->nspec);
  FXC_TRY(ctx->scratch.reserve(sizeof(float2) * (size_t)pitch * (size_t)plan->npairs));
  float* stack = reinterpret_cast<float*>(ctx->scratch.ptr);
  FXC_TRY(fxc_xc_stack(ctx, plan, d_spec, nwin, nchan, shape->nspec, spec_pitch, d_mask, scale,
                       stack, pitch, method));
  return fxc_xc_finalize(ctx, stack, plan->npairs, pitch, shape, d_ncf);
}

int fxc_xc_rows_accumulate(fxc_ctx* ctx, const float* d_src, int64_t src_rows, int64_t src_pitch,
                           const int64_t* h_src_idx, const int64_t* h_dst_idx, int64_t nrows, float* d_dst,
                           int64_t dst_rows, int64_t dst_pitch, int32_t ncols, int32_t assign) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(nrows >= 0 && ncols >= 0 && src_pitch >= ncols && dst_pitch >= ncols, "invalid shape");
  if (nrows == 0 || ncols == 0) return FXC_OK;
  FXC_CHECK_ARG(d_src && h_src_idx && h_dst_idx && d_dst, "null pointer");
  // both index lists address their buffers; destination rows are distinct
  // within one call (the kernel adds without atomics)
  std::vector<int64_t> sorted(h_dst_idx, h_dst_idx + nrows);
  std::sort(sorted.begin(), sorted.end());
  FXC_CHECK_ARG(sorted.front() >= 0 && sorted.back() < dst_rows, "destination row outside [0, %lld)",
                (long long)dst_rows);
  FXC_CHECK_ARG(std::adjacent_find(sorted.begin(), sorted.end()) == sorted.end(),
                "destination rows repeat within one call");
  for (int64_t r = 0; r < nrows; ++r)
    FXC_CHECK_ARG(h_src_idx[r] >= 0 && h_src_idx[r] < src_rows, "source row %lld outside [0, %lld)",
                  (long long)h_src_idx[r], (long long)src_rows);
  const size_t bytes = sizeof(int64_t) * (size_t)nrows;
  const size_t off = (bytes + 255) & ~size_t(255);
  FXC_TRY(ctx->scratch2.reserve(off + bytes));
  int64_t* d_si = reinterpret_cast<int64_t*>(ctx->scratch2.ptr);
  int64_t* d_di = reinterpret_cast<int64_t*>(reinterpret_cast<char*>(ctx->scratch2.ptr) + off);
  FXC_CUDA_TRY(cudaMemcpyAsync(d_si, h_src_idx, bytes, cudaMemcpyHostToDevice, ctx->stream));
  FXC_CUDA_TRY(cudaMemcpyAsync(d_di, h_dst_idx, bytes, cudaMemcpyHostToDevice, ctx->stream));
  const dim3 g((unsigned)std::min<int64_t>((ncols + 255) / 256, 64), (unsigned)std::min<int64_t>(nrows, 65535));
  k_xc_rows_accumulate<<<g, 256, 0, ctx->stream>>>(reinterpret_cast<const float2*>(d_src), src_pitch, d_si, d_di,
                                                   nrows, reinterpret_cast<float2*>(d_dst), dst_pitch, ncols,
                                                   assign != 0);
  count_launch();
  FXC_LAUNCH_CHECK();
  // the index staging is reused by the next call on this context
  FXC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FXC_OK;
}

int fxc_ctx_host_phases(fxc_ctx* ctx, double* out_ms, int32_t n) {
  clear_error();
  FXC_CHECK_ARG(ctx != nullptr && out_ms != nullptr && n >= 0, "null context or output");
  for (int32_t i = 0; i < n; ++i) out_ms[i] = i < 6 ? ctx->host_phase_ms[i] : -1.0;
  return FXC_OK;
}

int fxc_xc_run_host(fxc_ctx* ctx, const fxc_pairplan* plan, const float* h_spec, int64_t nwin,
                    int32_t nchan, int64_t spec_pitch, const uint8_t* h_mask, float scale,
                    const fxc_xc_shape* shape, float* h_ncf, int method) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(plan != nullptr && shape != nullptr, "null plan or shape");
  FXC_CHECK_ARG(h_spec != nullptr && h_ncf != nullptr, "null host pointer");
  FXC_CHECK_ARG(method == FXC_XC_PLAIN || method == FXC_XC_TENSOR, "unknown xc method %d", method);
  if (plan->npairs == 0) return FXC_OK;
  // The windows stream through a ring of device buffers on a copy stream and
  // are consumed on the compute stream as they land, so the host-to-device
  // copy -- the bound of this call -- hides most of the compute:
  //   plain   each chunk is stacked into the running sum (the plain kernel's
  //           read-modify-write is coalesced along the bins);
  //   tensor  each chunk is packed as it lands and contracted into the
  //           running stack: chunk by chunk for the whole-bin contraction
  //           (it accumulates in its coalesced transpose), in groups of up
  //           to four chunks for the tiled one (a partial stack that a
  //           coalesced add folds in). The last chunk is a group of its own,
  //           so what follows the last copy is one chunk's contraction (the
  //           plain kernel's when it has at most 16 windows), the finalize
  //           and the last NCF block's copy back.
  const int nspec = shape->nspec;
  const int64_t wchunk = 64;  // windows per chunk (two 32-window K-blocks)
  const int64_t kShortTailWindows = 16;
  const int kRing = 3;
  const int64_t nchunks = (nwin + wchunk - 1) / wchunk;
  const bool tensor = method == FXC_XC_TENSOR;
  const size_t row_bytes = sizeof(float2) * (size_t)nchan * (size_t)spec_pitch;  // one window
  const size_t chunk_bytes = row_bytes * (size_t)wchunk;
  const size_t mask_bytes = h_mask ? (size_t)nwin * (size_t)nchan : 0;
  const size_t ncf_bytes = sizeof(float) * (size_t)plan->npairs * (size_t)shape->cc_size;
  const int64_t pitch = xc_stack_pitch(nspec);
  const size_t stack_bytes = sizeof(float2) * (size_t)pitch * (size_t)plan->npairs;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t off_mask = al(chunk_bytes) * kRing;
  const size_t off_ncf = off_mask + al(mask_bytes);
  FXC_TRY(ctx->scratch2.reserve(off_ncf + al(ncf_bytes)));
  char* base = reinterpret_cast<char*>(ctx->scratch2.ptr);
  FXC_TRY(ctx->scratch.reserve(stack_bytes));
  float2* stack = reinterpret_cast<float2*>(ctx->scratch.ptr);
  uint4* packed = nullptr;
  if (tensor) {
    FXC_CHECK_ARG(plan->tensor != nullptr, "pair plan has no tensor tiles");
    // one chunk's operands: every chunk is packed and contracted on its own,
    // the contraction accumulating into the stack through its transpose
    const int64_t chunks = xc_packed_chunks(nchan, std::min(nwin, wchunk), nspec);
    if (chunks > 0) FXC_TRY(ctx->scratch3.reserve((size_t)chunks * 16));
    packed = reinterpret_cast<uint4*>(ctx->scratch3.ptr);
  }
  if (!ctx->copy_stream) FXC_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
  cudaStream_t cs = ctx->copy_stream;
  // the copy stream starts after work already queued on the compute stream
  cudaEvent_t start_ev;
  FXC_CUDA_TRY(cudaEventCreateWithFlags(&start_ev, cudaEventDisableTiming));
  std::vector<cudaEvent_t> landed((size_t)kRing), used((size_t)kRing);
  for (int r = 0; r < kRing; ++r) {
    cudaEventCreateWithFlags(&landed[r], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&used[r], cudaEventDisableTiming);
  }
  int rc = FXC_OK;
  auto cuda_ok = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == FXC_OK) {
      set_error("CUDA error in the host-buffer xc pipeline: %s", cudaGetErrorString(e));
      rc = FXC_ERR_CUDA;
    }
    return rc == FXC_OK;
  };
  cuda_ok(cudaEventRecord(start_ev, ctx->stream));
  cuda_ok(cudaStreamWaitEvent(cs, start_ev, 0));
  // phase record (kernel timing on): timing events around every H2D copy
  // and every chunk's compute, read back once both streams are idle
  const bool phases = ctx->ktime_on;
  std::vector<cudaEvent_t> pev;
  auto mark = [&](cudaStream_t st) -> int {
    if (!phases) return -1;
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return -1;
    cudaEventRecord(e, st);
    pev.push_back(e);
    return (int)pev.size() - 1;
  };
  std::vector<int> copy_b, copy_e, comp_b, comp_e;
  const int ev_t0 = mark(ctx->stream);
  const uint8_t* d_mask = nullptr;
  if (h_mask) {
    cuda_ok(cudaMemcpyAsync(base + off_mask, h_mask, mask_bytes, cudaMemcpyHostToDevice, cs));
    d_mask = reinterpret_cast<const uint8_t*>(base + off_mask);
  }
  if (nchunks == 0)  // no windows: every stacked bin is zero
    cuda_ok(cudaMemset2DAsync(stack, sizeof(float2) * (size_t)pitch, 0, sizeof(float2) * (size_t)nspec,
                              (size_t)plan->npairs, ctx->stream));
  for (int64_t c = 0; c < nchunks && rc == FXC_OK; ++c) {
    const int r = (int)(c % kRing);
    const int64_t w0 = c * wchunk, nw = std::min(wchunk, nwin - w0);
    char* slot = base + al(chunk_bytes) * r;
    if (c >= kRing) cuda_ok(cudaStreamWaitEvent(cs, used[r], 0));  // slot consumed
    copy_b.push_back(mark(cs));
    cuda_ok(cudaMemcpyAsync(slot, reinterpret_cast<const char*>(h_spec) + row_bytes * (size_t)w0,
                            row_bytes * (size_t)nw, cudaMemcpyHostToDevice, cs));
    copy_e.push_back(mark(cs));
    cuda_ok(cudaEventRecord(landed[r], cs));
    cuda_ok(cudaStreamWaitEvent(ctx->stream, landed[r], 0));
    comp_b.push_back(mark(ctx->stream));
    if (rc != FXC_OK) break;
    const float2* spec = reinterpret_cast<const float2*>(slot);
    // a short last chunk (the remainder of nwin / 64) costs the contraction
    // mostly its fixed per-bin work; the plain kernel stacks it for less
    const bool short_tail = tensor && c > 0 && c == nchunks - 1 && nw <= kShortTailWindows;
    if (short_tail) {
      rc = xc_stack_launch(ctx, plan, spec, nw, nchan, nspec, spec_pitch, d_mask ? d_mask + (size_t)w0 * nchan : nullptr,
                           scale, stack, pitch, FXC_XC_PLAIN, 1);
      cuda_ok(cudaEventRecord(used[r], ctx->stream));
    } else if (tensor) {
      // the fused pack + contraction reads the slot itself; otherwise pack
      // the chunk (the slot is free again once packed: the GEMM reads the
      // packed copy), then contract it into the stack
      const uint8_t* cmask = d_mask ? d_mask + (size_t)w0 * nchan : nullptr;
      rc = xc_gemm_f32_launch(ctx, plan, spec, nw, nchan, nspec, spec_pitch, cmask, 0, scale, stack, pitch,
                              c > 0 ? 1 : 0);
      if (rc == FXC_ERR_UNSUPPORTED) {
        clear_error();
        rc = xc_pack_launch(ctx, spec, nw, nchan, nspec, spec_pitch, cmask, packed);
        cuda_ok(cudaEventRecord(used[r], ctx->stream));
        if (rc == FXC_OK) rc = xc_gemm_launch(ctx, plan, packed, nw, nspec, scale, stack, pitch, c > 0 ? 1 : 0);
      } else {
        cuda_ok(cudaEventRecord(used[r], ctx->stream));
      }
    } else {
      rc = xc_stack_launch(ctx, plan, spec, nw, nchan, nspec, spec_pitch, d_mask ? d_mask + (size_t)w0 * nchan : nullptr,
                           scale, stack, pitch, FXC_XC_PLAIN, c > 0);
      cuda_ok(cudaEventRecord(used[r], ctx->stream));
    }
    comp_e.push_back(mark(ctx->stream));
  }
  const int ev_fin0 = mark(ctx->stream);
  // finalize in pair blocks; each block's NCFs go back on the copy stream
  // while the next block is transformed
  float* d_ncf = reinterpret_cast<float*>(base + off_ncf);
  const int64_t nblk = std::min<int64_t>(4, plan->npairs);
  const int64_t per_blk = (plan->npairs + nblk - 1) / nblk;
  for (int64_t b = 0; b < nblk && rc == FXC_OK; ++b) {
    const int64_t p0 = b * per_blk, np = std::min(per_blk, plan->npairs - p0);
    if (np <= 0) break;
    const size_t off = (size_t)p0 * (size_t)shape->cc_size;
    rc = xc_finalize_launch(ctx, stack + (size_t)p0 * (size_t)pitch, np, pitch, shape, d_ncf + off);
    const int r = (int)(b % kRing);
    cuda_ok(cudaEventRecord(landed[r], ctx->stream));
    cuda_ok(cudaStreamWaitEvent(cs, landed[r], 0));
    cuda_ok(cudaMemcpyAsync(h_ncf + off, d_ncf + off, sizeof(float) * (size_t)np * (size_t)shape->cc_size,
                            cudaMemcpyDeviceToHost, cs));
  }
  const int ev_end_cs = mark(cs);
  cudaStreamSynchronize(cs);
  cudaStreamSynchronize(ctx->stream);
  if (phases) {
    for (double& v : ctx->host_phase_ms) v = -1.0;
    auto ms = [&](int a, int b) -> double {
      float t = 0.f;
      if (a < 0 || b < 0 || cudaEventElapsedTime(&t, pev[(size_t)a], pev[(size_t)b]) != cudaSuccess) return -1.0;
      return (double)t;
    };
    double copy_busy = 0.0, comp_busy = 0.0;
    for (size_t i = 0; i < copy_b.size() && i < copy_e.size(); ++i) copy_busy += std::max(0.0, ms(copy_b[i], copy_e[i]));
    for (size_t i = 0; i < comp_b.size() && i < comp_e.size(); ++i) comp_busy += std::max(0.0, ms(comp_b[i], comp_e[i]));
    const double total = ms(ev_t0, ev_end_cs);
    const double last_copy = copy_e.empty() ? 0.0 : ms(ev_t0, copy_e.back());
    ctx->host_phase_ms[0] = total;
    ctx->host_phase_ms[1] = copy_busy;
    ctx->host_phase_ms[2] = last_copy;
    ctx->host_phase_ms[3] = comp_busy;
    ctx->host_phase_ms[4] = total - last_copy;
    ctx->host_phase_ms[5] = ms(ev_fin0, ev_end_cs);
    (void)cudaGetLastError();
  }
  for (cudaEvent_t e : pev) cudaEventDestroy(e);
  cudaEventDestroy(start_ev);
  for (int r = 0; r < kRing; ++r) {
    cudaEventDestroy(landed[r]);
    cudaEventDestroy(used[r]);
  }
  FXC_TRY(rc);
  FXC_CUDA_TRY(cudaGetLastError());
  return ctx_check_device_error(ctx);
}

}  // extern "C"
