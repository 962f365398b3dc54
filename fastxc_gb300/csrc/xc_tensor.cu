// BF16 hi/lo split tensor-core contraction S(f) = Y(f)^H Y(f) on tcgen05.
//
// Same result as the plain stack kernel (and as accumulateStepXc2DKernel,
// native/xc/kernels/cuda.kernels.cu:16-36, summed over the windows):
//   stack[p, f] = scale * sum_w conj(Y[w, src_p, f]) * Y[w, rec_p, f]
// computed for all pairs of a 128 x N channel tile at once, per frequency,
// as real GEMMs over the window axis:
//   Re S = Yr_a . Yr_b + Yi_a . Yi_b        Im S = Yr_a . Yi_b - Yi_a . Yr_b
// Every real operand x is split into bf16 hi = rn(x), lo = rn(x - hi) and
// each product is hi.hi + hi.lo + lo.hi accumulated in FP32 in TMEM (the
// dropped lo.lo term is ~2^-16 relative).
//
// Pipeline:
//   1. k_xc_pack: complex64 [w][c][f] -> per frequency four bf16 planes
//      (re-hi, re-lo, im-hi, im-lo), each stored exactly as the UMMA
//      K-major, no-swizzle core-matrix image: for every K-block of 32
//      windows, 4 chunks of 8 windows, each chunk [C_pad rows][8 bf16]
//      (16 bytes per row). A row range of a chunk is one contiguous run, so
//      the GEMM moves its tiles with plain cp.async.bulk copies.
//   2. k_xc_tc_gemm: one CTA per (channel tile, frequency).
//        warp 0      producer: bulk copies of the A (128 src rows) and B (N
//                    rec rows) tiles of each K-block into a 2-stage ring,
//                    completion counted on mbarriers (expect_tx bytes);
//        warp 1      allocates 512 TMEM columns; lane 0 issues the 12
//                    tcgen05.mma (M=128, N, K=16) per K step into two FP32
//                    accumulators (Re at column 0, Im at column 256) and
//                    frees each stage with tcgen05.commit;
//        warps 2..9  epilogue: tcgen05.ld of the accumulators, scale,
//                    conjugate reversed pairs, scatter to the pair rows
//                    (two warps per TMEM lane quarter, alternate chunks).
//      Only the upper triangle of channel tiles is computed (a pair is
//      computed in the orientation (min, max) and conjugated if reversed).
//   Up to 192 channels k_xc_tc_gemm_bin computes a whole bin per CTA; its
//   F32 form fuses step 1: the epilogue warps, idle during the K loop,
//   gather the bin's FP32 values of each K-block, split them into the four
//   bf16 planes and store the core-matrix chunks into the operand ring
//   themselves, so the spectra are read once and no packed copy exists.
//      Every mbarrier wait is bounded by %globaltimer (2 s); a timeout sets
//      the context's device error word, the CTA drains its copies and frees
//      TMEM before it exits.
#include <algorithm>
#include <cstdlib>
#include <map>
#include <vector>

#include "context.cuh"
#include "fft_launch.cuh"
#include "xc.cuh"

namespace fxc {

constexpr int kTcKb = kTcKbWindows;   // windows per K-block (32)
constexpr int kTcKc = kTcKb / 8;      // 16-byte core-matrix chunks per K-block row
constexpr int kTcM = 128;             // MMA M (src channel rows per tile)
constexpr int kTcNmax = 256;          // MMA N limit (rec channel rows per tile)
constexpr int kTcStages = 2;
constexpr int kTcThreads = 320;       // 10 warps: producer, MMA, 8 epilogue
constexpr int kTcPlanes = 4;          // re-hi, re-lo, im-hi, im-lo
constexpr uint32_t kTcAccImCol = 256; // TMEM column of the Im accumulator
constexpr int kTcABytes = kTcPlanes * kTcM * kTcKb * 2;     // 32 KB per stage
constexpr int kTcBBytesMax = kTcPlanes * kTcNmax * kTcKb * 2;  // 64 KB per stage
constexpr int kTcStageBytes = kTcABytes + kTcBBytesMax;
constexpr size_t kTcSmemBytes = (size_t)kTcStages * kTcStageBytes + 256;
constexpr int64_t kBinMajorCap = int64_t(2) << 30;  // bin-major scratch of one tiled pass (bytes)

struct TcTile {
  int32_t a0, am;  // first src row, valid src rows (<= 128)
  int32_t b0, bn;  // first rec row, valid rec rows (<= n)
  int32_t n;       // MMA N: bn rounded up to 16
  int32_t map_offset;
};

struct XcTensorPlan {
  int32_t nchan = 0;
  int32_t cpad = 0;
  int64_t ntiles = 0;
  TcTile* d_tiles = nullptr;
  int32_t* d_maps = nullptr;  // per tile [128][n]: q, -(q+2) for a reversed pair, -1 none
  int32_t* d_perm = nullptr;  // perm[q] = pair index p of bin-major slot q
  std::vector<TcTile> h_tiles;
  int32_t layout = FXC_XC_LAYOUT_AUTO;  // contraction layout preference
};

static int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

int xc_tensor_plan_init(fxc_ctx*, fxc_pairplan* plan) {
  plan->tensor = nullptr;
  const int32_t C = plan->nchan;
  XcTensorPlan* tp = new (std::nothrow) XcTensorPlan();
  if (!tp) {
    set_error("host allocation failed");
    return FXC_ERR_NOMEM;
  }
  tp->nchan = C;
  tp->cpad = (int32_t)round_up(C, 8);
  // Tiles over the upper triangle: src block [a0, a0+128), rec range
  // [a0, C) in chunks of <= 256. Duplicated pairs go to extra layers.
  struct Geo {
    int32_t a0, am, b0, bn;
  };
  std::vector<Geo> geos;
  for (int32_t a0 = 0; a0 < C; a0 += kTcM) {
    const int32_t am = std::min(kTcM, C - a0);
    for (int32_t b0 = a0; b0 < C; b0 += kTcNmax) geos.push_back({a0, am, b0, std::min(kTcNmax, C - b0)});
  }
  auto geo_of = [&](int32_t lo, int32_t hi) -> int {
    const int32_t ablk = lo / kTcM;
    int idx = 0;
    for (int32_t a0 = 0; a0 < ablk * kTcM; a0 += kTcM) idx += (int)((C - a0 + kTcNmax - 1) / kTcNmax);
    return idx + (int)((hi - ablk * kTcM) / kTcNmax);
  };
  std::vector<TcTile> tiles;
  std::vector<int32_t> maps;
  std::vector<std::map<int, int>> layers(1);  // geo -> tile index
  for (int64_t p = 0; p < plan->npairs; ++p) {
    const int32_t s = plan->h_src[p], r = plan->h_rec[p];
    const int32_t lo = std::min(s, r), hi = std::max(s, r);
    const int g = geo_of(lo, hi);
    const Geo& G = geos[g];
    for (size_t layer = 0;; ++layer) {
      if (layer == layers.size()) layers.emplace_back();
      auto it = layers[layer].find(g);
      int t;
      if (it == layers[layer].end()) {
        t = (int)tiles.size();
        layers[layer][g] = t;
        TcTile tt;
        tt.a0 = G.a0;
        tt.am = G.am;
        tt.b0 = G.b0;
        tt.bn = G.bn;
        tt.n = (int32_t)round_up(G.bn, 16);
        tt.map_offset = (int32_t)maps.size();
        tiles.push_back(tt);
        maps.insert(maps.end(), (size_t)kTcM * tt.n, -1);
      } else {
        t = it->second;
      }
      int32_t& cell = maps[(size_t)tiles[t].map_offset + (size_t)(lo - G.a0) * tiles[t].n + (hi - G.b0)];
      if (cell == -1) {
        cell = (s <= r) ? (int32_t)p : (int32_t)(-(p + 2));
        break;
      }
    }
  }
  // Bin-major slots: the pairs of tile 0 first, then tile 1, ...; within a
  // tile column by column, rows in order. The contraction writes a tile's
  // values into one contiguous run of a bin's row (the 32 rows of a warp at
  // one column into consecutive slots), and the transpose puts slot q back
  // at pair perm[q].
  std::vector<int32_t> perm((size_t)plan->npairs, -1);
  int64_t q = 0;
  for (const TcTile& t : tiles)
    for (int32_t c = 0; c < t.n; ++c)
      for (int32_t r = 0; r < kTcM; ++r) {
        int32_t& cell = maps[(size_t)t.map_offset + (size_t)r * t.n + c];
        if (cell == -1) continue;
        const int32_t pi = cell >= 0 ? cell : -cell - 2;
        perm[(size_t)q] = pi;
        cell = cell >= 0 ? (int32_t)q : (int32_t)(-(q + 2));
        ++q;
      }
  if (q != plan->npairs) {
    delete tp;
    set_error("tensor tile plan places %lld of %lld pairs", (long long)q, (long long)plan->npairs);
    return FXC_ERR_INVALID;
  }
  tp->ntiles = (int64_t)tiles.size();
  tp->h_tiles = tiles;
  if (!tiles.empty()) {
    cudaError_t e1 = cudaMalloc(&tp->d_tiles, sizeof(TcTile) * tiles.size());
    cudaError_t e2 = cudaMalloc(&tp->d_maps, sizeof(int32_t) * maps.size());
    cudaError_t e2b = cudaMalloc(&tp->d_perm, sizeof(int32_t) * perm.size());
    if (e1 != cudaSuccess || e2 != cudaSuccess || e2b != cudaSuccess) {
      (void)cudaGetLastError();
      if (tp->d_tiles) cudaFree(tp->d_tiles);
      if (tp->d_maps) cudaFree(tp->d_maps);
      if (tp->d_perm) cudaFree(tp->d_perm);
      delete tp;
      set_error("cudaMalloc of tensor tile plan failed");
      return FXC_ERR_NOMEM;
    }
    cudaMemcpy(tp->d_tiles, tiles.data(), sizeof(TcTile) * tiles.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(tp->d_perm, perm.data(), sizeof(int32_t) * perm.size(), cudaMemcpyHostToDevice);
    cudaError_t e3 =
        cudaMemcpy(tp->d_maps, maps.data(), sizeof(int32_t) * maps.size(), cudaMemcpyHostToDevice);
    if (e3 != cudaSuccess) {
      cudaFree(tp->d_tiles);
      cudaFree(tp->d_maps);
      cudaFree(tp->d_perm);
      delete tp;
      set_error("upload of tensor tile plan failed: %s", cudaGetErrorString(e3));
      return FXC_ERR_CUDA;
    }
  }
  plan->tensor = tp;
  return FXC_OK;
}

void xc_tensor_plan_free(fxc_pairplan* plan) {
  if (!plan->tensor) return;
  if (plan->tensor->d_tiles) cudaFree(plan->tensor->d_tiles);
  if (plan->tensor->d_maps) cudaFree(plan->tensor->d_maps);
  if (plan->tensor->d_perm) cudaFree(plan->tensor->d_perm);
  delete plan->tensor;
  plan->tensor = nullptr;
}

// ---------------------------------------------------------------------------
// Pack kernel
// ---------------------------------------------------------------------------
// CTA: 16 frequencies x 16 channels x one K-block of 32 windows.
// Thread (c = tid / 16, f = tid % 16) loads its 32 windows with all loads in
// flight at once (each 16-thread group reads one 128-byte run), then every
// thread writes 16-byte chunks (8 windows of one plane, one row):
// consecutive threads write consecutive rows (256 contiguous bytes).

constexpr int kPackF = 16;
constexpr int kPackC = 16;
constexpr size_t kPackSmem = sizeof(float2) * kTcKb * kPackC * (kPackF + 1);

// Two floats -> packed bf16x2 (lo in bits 0-15), rounded to nearest even
// (the spectra are finite: the producing stage sanitises them).
__device__ __forceinline__ uint32_t bf16x2_rn(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}

__global__ void __launch_bounds__(256)
    k_xc_pack(const float2* __restrict__ spec, int64_t nwin, int nchan, int nspec,
              int64_t spec_pitch, const uint8_t* __restrict__ mask, int nkb, int cpad, int kb0,
              int64_t w_base, uint4* __restrict__ packed) {
  extern __shared__ float2 psm[];  // [kTcKb][kPackC][kPackF + 1]
  const int f0 = blockIdx.x * kPackF;
  const int c0 = blockIdx.y * kPackC;
  const int kb = kb0 + blockIdx.z;  // spec holds windows from w_base on
  const int tid = threadIdx.x;
  {
    const int f = tid % kPackF;
    const int c = tid / kPackF;
    const int ch = c0 + c;
    const bool okcf = ch < nchan && f0 + f < nspec;
    const int64_t w0 = (int64_t)kb * kTcKb;
    float2 v[kTcKb];
#pragma unroll
    for (int k = 0; k < kTcKb; ++k) {
      const int64_t w = w0 + k;
      bool ok = okcf && w < nwin;
      if (ok && mask) ok = __ldg(mask + w * nchan + ch) != 0;
      v[k] = ok ? __ldg(spec + ((w - w_base) * nchan + ch) * spec_pitch + f0 + f) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < kTcKb; ++k) psm[(k * kPackC + c) * (kPackF + 1) + f] = v[k];
  }
  __syncthreads();
  // write: item = (f, kc, row); thread computes the 4 planes of 8 windows
  for (int it = tid; it < kPackF * kTcKc * kPackC; it += 256) {
    const int row = it % kPackC;
    const int kc = (it / kPackC) % kTcKc;
    const int f = it / (kPackC * kTcKc);
    if (f0 + f >= nspec || c0 + row >= cpad) continue;
    uint32_t w_rh[4], w_rl[4], w_ih[4], w_il[4];
#pragma unroll
    for (int e2 = 0; e2 < 4; ++e2) {
      // windows 2 e2 (low half) and 2 e2 + 1 (high half): hi = bf16(x),
      // lo = bf16(x - hi)
      const float2 v0 = psm[((kc * 8 + e2 * 2) * kPackC + row) * (kPackF + 1) + f];
      const float2 v1 = psm[((kc * 8 + e2 * 2 + 1) * kPackC + row) * (kPackF + 1) + f];
      const uint32_t rh = bf16x2_rn(v0.x, v1.x);
      const uint32_t ih = bf16x2_rn(v0.y, v1.y);
      w_rh[e2] = rh;
      w_ih[e2] = ih;
      w_rl[e2] = bf16x2_rn(v0.x - __uint_as_float(rh << 16), v1.x - __uint_as_float(rh & 0xffff0000u));
      w_il[e2] = bf16x2_rn(v0.y - __uint_as_float(ih << 16), v1.y - __uint_as_float(ih & 0xffff0000u));
    }
    const int64_t fo = f0 + f;
    // chunk index of (f, plane, kb, kc) -> rows [0, cpad)
    const int64_t base = (((fo * kTcPlanes) * nkb + kb) * kTcKc + kc) * cpad + c0 + row;
    const int64_t plane_stride = (int64_t)nkb * kTcKc * cpad;
    packed[base + 0 * plane_stride] = make_uint4(w_rh[0], w_rh[1], w_rh[2], w_rh[3]);
    packed[base + 1 * plane_stride] = make_uint4(w_rl[0], w_rl[1], w_rl[2], w_rl[3]);
    packed[base + 2 * plane_stride] = make_uint4(w_ih[0], w_ih[1], w_ih[2], w_ih[3]);
    packed[base + 3 * plane_stride] = make_uint4(w_il[0], w_il[1], w_il[2], w_il[3]);
  }
}

// ---------------------------------------------------------------------------
// tcgen05 GEMM
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false after ~2 s without completion.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_try(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t i = 1;; ++i) {
    if (mbar_try(bar, parity)) return true;
    if ((i & 255u) == 0 && globaltimer() - t0 > 2000000000ull) return false;
  }
}

// Cluster forms: the shared::cluster address of `addr` in CTA `rank`, a
// 16-byte store and an mbarrier arrival there, and a bounded wait whose
// acquire covers arrivals released by other CTAs of the cluster.
__device__ __forceinline__ uint32_t cluster_addr(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}

__device__ __forceinline__ void st_cluster16(uint32_t addr, uint4 v) {
  asm volatile("st.shared::cluster.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z),
               "r"(v.w)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_cluster(uint32_t remote_bar) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(remote_bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_cluster(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_cluster(uint32_t bar, uint32_t parity) {
  if (mbar_try_cluster(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t i = 1;; ++i) {
    if (mbar_try_cluster(bar, parity)) return true;
    if ((i & 255u) == 0 && globaltimer() - t0 > 2000000000ull) return false;
  }
}

__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %cluster_ctarank;" : "=r"(r));
  return r;
}

// 16 accumulator columns of one TMEM row into a bin-major row: column j goes
// to slot q = mv[j] (conjugated for -(q + 2), skipped for -1).
__device__ __forceinline__ void store_slots16(float2* __restrict__ row, const int32_t* mv, const float* re,
                                              const float* im, float scale) {
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const int32_t v = mv[j];
    if (v == -1) continue;
    const bool rev = v < -1;
    row[rev ? -v - 2 : v] = make_float2(re[j] * scale, (rev ? -im[j] : im[j]) * scale);
  }
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// tcgen05 shared-memory descriptor, K-major, no swizzle:
// start>>4 [0,14), LBO>>4 [16,30) (K-direction core-matrix stride),
// SBO>>4 [32,46) (M/N-direction 8-row stride), version 1 at [46,48).
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A bf16 (7-9 = 1),
// B bf16 (10-12 = 1), negate A (13), K-major A/B (15,16 = 0), N>>3 at 17,
// M>>4 at 24.
__host__ __device__ constexpr uint32_t umma_idesc(int m, int n, bool neg_a) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((neg_a ? 1u : 0u) << 13) |
         ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Ties 16 registers that a tcgen05.ld fills asynchronously to this point:
// placed after tcgen05.wait::ld, it keeps the compiler from moving their
// first use above the wait (the load's outputs are otherwise ordinary
// register values to it).
__device__ __forceinline__ void reg_fence16(float (&v)[16]) {
  asm volatile(""
               : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7]),
                 "+f"(v[8]), "+f"(v[9]), "+f"(v[10]), "+f"(v[11]), "+f"(v[12]), "+f"(v[13]), "+f"(v[14]),
                 "+f"(v[15])
               :
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Output: bin-major rows, binmajor[f * bin_pitch + q] for the plan's slots
// q (each tile owns one contiguous run of slots, column-major, so the 32
// rows of a warp store one column into consecutive slots).
// Persistent: CTA c runs the (bin, tile) items c, c + G, c + 2G, ... of
// total = nspec * ntiles, numbered bin-major, so the G CTAs at work at any
// time hold consecutive items: the tiles of a few adjacent bins, whose
// operand rows are shared in L2. TMEM, the
// barriers and the operand ring live across items: the producer loads the
// next item's K-blocks while the current item's epilogue runs, and the MMAs
// of an item start once the epilogue of the previous one has drained the
// accumulators (tmem_empty, one arrival per epilogue warp). Rows of a stage
// past a tile's valid rows hold stale data; they only reach accumulator rows
// (>= am) and columns (>= bn) that the epilogue never stores.
__global__ void __launch_bounds__(kTcThreads, 1)
    k_xc_tc_gemm(const uint4* __restrict__ packed, int nkb, int cpad,
                 const TcTile* __restrict__ tiles, int ntiles, const int32_t* __restrict__ maps, int nspec,
                 float scale, float2* __restrict__ binmajor, int64_t bin_pitch, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* stage_base = smem;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)kTcStages * kTcStageBytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 8);
  const uint32_t bar_full0 = smem_u32(bars + 0);
  const uint32_t bar_empty0 = smem_u32(bars + 2);
  const uint32_t bar_acc = smem_u32(bars + 4);
  const uint32_t bar_tfree = smem_u32(bars + 5);
  const uint32_t bar_drain = smem_u32(bars + 6);

  const int64_t total = (int64_t)ntiles * nspec;
  const int64_t G = gridDim.x;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const uint32_t a_plane_bytes = (uint32_t)kTcM * kTcKb * 2;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kTcStages; ++s) {
      mbar_init(bar_full0 + 8 * s, 1);
      mbar_init(bar_empty0 + 8 * s, 1);
    }
    mbar_init(bar_acc, 1);
    mbar_init(bar_tfree, 8);
    mbar_init(bar_drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int64_t q = 0;  // K-blocks issued
      bool failed = false;
      for (int64_t i = blockIdx.x; i < total && !failed; i += G) {
        const int f = (int)(i / ntiles);
        const TcTile tile = tiles[i % ntiles];
        const uint32_t b_plane_bytes = (uint32_t)tile.n * kTcKb * 2;
        const uint32_t tx = (uint32_t)kTcPlanes * kTcKc * (uint32_t)(tile.am + tile.bn) * 16u;
        for (int kb = 0; kb < nkb; ++kb, ++q) {
          const int s = (int)(q % kTcStages);
          const uint32_t ph = (uint32_t)(q / kTcStages) & 1u;
          if (!mbar_wait(bar_empty0 + 8 * s, ph ^ 1u)) {
            failed = true;
            break;
          }
          const uint32_t full = bar_full0 + 8 * s;
          mbar_expect_tx(full, tx);
          const uint32_t st = smem_u32(stage_base + (size_t)s * kTcStageBytes);
          for (int pl = 0; pl < kTcPlanes; ++pl) {
            const int64_t pbase = (((int64_t)f * kTcPlanes + pl) * nkb + kb) * kTcKc * cpad;
            for (int kc = 0; kc < kTcKc; ++kc) {
              const uint4* srcA = packed + pbase + (int64_t)kc * cpad + tile.a0;
              const uint4* srcB = packed + pbase + (int64_t)kc * cpad + tile.b0;
              bulk_g2s(st + pl * a_plane_bytes + kc * kTcM * 16, srcA, (uint32_t)tile.am * 16u, full);
              bulk_g2s(st + kTcABytes + pl * b_plane_bytes + kc * tile.n * 16, srcB, (uint32_t)tile.bn * 16u,
                       full);
            }
          }
        }
      }
      if (failed) {
        atomicExch(err, 1);
        // the copies of the last issued K-blocks may still be in flight
        for (int64_t r = q - 1; r >= 0 && r >= q - kTcStages; --r)
          (void)mbar_wait(bar_full0 + 8 * (int)(r % kTcStages), (uint32_t)(r / kTcStages) & 1u);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t acc_re = tmem, acc_im = tmem + kTcAccImCol;
      int64_t q = 0;
      bool failed = false;
      for (int64_t i = blockIdx.x, li = 0; i < total && !failed; i += G, ++li) {
        const TcTile tile = tiles[i % ntiles];
        const int n = tile.n;
        const uint32_t id_pos = umma_idesc(kTcM, n, false);
        const uint32_t id_neg = umma_idesc(kTcM, n, true);
        const uint32_t b_plane_bytes = (uint32_t)n * kTcKb * 2;
        const uint32_t a_lbo = kTcM * 16, b_lbo = (uint32_t)n * 16, sbo = 128;
        // the epilogue of the previous item has read the accumulators
        if (li > 0 && !mbar_wait(bar_tfree, (uint32_t)(li - 1) & 1u)) {
          failed = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        bool first = true;
        for (int kb = 0; kb < nkb; ++kb, ++q) {
          const int s = (int)(q % kTcStages);
          const uint32_t ph = (uint32_t)(q / kTcStages) & 1u;
          if (!mbar_wait(bar_full0 + 8 * s, ph)) {
            failed = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = smem_u32(stage_base + (size_t)s * kTcStageBytes);
          const uint32_t sa = st, sb = st + kTcABytes;
#pragma unroll
          for (int ks = 0; ks < kTcKc / 2; ++ks) {
            const uint32_t koff_a = ks * 2 * a_lbo, koff_b = ks * 2 * b_lbo;
            uint64_t A[4], B[4];
#pragma unroll
            for (int pl = 0; pl < 4; ++pl) {
              A[pl] = umma_desc(sa + pl * a_plane_bytes + koff_a, a_lbo, sbo);
              B[pl] = umma_desc(sb + pl * b_plane_bytes + koff_b, b_lbo, sbo);
            }
            const uint32_t acc = first ? 0u : 1u;
            // Re += re.re + im.im (hi.hi, hi.lo, lo.hi)
            umma_bf16(acc_re, A[0], B[0], id_pos, acc);
            umma_bf16(acc_re, A[0], B[1], id_pos, 1);
            umma_bf16(acc_re, A[1], B[0], id_pos, 1);
            umma_bf16(acc_re, A[2], B[2], id_pos, 1);
            umma_bf16(acc_re, A[2], B[3], id_pos, 1);
            umma_bf16(acc_re, A[3], B[2], id_pos, 1);
            // Im += re.im - im.re
            umma_bf16(acc_im, A[0], B[2], id_pos, acc);
            umma_bf16(acc_im, A[0], B[3], id_pos, 1);
            umma_bf16(acc_im, A[1], B[2], id_pos, 1);
            umma_bf16(acc_im, A[2], B[0], id_neg, 1);
            umma_bf16(acc_im, A[2], B[1], id_neg, 1);
            umma_bf16(acc_im, A[3], B[0], id_neg, 1);
            first = false;
          }
          umma_commit(bar_empty0 + 8 * s);  // stage free once these MMAs are done
        }
        if (!failed) umma_commit(bar_acc);  // this item's accumulators are complete
      }
      if (failed) atomicExch(err, 1);
      // every MMA issued has completed before TMEM is freed
      umma_commit(bar_drain);
      (void)mbar_wait(bar_drain, 0);
    }
  } else {
    // epilogue warps 2..9: TMEM lane quarter = warp % 4; the two warps of a
    // quarter take alternate 16-column chunks. The pair-map words of the next
    // chunk are fetched (16-byte loads) while the current chunk is stored.
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const int row = q * 32 + lane;  // src row within the tile
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
    for (int64_t i = blockIdx.x, li = 0; i < total; i += G, ++li) {
      const int64_t f = i / ntiles;
      const TcTile tile = tiles[i % ntiles];
      const int n = tile.n;
      const int4* map4 = reinterpret_cast<const int4*>(maps + tile.map_offset + (int64_t)row * n);
      const bool row_ok = row < tile.am;
      int4 mcur[4], mnxt[4];
      int c0 = 16 * half;
      if (row_ok && c0 < n) {
#pragma unroll
        for (int k = 0; k < 4; ++k) mcur[k] = __ldg(map4 + c0 / 4 + k);
      }
      if (!mbar_wait(bar_acc, (uint32_t)li & 1u)) {
        atomicExch(err, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (; c0 < n; c0 += 32) {
        const int c1 = c0 + 32;
        if (row_ok && c1 < n) {
#pragma unroll
          for (int k = 0; k < 4; ++k) mnxt[k] = __ldg(map4 + c1 / 4 + k);
        }
        float re[16], im[16];
        tmem_ld16(lane_base + (uint32_t)c0, re);
        tmem_ld16(lane_base + kTcAccImCol + (uint32_t)c0, im);
        tmem_ld_wait();
        if (row_ok)  // padding columns (b >= bn) hold -1
          store_slots16(binmajor + f * bin_pitch, reinterpret_cast<const int32_t*>(mcur), re, im, scale);
#pragma unroll
        for (int k = 0; k < 4; ++k) mcur[k] = mnxt[k];
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(bar_tfree);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Whole-bin GEMM for up to 192 channels
// ---------------------------------------------------------------------------
// When the channel count C <= 192 the upper triangle of one bin is at most
// two tiles: T0 = rows [0, 128) x cols [0, C) and T1 = rows [128, C) x cols
// [128, C). Their four FP32 accumulators (Re/Im, N0 + N1 <= 256 columns
// each) fill the 512 TMEM columns exactly, so one CTA computes the whole
// bin from ONE load of the bin's C rows per K-block: the stage buffer holds
// 256 rows per (plane, 8-window chunk) -- rows [C, 256) stay zero -- and
// the four operands are descriptors into it (A0 = rows 0..127, B0 = rows
// 0..N0-1, A1 = rows 128..255, B1 = rows 128..128+N1-1). Against one CTA
// per (tile, bin) this halves the operand traffic and pays the per-CTA
// setup and the epilogue once per bin.
constexpr int kBinRows = 256;
constexpr int kBinStages = 3;
constexpr int kBinStageBytes = kTcPlanes * kTcKc * kBinRows * 16;  // 64 KB
constexpr size_t kBinSmemBytes = (size_t)kBinStages * kBinStageBytes + 256;
static_assert(kBinSmemBytes <= 227 * 1024, "whole-bin ring exceeds shared memory");
// The fused form: operand chunks of 192 rows (48 KB stages; tile 1's A
// operand, rows 128..255, reads 64 rows into the next chunk -- or, for the
// last chunk, into 1 KB of slack -- which only reach accumulator rows the
// epilogue never stores), then a ring of 3 staging buffers for the FP32
// input, each half a K-block (16 windows) of one CTA's 48 rows x 4 bins.
constexpr int kBinRowsF = 192;
constexpr int kBinStageBytesF = kTcPlanes * kTcKc * kBinRowsF * 16;  // 48 KB
constexpr int kStagingOffF = kBinStages * kBinStageBytesF + 1024;
constexpr int kHalfBytesF = 16 * 2 * 48 * 16;  // [16 windows][2 bin pairs][48 rows][16 B]
constexpr int kStagingBufsF = 3;
constexpr size_t kBinSmemBytesF = (size_t)kStagingOffF + (size_t)kStagingBufsF * kHalfBytesF + 256;
static_assert(kBinSmemBytesF <= 227 * 1024, "fused whole-bin ring exceeds shared memory");

// Operand source of the whole-bin kernel when it reads the FP32 spectra
// itself (F32 = true): complex64 [w - w_base][c][pitch] with windows
// [0, nwin) of the call, and an optional [w][c] window mask.
struct BinSrc {
  const float2* spec;
  int64_t nwin, pitch, w_base;
  const uint8_t* mask;
  int nspec;
};
constexpr int kConvThreads = kTcThreads - 64;  // warps 2..9
constexpr int kBinCluster = 4;                 // bins (CTAs) per cluster of the fused form
// (row, 8-window chunk) units of one CTA's row quarter: 48 rows x 4 chunks
static_assert((192 / kBinCluster) * kTcKc <= kConvThreads, "one unit per converter thread");

// Eight windows of one complex value -> the four bf16 planes of one 16-byte
// core-matrix row: re-hi, re-lo, im-hi, im-lo (hi = rn(x), lo = rn(x - hi)).
__device__ __forceinline__ void split_bf16x8(const float2 (&v)[8], uint4 (&o)[4]) {
  uint32_t w_rh[4], w_rl[4], w_ih[4], w_il[4];
#pragma unroll
  for (int e2 = 0; e2 < 4; ++e2) {
    const float2 v0 = v[2 * e2], v1 = v[2 * e2 + 1];
    const uint32_t rh = bf16x2_rn(v0.x, v1.x);
    const uint32_t ih = bf16x2_rn(v0.y, v1.y);
    w_rh[e2] = rh;
    w_ih[e2] = ih;
    w_rl[e2] = bf16x2_rn(v0.x - __uint_as_float(rh << 16), v1.x - __uint_as_float(rh & 0xffff0000u));
    w_il[e2] = bf16x2_rn(v0.y - __uint_as_float(ih << 16), v1.y - __uint_as_float(ih & 0xffff0000u));
  }
  o[0] = make_uint4(w_rh[0], w_rh[1], w_rh[2], w_rh[3]);
  o[1] = make_uint4(w_rl[0], w_rl[1], w_rl[2], w_rl[3]);
  o[2] = make_uint4(w_ih[0], w_ih[1], w_ih[2], w_ih[3]);
  o[3] = make_uint4(w_il[0], w_il[1], w_il[2], w_il[3]);
}

// F32 = false: the operands come packed (k_xc_pack) and warp 0 moves them
// with bulk copies. F32 = true: the pack is fused in, and the kernel runs
// as clusters of 4 CTAs, one per bin of 4 consecutive bins (the 32 bytes of
// one (window, channel) row of the spectra: one DRAM sector). CTA r of a
// cluster loads rows [48 r, 48 r + 48) of all 4 bins, whole sectors, with
// its warps 2..9 (idle until the epilogue); splits them into the four bf16
// planes in registers and stores each bin's core-matrix chunks straight into
// the operand ring of that bin's CTA through distributed shared memory. So
// the spectra are read once, in full sectors, and no packed copy exists.
// Each converter warp then fences its writes for the async proxy and
// arrives on the stage's full barrier of all 4 CTAs (32 arrivals per
// stage); each CTA's MMA thread frees a stage in all 4 CTAs at once with a
// multicast tcgen05.commit (4 arrivals per empty barrier). Cluster barriers
// before the first remote access and before TMEM is released keep every
// CTA alive while its peers may still write to it.
template <bool F32>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_xc_tc_gemm_bin(const uint4* __restrict__ packed, BinSrc src, int nkb, int cpad, int nchan,
                     const TcTile* __restrict__ tiles, int ntiles, const int32_t* __restrict__ maps,
                     float scale, float2* __restrict__ binmajor, int64_t bin_pitch, int npairs,
                     int* __restrict__ err) {
  // Output: row f of the bin-major stack, binmajor[f * bin_pitch + p] for
  // p < npairs. Once every MMA has completed the operand stages are idle, so
  // the epilogue scatters the pairs into them by pair index and then writes
  // the row out in contiguous 16-byte stores (the [pair][bin] layout would
  // need one 8-byte store per pair, each in a sector of its own).
  constexpr int kRows = F32 ? kBinRowsF : kBinRows;
  constexpr int kStageBytes = F32 ? kBinStageBytesF : kBinStageBytes;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* stage_base = smem;
  uint64_t* bars = reinterpret_cast<uint64_t*>(
      smem + (F32 ? (size_t)kStagingOffF + (size_t)kStagingBufsF * kHalfBytesF : (size_t)kBinStages * kBinStageBytes));
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kBinStages + 1);
  int* epi_failed = reinterpret_cast<int*>(tmem_slot + 1);
  int* conv_ok = epi_failed + 1;
  const uint32_t bar_full0 = smem_u32(bars);
  const uint32_t bar_empty0 = smem_u32(bars + kBinStages);
  const uint32_t bar_acc = smem_u32(bars + 2 * kBinStages);
  const int f = blockIdx.x;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const TcTile t0 = tiles[0];
  const bool two = ntiles > 1;
  const int n0 = t0.n, n1 = two ? tiles[1].n : 0;
  const uint32_t chunk_bytes = (uint32_t)kRows * 16;  // one (plane, kc) chunk

  // zero the rows the copies never write (C .. rows) of every chunk once
  for (int s = 0; s < kBinStages; ++s) {
    uint4* st = reinterpret_cast<uint4*>(stage_base + (size_t)s * kStageBytes);
    const int per = kRows - nchan;
    for (int i = threadIdx.x; i < kTcPlanes * kTcKc * per; i += kTcThreads) {
      const int ch = i / per, r = nchan + i % per;
      st[(size_t)ch * kRows + r] = make_uint4(0, 0, 0, 0);
    }
  }
  if constexpr (F32) {
    // the slack past the last chunk (read by tile 1's A operand only)
    uint4* sl = reinterpret_cast<uint4*>(stage_base + (size_t)kBinStages * kStageBytes);
    for (int i = threadIdx.x; i < 1024 / 16; i += kTcThreads) sl[i] = make_uint4(0, 0, 0, 0);
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < kBinStages; ++s) {
      mbar_init(bar_full0 + 8 * s, F32 ? kBinCluster * (kConvThreads / 32) : 1);
      mbar_init(bar_empty0 + 8 * s, F32 ? kBinCluster : 1);
    }
    mbar_init(bar_acc, 1);
    *epi_failed = 0;
    *conv_ok = 1;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  // every CTA's barriers are initialised and its rows [C, 256) zeroed
  // before any peer writes into it
  if constexpr (F32) cluster_sync_all();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  // TMEM columns: T0 Re [0, n0), T0 Im [n0, 2 n0), T1 Re [2 n0, 2 n0 + n1), T1 Im after
  const uint32_t c_re0 = 0, c_im0 = (uint32_t)n0, c_re1 = 2u * n0, c_im1 = 2u * n0 + n1;

  if (warp == 0) {
    if (!F32 && lane == 0) {
      const uint32_t tx = (uint32_t)kTcPlanes * kTcKc * (uint32_t)nchan * 16u;
      int issued = 0;
      bool failed = false;
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % kBinStages;
        const uint32_t ph = (uint32_t)(kb / kBinStages) & 1u;
        if (!mbar_wait(bar_empty0 + 8 * s, ph ^ 1u)) {
          failed = true;
          break;
        }
        const uint32_t full = bar_full0 + 8 * s;
        mbar_expect_tx(full, tx);
        const uint32_t st = smem_u32(stage_base + (size_t)s * kBinStageBytes);
        for (int pl = 0; pl < kTcPlanes; ++pl) {
          const int64_t pbase = (((int64_t)f * kTcPlanes + pl) * nkb + kb) * kTcKc * cpad;
          for (int kc = 0; kc < kTcKc; ++kc)
            bulk_g2s(st + (pl * kTcKc + kc) * chunk_bytes, packed + pbase + (int64_t)kc * cpad,
                     (uint32_t)nchan * 16u, full);
        }
        ++issued;
      }
      if (failed) {
        atomicExch(err, 1);
        const int lo = issued > kBinStages ? issued - kBinStages : 0;
        for (int kb = lo; kb < issued; ++kb)
          (void)mbar_wait(bar_full0 + 8 * (kb % kBinStages), (uint32_t)(kb / kBinStages) & 1u);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idp0 = umma_idesc(kTcM, n0, false), idn0 = umma_idesc(kTcM, n0, true);
      const uint32_t idp1 = umma_idesc(kTcM, two ? n1 : 16, false), idn1 = umma_idesc(kTcM, two ? n1 : 16, true);
      const uint32_t lbo = kTcKc * chunk_bytes / kTcKc;  // next 8-window chunk of the same plane
      const uint32_t sbo = 128;
      bool failed = false;
      bool first = true;
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % kBinStages;
        const uint32_t ph = (uint32_t)(kb / kBinStages) & 1u;
        if (!(F32 ? mbar_wait_cluster(bar_full0 + 8 * s, ph) : mbar_wait(bar_full0 + 8 * s, ph))) {
          failed = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = smem_u32(stage_base + (size_t)s * kStageBytes);
#pragma unroll
        for (int ks = 0; ks < kTcKc / 2; ++ks) {
          uint64_t P0[4], P1[4];  // rows 0.. and rows 128.. of each plane at this K step
#pragma unroll
          for (int pl = 0; pl < 4; ++pl) {
            const uint32_t base = st + (pl * kTcKc + ks * 2) * chunk_bytes;
            P0[pl] = umma_desc(base, lbo, sbo);
            P1[pl] = umma_desc(base + kTcM * 16, lbo, sbo);
          }
          const uint32_t acc = first ? 0u : 1u;
          // tile 0: rows 0..127 x cols 0..n0-1
          umma_bf16(tmem + c_re0, P0[0], P0[0], idp0, acc);
          umma_bf16(tmem + c_re0, P0[0], P0[1], idp0, 1);
          umma_bf16(tmem + c_re0, P0[1], P0[0], idp0, 1);
          umma_bf16(tmem + c_re0, P0[2], P0[2], idp0, 1);
          umma_bf16(tmem + c_re0, P0[2], P0[3], idp0, 1);
          umma_bf16(tmem + c_re0, P0[3], P0[2], idp0, 1);
          umma_bf16(tmem + c_im0, P0[0], P0[2], idp0, acc);
          umma_bf16(tmem + c_im0, P0[0], P0[3], idp0, 1);
          umma_bf16(tmem + c_im0, P0[1], P0[2], idp0, 1);
          umma_bf16(tmem + c_im0, P0[2], P0[0], idn0, 1);
          umma_bf16(tmem + c_im0, P0[2], P0[1], idn0, 1);
          umma_bf16(tmem + c_im0, P0[3], P0[0], idn0, 1);
          if (two) {
            // tile 1: rows 128..255 (zero past C) x cols 128..128+n1-1
            umma_bf16(tmem + c_re1, P1[0], P1[0], idp1, acc);
            umma_bf16(tmem + c_re1, P1[0], P1[1], idp1, 1);
            umma_bf16(tmem + c_re1, P1[1], P1[0], idp1, 1);
            umma_bf16(tmem + c_re1, P1[2], P1[2], idp1, 1);
            umma_bf16(tmem + c_re1, P1[2], P1[3], idp1, 1);
            umma_bf16(tmem + c_re1, P1[3], P1[2], idp1, 1);
            umma_bf16(tmem + c_im1, P1[0], P1[2], idp1, acc);
            umma_bf16(tmem + c_im1, P1[0], P1[3], idp1, 1);
            umma_bf16(tmem + c_im1, P1[1], P1[2], idp1, 1);
            umma_bf16(tmem + c_im1, P1[2], P1[0], idn1, 1);
            umma_bf16(tmem + c_im1, P1[2], P1[1], idn1, 1);
            umma_bf16(tmem + c_im1, P1[3], P1[0], idn1, 1);
          }
          first = false;
        }
        if constexpr (F32) {
          // the stage is free in every CTA of the cluster once this CTA's
          // MMAs have read it: one arrival on each CTA's empty barrier
          asm volatile(
              "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::
                  "r"(bar_empty0 + 8 * s),
              "h"((uint16_t)((1u << kBinCluster) - 1))
              : "memory");
        } else {
          umma_commit(bar_empty0 + 8 * s);
        }
      }
      if (failed) atomicExch(err, 1);
      umma_commit(bar_acc);
    }
  } else {
    if constexpr (F32) {
      // operand producer for this CTA's row quarter of the cluster's 4 bins.
      // Half K-blocks (16 windows) stream into a ring of 3 staging buffers
      // by 16-byte cp.async copies issued two halves ahead, so their DRAM
      // latency overlaps the conversion of the half before; the layout
      // [window][bin pair][row][16 B] puts consecutive rows 16 bytes apart
      // for the conversion reads.
      const uint32_t rank = cluster_ctarank();
      const int f0 = f - (int)rank;
      const int q4 = (nchan + kBinCluster - 1) / kBinCluster;
      const int row0 = (int)rank * q4;
      const int nq = max(0, min(nchan, row0 + q4) - row0);
      const int t = threadIdx.x - 64;
      unsigned char* stg = smem + kStagingOffF;
      uint32_t stage_r[kBinCluster], full_r[kBinCluster];
#pragma unroll
      for (int b = 0; b < kBinCluster; ++b) {
        stage_r[b] = cluster_addr(smem_u32(stage_base), (uint32_t)b);
        full_r[b] = cluster_addr(bar_full0, (uint32_t)b);
      }
      const int nhalf = 2 * nkb;
      auto issue = [&](int h) {
        if (h < nhalf) {
          unsigned char* buf = stg + (h % kStagingBufsF) * kHalfBytesF;
          for (int i = t; i < 32 * nq; i += kConvThreads) {
            const int row = i % nq, rest = i / nq, pair = rest & 1, w16 = rest >> 1;
            const int64_t w = (int64_t)h * 16 + w16;
            unsigned char* d = buf + ((w16 * 2 + pair) * 48 + row) * 16;
            if (w < src.nwin) {
              const float2* g = src.spec + ((w - src.w_base) * nchan + row0 + row) * src.pitch + f0 + 2 * pair;
              asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(d)), "l"(g) : "memory");
            } else {
              *reinterpret_cast<uint4*>(d) = make_uint4(0, 0, 0, 0);  // windows past the call's last
            }
          }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
      };
      issue(0);
      issue(1);
      bool failed = false;
      for (int h = 0; h < nhalf; ++h) {
        issue(h + 2);  // into the buffer read at h - 1, released by that iteration's closing barrier
        asm volatile("cp.async.wait_group 2;" ::: "memory");  // this thread's copies of half h
        const int kb = h >> 1;
        const int s = kb % kBinStages;
        if ((h & 1) == 0 && t == 0)
          *conv_ok = mbar_wait_cluster(bar_empty0 + 8 * s, ((uint32_t)(kb / kBinStages) & 1u) ^ 1u) ? 1 : 0;
        // half h landed for every converter thread; the stage verdict is
        // the same for all of them, so all leave the loop together
        asm volatile("bar.sync 2, %0;" ::"n"(kConvThreads) : "memory");
        if (*conv_ok == 0) {
          failed = true;
          break;
        }
        const unsigned char* buf = stg + (h % kStagingBufsF) * kHalfBytesF;
        if (t < 4 * nq) {
          const int row = t % nq, rest = t / nq, pair = rest & 1, kcp = rest >> 1;
          float2 x0[8], x1[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            const float4 q = *reinterpret_cast<const float4*>(buf + (((kcp * 8 + e) * 2 + pair) * 48 + row) * 16);
            x0[e] = make_float2(q.x, q.y);
            x1[e] = make_float2(q.z, q.w);
          }
          const int b0 = 2 * pair;
          if (f0 + b0 >= src.nspec)
#pragma unroll
            for (int e = 0; e < 8; ++e) x0[e] = make_float2(0.f, 0.f);  // past the last bin
          if (f0 + b0 + 1 >= src.nspec)
#pragma unroll
            for (int e = 0; e < 8; ++e) x1[e] = make_float2(0.f, 0.f);
          uint4 o0[4], o1[4];
          split_bf16x8(x0, o0);
          split_bf16x8(x1, o1);
          const int kc = (h & 1) * 2 + kcp;
          const uint32_t off = (uint32_t)s * kStageBytes + (uint32_t)(kc * kRows + row0 + row) * 16;
#pragma unroll
          for (int pl = 0; pl < kTcPlanes; ++pl) {
            const uint32_t po = off + (uint32_t)(pl * kTcKc * kRows) * 16;
            st_cluster16(stage_r[b0] + po, o0[pl]);
            st_cluster16(stage_r[b0 + 1] + po, o1[pl]);
          }
        }
        if (h & 1) {
          // the K-block is complete in every CTA this thread wrote to
          asm volatile("fence.proxy.async.shared::cluster;" ::: "memory");
          __syncwarp();
          if (lane == 0) {
#pragma unroll
            for (int b = 0; b < kBinCluster; ++b) mbar_arrive_cluster(full_r[b] + 8 * s);
          }
        }
        asm volatile("bar.sync 2, %0;" ::"n"(kConvThreads) : "memory");  // buffer h free
      }
      asm volatile("cp.async.wait_all;" ::: "memory");
      if (failed) atomicExch(err, 1);
    }
    // epilogue: lane quarter q = warp % 4 holds rows q*32.. of both tiles;
    // the two warps of a quarter take alternate 16-column chunks of the
    // combined column space [0, n0) + [n0, n0 + n1)
    // Every epilogue thread reaches the named barrier below whether or not
    // its bounded wait succeeded; a failure anywhere skips the write-out.
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    float2* sout = reinterpret_cast<float2*>(stage_base);  // [npairs], stages idle after the last MMA
    const int ncols = n0 + n1;
    const int row = q * 32 + lane;
    const TcTile t1 = two ? tiles[1] : t0;
    // the pair map of a 16-column chunk (-1 where the row has no pair); the
    // next chunk's map is in flight while the current one is scattered, and
    // the first one while the MMAs run
    auto load_map = [&](int cc, int4 (&m)[4]) {
      const bool in1 = cc >= n0;
      const TcTile& tt = in1 ? t1 : t0;
      if (cc < ncols && row < tt.am) {
        const int4* m4 = reinterpret_cast<const int4*>(maps + tt.map_offset + (int64_t)row * (in1 ? n1 : n0) +
                                                       (in1 ? cc - n0 : cc));
#pragma unroll
        for (int v = 0; v < 4; ++v) m[v] = __ldg(m4 + v);
      } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) m[v] = make_int4(-1, -1, -1, -1);
      }
    };
    int4 mcur[4], mnext[4];
    load_map(16 * half, mcur);
    const bool ok = mbar_wait(bar_acc, 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok) {
      atomicExch(err, 1);
      atomicExch(epi_failed, 1);
    } else {
      const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
      for (int cc = 16 * half; cc < ncols; cc += 32) {
        load_map(cc + 32, mnext);
        const bool in1 = cc >= n0;  // warp-uniform
        const int c0 = in1 ? cc - n0 : cc;
        float re[16], im[16];
        tmem_ld16(lane_base + (in1 ? c_re1 : c_re0) + (uint32_t)c0, re);
        tmem_ld16(lane_base + (in1 ? c_im1 : c_im0) + (uint32_t)c0, im);
        tmem_ld_wait();
        const int32_t* mv = reinterpret_cast<const int32_t*>(mcur);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int32_t v = mv[j];
          if (v != -1) {
            const bool rev = v < -1;
            sout[rev ? -v - 2 : v] = make_float2(re[j] * scale, (rev ? -im[j] : im[j]) * scale);
          }
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) mcur[v] = mnext[v];
      }
    }
    asm volatile("bar.sync 1, %0;" ::"n"(kTcThreads - 64) : "memory");
    if (*epi_failed == 0 && (!F32 || f < src.nspec)) {
      // pairs [0, npairs) as float4 pairs; an odd count writes one padding
      // element of the row (bin_pitch is a multiple of 4)
      const float4* src4 = reinterpret_cast<const float4*>(sout);
      float4* dst4 = reinterpret_cast<float4*>(binmajor + (int64_t)f * bin_pitch);
      for (int i = threadIdx.x - 64; i < (npairs + 1) / 2; i += kTcThreads - 64) dst4[i] = src4[i];
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  // no CTA leaves while a peer may still store into it or arrive on it
  if constexpr (F32) cluster_sync_all();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

// Persistent form of the packed whole-bin contraction: one CTA per SM runs
// the bins blockIdx.x, blockIdx.x + G, ... with TMEM, the barriers and the
// operand ring kept across bins (the per-bin CTA pays a launch, the TMEM
// allocation, the ring's first loads and a smem-staged write-out, about a
// fifth of its time at 720 windows). The producer streams the next bin's
// K-blocks while the current bin's epilogue runs; the MMAs of a bin start
// once the eight epilogue warps have read the previous bin's accumulators
// (bar_tfree); the epilogue stores straight from registers by slot -- a
// warp's 32 rows of one column are consecutive slots -- so the ring is
// never borrowed for staging. Rows [C, 256) of every stage chunk are zeroed
// once and no copy writes them.
__global__ void __launch_bounds__(kTcThreads, 1)
    k_xc_tc_gemm_bin_p(const uint4* __restrict__ packed, int nspec, int nkb, int cpad, int nchan,
                       const TcTile* __restrict__ tiles, int ntiles, const int32_t* __restrict__ maps,
                       float scale, float2* __restrict__ binmajor, int64_t bin_pitch, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* stage_base = smem;
  // full[kBinStages], empty[kBinStages], acc, tfree, drain
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)kBinStages * kBinStageBytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kBinStages + 3);
  const uint32_t bar_full0 = smem_u32(bars);
  const uint32_t bar_empty0 = smem_u32(bars + kBinStages);
  const uint32_t bar_acc = smem_u32(bars + 2 * kBinStages);
  const uint32_t bar_tfree = smem_u32(bars + 2 * kBinStages + 1);
  const uint32_t bar_drain = smem_u32(bars + 2 * kBinStages + 2);
  const int G = (int)gridDim.x;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const TcTile t0 = tiles[0];
  const bool two = ntiles > 1;
  const TcTile t1 = two ? tiles[1] : t0;
  const int n0 = t0.n, n1 = two ? t1.n : 0;
  const uint32_t chunk_bytes = (uint32_t)kBinRows * 16;  // one (plane, kc) chunk

  for (int s = 0; s < kBinStages; ++s) {
    uint4* st = reinterpret_cast<uint4*>(stage_base + (size_t)s * kBinStageBytes);
    const int per = kBinRows - nchan;
    for (int i = threadIdx.x; i < kTcPlanes * kTcKc * per; i += kTcThreads) {
      const int ch = i / per, r = nchan + i % per;
      st[(size_t)ch * kBinRows + r] = make_uint4(0, 0, 0, 0);
    }
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < kBinStages; ++s) {
      mbar_init(bar_full0 + 8 * s, 1);
      mbar_init(bar_empty0 + 8 * s, 1);
    }
    mbar_init(bar_acc, 1);
    mbar_init(bar_tfree, 8);
    mbar_init(bar_drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  // TMEM columns: T0 Re [0, n0), T0 Im [n0, 2 n0), T1 Re [2 n0, 2 n0 + n1), T1 Im after
  const uint32_t c_re0 = 0, c_im0 = (uint32_t)n0, c_re1 = 2u * n0, c_im1 = 2u * n0 + n1;

  if (warp == 0) {
    if (lane == 0) {
      const uint32_t tx = (uint32_t)kTcPlanes * kTcKc * (uint32_t)nchan * 16u;
      int64_t q = 0;  // K-blocks issued
      bool failed = false;
      for (int f = blockIdx.x; f < nspec && !failed; f += G) {
        for (int kb = 0; kb < nkb; ++kb, ++q) {
          const int s = (int)(q % kBinStages);
          const uint32_t ph = (uint32_t)(q / kBinStages) & 1u;
          if (!mbar_wait(bar_empty0 + 8 * s, ph ^ 1u)) {
            failed = true;
            break;
          }
          const uint32_t full = bar_full0 + 8 * s;
          mbar_expect_tx(full, tx);
          const uint32_t st = smem_u32(stage_base + (size_t)s * kBinStageBytes);
          for (int pl = 0; pl < kTcPlanes; ++pl) {
            const int64_t pbase = (((int64_t)f * kTcPlanes + pl) * nkb + kb) * kTcKc * cpad;
            for (int kc = 0; kc < kTcKc; ++kc)
              bulk_g2s(st + (pl * kTcKc + kc) * chunk_bytes, packed + pbase + (int64_t)kc * cpad,
                       (uint32_t)nchan * 16u, full);
          }
        }
      }
      if (failed) {
        atomicExch(err, 1);
        // the copies of the last issued K-blocks may still be in flight
        for (int64_t r = q - 1; r >= 0 && r >= q - kBinStages; --r)
          (void)mbar_wait(bar_full0 + 8 * (int)(r % kBinStages), (uint32_t)(r / kBinStages) & 1u);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idp0 = umma_idesc(kTcM, n0, false), idn0 = umma_idesc(kTcM, n0, true);
      const uint32_t idp1 = umma_idesc(kTcM, two ? n1 : 16, false), idn1 = umma_idesc(kTcM, two ? n1 : 16, true);
      const uint32_t lbo = chunk_bytes;  // next 8-window chunk of the same plane
      const uint32_t sbo = 128;
      int64_t q = 0;
      bool failed = false;
      for (int f = blockIdx.x, li = 0; f < nspec && !failed; f += G, ++li) {
        // the epilogue has read the previous bin's accumulators
        if (li > 0 && !mbar_wait(bar_tfree, (uint32_t)(li - 1) & 1u)) {
          failed = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        bool first = true;
        for (int kb = 0; kb < nkb; ++kb, ++q) {
          const int s = (int)(q % kBinStages);
          const uint32_t ph = (uint32_t)(q / kBinStages) & 1u;
          if (!mbar_wait(bar_full0 + 8 * s, ph)) {
            failed = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = smem_u32(stage_base + (size_t)s * kBinStageBytes);
#pragma unroll
          for (int ks = 0; ks < kTcKc / 2; ++ks) {
            uint64_t P0[4], P1[4];  // rows 0.. and rows 128.. of each plane at this K step
#pragma unroll
            for (int pl = 0; pl < 4; ++pl) {
              const uint32_t base = st + (pl * kTcKc + ks * 2) * chunk_bytes;
              P0[pl] = umma_desc(base, lbo, sbo);
              P1[pl] = umma_desc(base + kTcM * 16, lbo, sbo);
            }
            const uint32_t acc = first ? 0u : 1u;
            // tile 0: rows 0..127 x cols 0..n0-1
            umma_bf16(tmem + c_re0, P0[0], P0[0], idp0, acc);
            umma_bf16(tmem + c_re0, P0[0], P0[1], idp0, 1);
            umma_bf16(tmem + c_re0, P0[1], P0[0], idp0, 1);
            umma_bf16(tmem + c_re0, P0[2], P0[2], idp0, 1);
            umma_bf16(tmem + c_re0, P0[2], P0[3], idp0, 1);
            umma_bf16(tmem + c_re0, P0[3], P0[2], idp0, 1);
            umma_bf16(tmem + c_im0, P0[0], P0[2], idp0, acc);
            umma_bf16(tmem + c_im0, P0[0], P0[3], idp0, 1);
            umma_bf16(tmem + c_im0, P0[1], P0[2], idp0, 1);
            umma_bf16(tmem + c_im0, P0[2], P0[0], idn0, 1);
            umma_bf16(tmem + c_im0, P0[2], P0[1], idn0, 1);
            umma_bf16(tmem + c_im0, P0[3], P0[0], idn0, 1);
            if (two) {
              // tile 1: rows 128..255 (zero past C) x cols 128..128+n1-1
              umma_bf16(tmem + c_re1, P1[0], P1[0], idp1, acc);
              umma_bf16(tmem + c_re1, P1[0], P1[1], idp1, 1);
              umma_bf16(tmem + c_re1, P1[1], P1[0], idp1, 1);
              umma_bf16(tmem + c_re1, P1[2], P1[2], idp1, 1);
              umma_bf16(tmem + c_re1, P1[2], P1[3], idp1, 1);
              umma_bf16(tmem + c_re1, P1[3], P1[2], idp1, 1);
              umma_bf16(tmem + c_im1, P1[0], P1[2], idp1, acc);
              umma_bf16(tmem + c_im1, P1[0], P1[3], idp1, 1);
              umma_bf16(tmem + c_im1, P1[1], P1[2], idp1, 1);
              umma_bf16(tmem + c_im1, P1[2], P1[0], idn1, 1);
              umma_bf16(tmem + c_im1, P1[2], P1[1], idn1, 1);
              umma_bf16(tmem + c_im1, P1[3], P1[0], idn1, 1);
            }
            first = false;
          }
          umma_commit(bar_empty0 + 8 * s);  // stage free once these MMAs are done
        }
        if (!failed) umma_commit(bar_acc);  // this bin's accumulators are complete
      }
      if (failed) atomicExch(err, 1);
      // every MMA issued has completed before TMEM is freed
      umma_commit(bar_drain);
      (void)mbar_wait(bar_drain, 0);
    }
  } else {
    // epilogue warps 2..9: lane quarter qq = warp % 4 holds rows qq*32.. of
    // both tiles; the two warps of a quarter take alternate 16-column chunks
    // of the combined column space [0, n0) + [n0, n0 + n1). The pair map of
    // the next chunk is fetched while the current one is stored.
    const int qq = warp & 3;
    const int half = (warp - 2) >> 2;
    const int ncols = n0 + n1;
    const int row = qq * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(qq * 32) << 16);
    auto load_map = [&](int cc, int4 (&m)[4]) {
      const bool in1 = cc >= n0;
      const TcTile& tt = in1 ? t1 : t0;
      if (cc < ncols && row < tt.am) {
        const int4* m4 = reinterpret_cast<const int4*>(maps + tt.map_offset + (int64_t)row * (in1 ? n1 : n0) +
                                                       (in1 ? cc - n0 : cc));
#pragma unroll
        for (int v = 0; v < 4; ++v) m[v] = __ldg(m4 + v);
      } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) m[v] = make_int4(-1, -1, -1, -1);
      }
    };
    // the accumulator columns of chunk cc (16 Re + 16 Im per lane)
    auto ld_chunk = [&](int cc, float (&re)[16], float (&im)[16]) {
      const bool in1 = cc >= n0;  // warp-uniform
      const int c0 = in1 ? cc - n0 : cc;
      tmem_ld16(lane_base + (in1 ? c_re1 : c_re0) + (uint32_t)c0, re);
      tmem_ld16(lane_base + (in1 ? c_im1 : c_im0) + (uint32_t)c0, im);
    };
    // Software-pipelined: chunk cc + 32 is read from TMEM while chunk cc is
    // stored, and TMEM is released (bar_tfree) as soon as the warp's last
    // chunk has landed in registers, before that chunk's stores.
    for (int f = blockIdx.x, li = 0; f < nspec; f += G, ++li) {
      int4 mcur[4], mnext[4];
      load_map(16 * half, mcur);
      if (!mbar_wait(bar_acc, (uint32_t)li & 1u)) {
        atomicExch(err, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      float2* orow = binmajor + (int64_t)f * bin_pitch;
      float re[2][16], im[2][16];
      int cc = 16 * half;
      if (cc < ncols) {
        ld_chunk(cc, re[0], im[0]);
        tmem_ld_wait();
        reg_fence16(re[0]);
        reg_fence16(im[0]);
      }
      bool released = false;
      for (int k = 0; cc < ncols; cc += 32, k ^= 1) {
        const bool more = cc + 32 < ncols;
        load_map(cc + 32, mnext);
        if (more) {
          if (k == 0) ld_chunk(cc + 32, re[1], im[1]); else ld_chunk(cc + 32, re[0], im[0]);
        } else {
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(bar_tfree);
          released = true;
        }
        if (k == 0)
          store_slots16(orow, reinterpret_cast<const int32_t*>(mcur), re[0], im[0], scale);
        else
          store_slots16(orow, reinterpret_cast<const int32_t*>(mcur), re[1], im[1], scale);
        if (more) {
          tmem_ld_wait();
          if (k == 0) {
            reg_fence16(re[1]);
            reg_fence16(im[1]);
          } else {
            reg_fence16(re[0]);
            reg_fence16(im[0]);
          }
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) mcur[v] = mnext[v];
      }
      if (!released) {  // no chunk for this warp
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(bar_tfree);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

// Bin-major rows -> the [pair][bin] stack: stack[perm[q]][f] (+)=
// binmajor[f][q], through 32 x 32 shared-memory tiles so both sides move in
// 256-byte runs (each slot's 32 bins are one run of its pair row).
__global__ void __launch_bounds__(256)
    k_xc_binmajor_to_stack(const float2* __restrict__ binmajor, int64_t bin_pitch, int64_t npairs, int nspec,
                           const int32_t* __restrict__ perm, float2* __restrict__ stack, int64_t stack_pitch,
                           int accumulate) {
  __shared__ float2 tile[32][33];
  const int64_t p0 = (int64_t)blockIdx.x * 32;
  const int f0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
  for (int k = ty; k < 32; k += 8) {
    const int f = f0 + k;
    const int64_t p = p0 + tx;
    if (f < nspec && p < npairs) tile[k][tx] = __ldcs(binmajor + (int64_t)f * bin_pitch + p);
  }
  __syncthreads();
#pragma unroll
  for (int k = ty; k < 32; k += 8) {
    const int64_t q = p0 + k;
    const int f = f0 + tx;
    if (q < npairs && f < nspec) {
      float2 v = tile[tx][k];
      float2* d = stack + (int64_t)__ldg(perm + q) * stack_pitch + f;
      if (accumulate) {
        const float2 o = *d;
        v.x += o.x;
        v.y += o.y;
      }
      *d = v;
    }
  }
}

// True when the plan's tiles are exactly the whole-bin geometry (C <= 192,
// no duplicated pairs needing extra tile layers).
static bool whole_bin_plan(const XcTensorPlan* tp) {
  const int C = tp->nchan;
  if (C < 1 || C > 192 || tp->h_tiles.empty()) return false;
  const auto& t = tp->h_tiles;
  if (C <= kTcM) return t.size() == 1 && t[0].a0 == 0 && t[0].b0 == 0 && t[0].am == C && t[0].bn == C;
  return t.size() == 2 && t[0].a0 == 0 && t[0].b0 == 0 && t[0].am == kTcM && t[0].bn == C && t[1].a0 == kTcM &&
         t[1].b0 == kTcM && t[1].am == C - kTcM && t[1].bn == C - kTcM;
}

// Whether the whole-bin kernel (one CTA per bin) can run this plan: the
// whole-bin tile geometry and a bin-major row that fits its staging.
static bool whole_bin_eligible(const fxc_pairplan* plan) {
  return plan->tensor && whole_bin_plan(plan->tensor) &&
         plan->npairs * (int64_t)sizeof(float2) <= (int64_t)kBinStages * kBinStageBytes;
}

// The layout a tensor contraction runs. A plan's preference
// (xc_tensor_set_layout, chosen by the autotuner from timings) wins where
// the plan is eligible for it. Without one: the whole-bin kernel unless the
// contraction is short (at most three K-blocks) over at most 128 channels,
// where the persistent tiled kernel, which pays the per-CTA setup once per
// SM rather than once per bin, is ahead (at 90 channels and 24 windows
// 0.038 ms against 0.050 ms per 512 bins; at 192 channels the two tie for
// short contractions and from 264 windows the whole-bin kernel leads).
static bool use_whole_bin(const fxc_pairplan* plan, int nkb) {
  if (!whole_bin_eligible(plan) || getenv("FXC_GEMM_TILED")) return false;
  if (plan->tensor->layout == FXC_XC_LAYOUT_WHOLE_BIN) return true;
  if (plan->tensor->layout == FXC_XC_LAYOUT_TILED) return false;
  return nkb > 3 || plan->tensor->nchan > kTcM;
}

int xc_tensor_layouts(const fxc_pairplan* plan) {
  if (!plan->tensor || plan->tensor->ntiles == 0) return 0;
  return (1 << FXC_XC_LAYOUT_TILED) | (whole_bin_eligible(plan) ? 1 << FXC_XC_LAYOUT_WHOLE_BIN : 0);
}

int xc_tensor_layout(const fxc_pairplan* plan) { return plan->tensor ? plan->tensor->layout : FXC_XC_LAYOUT_AUTO; }

void xc_tensor_set_layout(const fxc_pairplan* plan, int layout) {
  if (plan->tensor) plan->tensor->layout = layout;
}

int xc_tensor_effective_layout(const fxc_pairplan* plan, int64_t nwin) {
  if (!plan->tensor) return FXC_XC_LAYOUT_AUTO;
  return use_whole_bin(plan, (int)((nwin + kTcKb - 1) / kTcKb)) ? FXC_XC_LAYOUT_WHOLE_BIN : FXC_XC_LAYOUT_TILED;
}

int64_t xc_packed_chunks(int32_t nchan, int64_t nwin, int32_t nspec) {
  const int64_t nkb = (nwin + kTcKb - 1) / kTcKb;
  return (int64_t)nspec * kTcPlanes * nkb * kTcKc * round_up(nchan, 8);
}

int xc_pack_launch(fxc_ctx* ctx, const float2* spec, int64_t nwin, int nchan, int nspec,
                   int64_t spec_pitch, const uint8_t* mask, uint4* packed, int kb0, int kb1,
                   int64_t w_base) {
  const int nkb = (int)((nwin + kTcKb - 1) / kTcKb);
  if (kb1 < 0) kb1 = nkb;
  if (nkb == 0 || nspec == 0 || kb1 <= kb0) return FXC_OK;
  const int cpad = (int)round_up(nchan, 8);
  FXC_CHECK_ARG((cpad + kPackC - 1) / kPackC <= 65535 && nkb <= 65535, "pack grid too large");
  FXC_CHECK_ARG(kb0 >= 0 && kb1 <= nkb && w_base <= (int64_t)kb0 * kTcKb, "pack block range invalid");
  dim3 pg((unsigned)((nspec + kPackF - 1) / kPackF), (unsigned)((cpad + kPackC - 1) / kPackC),
          (unsigned)(kb1 - kb0));
  FXC_TRY(set_smem_limit(k_xc_pack, kPackSmem));
  k_xc_pack<<<pg, 256, kPackSmem, ctx->stream>>>(spec, nwin, nchan, nspec, spec_pitch, mask, nkb,
                                                 cpad, kb0, w_base, packed);
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

// The whole-bin contraction into bin-major rows ([bin][bin_pitch] complex,
// context scratch): the producer of both the [pair][bin] transpose and the
// direct finalize.
// Operands from `packed` (src == null) or straight from the FP32 spectra
// (the fused pack, src != null).
static int gemm_bin_rows(fxc_ctx* ctx, const fxc_pairplan* plan, const uint4* packed, const BinSrc* src, int nkb,
                         int nspec, float scale, float2** rows, int64_t* bin_pitch) {
  const XcTensorPlan* tp = plan->tensor;
  *bin_pitch = round_up(plan->npairs, 4);
  FXC_TRY(ctx->scratch5.reserve(sizeof(float2) * (size_t)*bin_pitch * (size_t)nspec));
  *rows = reinterpret_cast<float2*>(ctx->scratch5.ptr);
  KernelTimer kt(ctx, "k_xc_tc_gemm_bin");
  if (src) {
    // clusters of kBinCluster CTAs, one per bin (the last cluster's CTAs
    // past nspec load and convert their rows but write no output)
    FXC_TRY(set_smem_limit(k_xc_tc_gemm_bin<true>, kBinSmemBytesF));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)round_up(nspec, kBinCluster));
    cfg.blockDim = dim3((unsigned)kTcThreads);
    cfg.dynamicSmemBytes = kBinSmemBytesF;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kBinCluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FXC_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_xc_tc_gemm_bin<true>, (const uint4*)nullptr, *src, nkb, (int)tp->cpad,
                                    (int)tp->nchan, (const TcTile*)tp->d_tiles, (int)tp->ntiles,
                                    (const int32_t*)tp->d_maps, scale, *rows, *bin_pitch, (int)plan->npairs,
                                    ctx->d_err));
  } else if (!getenv("FXC_GEMM_BIN_PERCTA")) {
    // persistent: one CTA per SM over the bins
    FXC_TRY(set_smem_limit(k_xc_tc_gemm_bin_p, kBinSmemBytes));
    int nsm = 0;
    FXC_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
    const unsigned grid = (unsigned)std::min<int64_t>(nspec, std::max(nsm, 1));
    k_xc_tc_gemm_bin_p<<<grid, kTcThreads, kBinSmemBytes, ctx->stream>>>(
        packed, nspec, nkb, tp->cpad, tp->nchan, tp->d_tiles, (int)tp->ntiles, tp->d_maps, scale, *rows,
        *bin_pitch, ctx->d_err);
  } else {
    FXC_TRY(set_smem_limit(k_xc_tc_gemm_bin<false>, kBinSmemBytes));
    k_xc_tc_gemm_bin<false><<<(unsigned)nspec, kTcThreads, kBinSmemBytes, ctx->stream>>>(
        packed, BinSrc{}, nkb, tp->cpad, tp->nchan, tp->d_tiles, (int)tp->ntiles, tp->d_maps, scale, *rows,
        *bin_pitch, (int)plan->npairs, ctx->d_err);
  }
  kt.stop();
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

// The fused pack + whole-bin contraction of FP32 spectra into the stack, or
// FXC_ERR_UNSUPPORTED where the plan does not take the whole-bin layout or
// the fused form is not selected (FXC_GEMM_FUSED=1 selects it; the caller
// then packs). Measured at 192 channels x 720 windows x 18 523 bins: the
// contraction 15.6 ms against 6.8 ms for the packed one (+ 6.6 ms of
// k_xc_pack), its stack bit-identical. With the loads replaced by
// constants it still took 9.9 ms: the 4-CTA lockstep of every K-block
// (empty and full barriers across the cluster), the distributed-shared-
// memory stores and 144 of the 152 SMs (36 clusters of 4 fit) cost more than
// the 2.4 us of MMAs per K-block leave; the loads through the cp.async
// staging ring then add another 5.7 ms.
int xc_gemm_f32_launch(fxc_ctx* ctx, const fxc_pairplan* plan, const float2* spec, int64_t nwin, int nchan,
                       int nspec, int64_t spec_pitch, const uint8_t* mask, int64_t w_base, float scale,
                       float2* stack, int64_t stack_pitch, int accumulate) {
  const XcTensorPlan* tp = plan->tensor;
  FXC_CHECK_ARG(tp != nullptr, "pair plan has no tensor tiles");
  const int nkb = (int)((nwin + kTcKb - 1) / kTcKb);
  const char* fe = getenv("FXC_GEMM_FUSED");
  if (!fe || fe[0] != '1' || nkb == 0 || !use_whole_bin(plan, nkb)) return FXC_ERR_UNSUPPORTED;
  // 16-byte copies of 2 bins: 16-byte aligned rows, every bin of the last
  // cluster inside the row pitch; no window mask (masked calls pack)
  if ((reinterpret_cast<uintptr_t>(spec) & 15u) != 0 || spec_pitch % 2 != 0 ||
      spec_pitch < round_up(nspec, kBinCluster) || mask != nullptr)
    return FXC_ERR_UNSUPPORTED;
  FXC_CHECK_ARG(nchan == tp->nchan && nchan <= 192, "channel count %d does not match the plan", nchan);
  FXC_CHECK_ARG(nspec <= 65535, "nspec %d above the tensor grid limit", nspec);
  if (tp->ntiles == 0 || nspec == 0) return FXC_OK;
  const BinSrc src{spec, nwin, spec_pitch, w_base, mask, nspec};
  float2* binmajor = nullptr;
  int64_t bin_pitch = 0;
  FXC_TRY(gemm_bin_rows(ctx, plan, nullptr, &src, nkb, nspec, scale, &binmajor, &bin_pitch));
  const dim3 tg((unsigned)((plan->npairs + 31) / 32), (unsigned)((nspec + 31) / 32));
  k_xc_binmajor_to_stack<<<tg, 256, 0, ctx->stream>>>(binmajor, bin_pitch, plan->npairs, nspec, tp->d_perm, stack,
                                                       stack_pitch, accumulate);
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

int xc_gemm_launch(fxc_ctx* ctx, const fxc_pairplan* plan, const uint4* packed, int64_t nwin,
                   int nspec, float scale, float2* stack, int64_t stack_pitch, int accumulate) {
  const XcTensorPlan* tp = plan->tensor;
  FXC_CHECK_ARG(tp != nullptr, "pair plan has no tensor tiles");
  if (tp->ntiles == 0 || nspec == 0) return FXC_OK;
  FXC_CHECK_ARG(nspec <= 65535, "nspec %d above the tensor grid limit", nspec);
  const int nkb = (int)((nwin + kTcKb - 1) / kTcKb);
  if (nkb == 0) {
    if (accumulate) return FXC_OK;
    // no windows: every stacked bin is zero
    FXC_CUDA_TRY(cudaMemset2DAsync(stack, sizeof(float2) * (size_t)stack_pitch, 0,
                                   sizeof(float2) * (size_t)nspec, (size_t)plan->npairs,
                                   ctx->stream));
    return FXC_OK;
  }
  if (use_whole_bin(plan, nkb)) {
    // bin-major rows in context scratch, then transposed into the stack
    float2* binmajor = nullptr;
    int64_t bin_pitch = 0;
    FXC_TRY(gemm_bin_rows(ctx, plan, packed, nullptr, nkb, nspec, scale, &binmajor, &bin_pitch));
    const dim3 tg((unsigned)((plan->npairs + 31) / 32), (unsigned)((nspec + 31) / 32));
    k_xc_binmajor_to_stack<<<tg, 256, 0, ctx->stream>>>(binmajor, bin_pitch, plan->npairs, nspec, tp->d_perm,
                                                         stack, stack_pitch, accumulate);
    count_launch();
    FXC_LAUNCH_CHECK();
    return FXC_OK;
  }
  FXC_TRY(set_smem_limit(k_xc_tc_gemm, kTcSmemBytes));
  // one persistent CTA per SM (the operand ring fills the shared memory)
  int nsm = 0;
  FXC_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
  // bin-major rows of at most kBinMajorCap bytes per pass, then transposed
  const int64_t bin_pitch = round_up(plan->npairs, 4);
  const int64_t fb = std::max<int64_t>(1, std::min<int64_t>(nspec, kBinMajorCap / (bin_pitch * 8)));
  FXC_TRY(ctx->scratch5.reserve(sizeof(float2) * (size_t)bin_pitch * (size_t)fb));
  float2* binmajor = reinterpret_cast<float2*>(ctx->scratch5.ptr);
  const int64_t per_bin = (int64_t)kTcPlanes * nkb * kTcKc * tp->cpad;  // 16-byte chunks per bin
  for (int64_t f0 = 0; f0 < nspec; f0 += fb) {
    const int nb = (int)std::min<int64_t>(fb, nspec - f0);
    const int64_t items = tp->ntiles * (int64_t)nb;
    const unsigned grid = (unsigned)std::min<int64_t>(items, std::max(nsm, 1));
    KernelTimer kt(ctx, "k_xc_tc_gemm");
    k_xc_tc_gemm<<<grid, kTcThreads, kTcSmemBytes, ctx->stream>>>(
        packed + f0 * per_bin, nkb, tp->cpad, tp->d_tiles, (int)tp->ntiles, tp->d_maps, nb, scale, binmajor,
        bin_pitch, ctx->d_err);
    kt.stop();
    count_launch();
    FXC_LAUNCH_CHECK();
    const dim3 tg((unsigned)((plan->npairs + 31) / 32), (unsigned)((nb + 31) / 32));
    k_xc_binmajor_to_stack<<<tg, 256, 0, ctx->stream>>>(binmajor, bin_pitch, plan->npairs, nb, tp->d_perm,
                                                         stack + f0, stack_pitch, accumulate);
    count_launch();
    FXC_LAUNCH_CHECK();
  }
  return FXC_OK;
}

int xc_gemm_finalize_launch(fxc_ctx* ctx, const fxc_pairplan* plan, const uint4* packed, int64_t nwin,
                            int nspec, float scale, const fxc_xc_shape* s, float* ncf) {
  // A finalize reading the bin-major rows directly (stride npairs x 8 B per
  // bin) was 1.5 ms slower at 192 channels than the transpose + a finalize
  // of contiguous rows: each pair's CTA touches every page of the rows.
  FXC_CHECK_ARG(plan->tensor != nullptr, "pair plan has no tensor tiles");
  if (plan->npairs == 0) return FXC_OK;
  const int64_t pitch = xc_stack_pitch(nspec);
  FXC_TRY(ctx->scratch.reserve(sizeof(float2) * (size_t)pitch * (size_t)plan->npairs));
  float2* stack = reinterpret_cast<float2*>(ctx->scratch.ptr);
  FXC_TRY(xc_gemm_launch(ctx, plan, packed, nwin, nspec, scale, stack, pitch));
  return xc_finalize_launch(ctx, stack, plan->npairs, pitch, s, ncf);
}

int xc_stack_tensor_launch(fxc_ctx* ctx, const fxc_pairplan* plan, const float2* spec,
                           int64_t nwin, int nchan, int nspec, int64_t spec_pitch,
                           const uint8_t* mask, float scale, float2* stack, int64_t stack_pitch,
                           int accumulate) {
  const XcTensorPlan* tp = plan->tensor;
  FXC_CHECK_ARG(tp != nullptr, "pair plan has no tensor tiles");
  if (tp->ntiles == 0) return FXC_OK;
  {
    const int rc = xc_gemm_f32_launch(ctx, plan, spec, nwin, nchan, nspec, spec_pitch, mask, 0, scale, stack,
                                      stack_pitch, accumulate);
    if (rc != FXC_ERR_UNSUPPORTED) return rc;
    clear_error();
  }
  const int64_t chunks = xc_packed_chunks(nchan, nwin, nspec);
  if (chunks > 0) FXC_TRY(ctx->scratch3.reserve((size_t)chunks * 16));
  uint4* packed = reinterpret_cast<uint4*>(ctx->scratch3.ptr);
  FXC_TRY(xc_pack_launch(ctx, spec, nwin, nchan, nspec, spec_pitch, mask, packed));
  return xc_gemm_launch(ctx, plan, packed, nwin, nspec, scale, stack, stack_pitch, accumulate);
}

}  // namespace fxc

using namespace fxc;

extern "C" {

int fxc_xc_packed_bytes(int32_t nchan, int64_t nwin, int32_t nspec, int64_t* out_bytes) {
  clear_error();
  FXC_CHECK_ARG(out_bytes != nullptr, "out_bytes is null");
  FXC_CHECK_ARG(nchan > 0 && nwin >= 0 && nspec >= 0, "invalid shape");
  *out_bytes = xc_packed_chunks(nchan, nwin, nspec) * 16;
  return FXC_OK;
}

int fxc_xc_pack(fxc_ctx* ctx, const float* d_spec, int64_t nwin, int32_t nchan, int32_t nspec,
                int64_t spec_pitch, const uint8_t* d_mask, void* d_packed) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(nchan > 0 && nwin >= 0 && nspec >= 0 && spec_pitch >= nspec, "invalid shape");
  FXC_CHECK_ARG(nwin == 0 || nspec == 0 || (d_spec && d_packed), "null pointer");
  FXC_CHECK_ARG(((uintptr_t)d_packed & 15) == 0, "d_packed must be 16-byte aligned");
  return xc_pack_launch(ctx, reinterpret_cast<const float2*>(d_spec), nwin, nchan, nspec,
                        spec_pitch, d_mask, reinterpret_cast<uint4*>(d_packed));
}

int fxc_xc_stack_packed(fxc_ctx* ctx, const fxc_pairplan* plan, const void* d_packed, int64_t nwin,
                        int32_t nspec, float scale, float* d_stack, int64_t stack_pitch) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(plan != nullptr, "null pair plan");
  FXC_CHECK_ARG(nwin >= 0 && nspec >= 1 && stack_pitch >= nspec, "invalid shape");
  FXC_CHECK_ARG(plan->npairs == 0 || (d_packed && d_stack), "null pointer");
  return xc_gemm_launch(ctx, plan, reinterpret_cast<const uint4*>(d_packed), nwin, nspec, scale,
                        reinterpret_cast<float2*>(d_stack), stack_pitch);
}

int fxc_xc_stack_finalize_packed(fxc_ctx* ctx, const fxc_pairplan* plan, const void* d_packed, int64_t nwin,
                                 int32_t nspec, float scale, const fxc_xc_shape* shape, float* d_ncf) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(plan != nullptr && shape != nullptr, "null plan or shape");
  FXC_CHECK_ARG(nwin >= 0 && nspec >= 1 && shape->nspec == nspec, "invalid shape");
  FXC_CHECK_ARG(shape->nfft == 2 * (shape->nspec - 1) && shape->cc_size == 2 * shape->half_cc + 1,
                "inconsistent shape");
  FXC_CHECK_ARG(plan->npairs == 0 || (d_packed && d_ncf), "null pointer");
  return xc_gemm_finalize_launch(ctx, plan, reinterpret_cast<const uint4*>(d_packed), nwin, nspec, scale, shape,
                                 d_ncf);
}

}  // extern "C"
