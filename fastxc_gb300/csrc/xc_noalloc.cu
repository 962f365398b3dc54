// fxc_xc_run_noalloc: the xc correlation + stack + finalize pipeline without
// any device allocation.
//
// Who needs it: callers that cannot call cudaMalloc -- code running inside a
// host framework that owns all device memory through its own pool, code that
// must not grow the process's device footprint after start-up, or callers
// that run under a memory budget fixed before the job starts. fxc_xc_run
// grows a per-context scratch buffer with cudaMalloc and its FFT tables are
// cudaMalloc'ed once per device; this variant keeps every byte it needs in
// one file-scope device array instead.
//
// The array (kNoallocBytes, 64 MiB) is part of the module image: every GPU
// that loads the library holds it until the process exits. Its contents per
// call, each region 256-byte aligned:
//   pair tiles | tile pair maps | twiddle table (nfft) | digit-reversal
//   table (nfft/2) | stacked spectra [npairs][pitch]
// All of it is rewritten by every call before it is read (the stack kernel
// writes every bin the finalize kernel reads), so nothing has to be cleared;
// the array simply keeps the last call's contents. All calls share the one
// array, so calls whose work overlaps on the GPU (different streams, or
// concurrent host threads) race and must be serialised by the caller.
#include <mutex>
#include <vector>

#include "context.cuh"
#include "fft.cuh"
#include "fft_launch.cuh"
#include "xc.cuh"

namespace fxc {

constexpr size_t kNoallocBytes = size_t(64) << 20;
constexpr int kNoallocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_xc_noalloc_scratch[kNoallocBytes];

// Device address of the array, looked up once per device with that device
// current (in host code the symbol itself is only a host-side stand-in).
static int noalloc_scratch_address(int device, unsigned char** out) {
  static std::mutex mu;
  static unsigned char* addr[kNoallocMaxDevices] = {nullptr};
  FXC_CHECK_ARG(device >= 0 && device < kNoallocMaxDevices, "device %d out of range", device);
  std::lock_guard<std::mutex> lock(mu);
  if (addr[device] == nullptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_xc_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      (void)cudaGetLastError();
      set_error("cudaGetSymbolAddress of the no-alloc scratch array failed on device %d: %s", device,
                cudaGetErrorString(e));
      return FXC_ERR_CUDA;
    }
    addr[device] = static_cast<unsigned char*>(p);
  }
  *out = addr[device];
  return FXC_OK;
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace fxc

using namespace fxc;

extern "C" int fxc_xc_run_noalloc(fxc_ctx* ctx, const int32_t* h_src, const int32_t* h_rec,
                                  int64_t npairs, const float* d_spec, int64_t nwin, int32_t nchan,
                                  int64_t spec_pitch, const uint8_t* d_mask, float scale,
                                  const fxc_xc_shape* shape, float* d_ncf) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(shape != nullptr, "null shape");
  FXC_CHECK_ARG(npairs >= 0 && nchan > 0 && nwin >= 0, "invalid npairs/nchan/nwin");
  FXC_CHECK_ARG(npairs == 0 || (h_src && h_rec && d_spec && d_ncf), "null pointer argument");
  FXC_CHECK_ARG(spec_pitch >= shape->nspec, "spec_pitch %lld < nspec %d", (long long)spec_pitch,
                shape->nspec);
  FXC_CHECK_ARG(shape->nfft == 2 * (shape->nspec - 1) && shape->cc_size == 2 * shape->half_cc + 1,
                "inconsistent shape");
  if (npairs == 0) return FXC_OK;
  const int N = shape->nfft;
  const int M = N / 2;
  FXC_CHECK_ARG(N % 2 == 0 && M <= kFftLargeNmax, "nfft %d not supported", N);

  std::vector<XcTile> tiles;
  std::vector<int32_t> maps;
  FXC_TRY(pairplan_build(h_src, h_rec, npairs, nchan, &tiles, &maps));

  const int64_t pitch = xc_stack_pitch(shape->nspec);
  const size_t off_tiles = 0;
  const size_t off_maps = align256(off_tiles + sizeof(XcTile) * tiles.size());
  const size_t off_tw = align256(off_maps + sizeof(int32_t) * maps.size());
  const size_t off_perm = align256(off_tw + sizeof(float2) * (size_t)N);
  const size_t off_stack = align256(off_perm + sizeof(int) * (size_t)M);
  const size_t total = off_stack + sizeof(float2) * (size_t)pitch * (size_t)npairs;
  if (total > kNoallocBytes) {
    set_error("fxc_xc_run_noalloc: %lld pairs x nspec %d need %zu bytes of scratch, above the "
              "fixed %zu-byte (64 MiB) array; use fxc_xc_run or fewer pairs per call",
              (long long)npairs, shape->nspec, total, kNoallocBytes);
    return FXC_ERR_INVALID;
  }

  unsigned char* base = nullptr;
  FXC_TRY(noalloc_scratch_address(ctx->device, &base));

  std::vector<float2> tw((size_t)N);
  fft_twiddle_values(N, tw.data());
  FftPlan fp;
  FXC_TRY(fft_make_plan_with(M, nullptr, 2, nullptr, &fp));
  std::vector<int> perm((size_t)M);
  fft_perm_values(fp, perm.data());

  FXC_CUDA_TRY(cudaMemcpyAsync(base + off_tiles, tiles.data(), sizeof(XcTile) * tiles.size(),
                               cudaMemcpyHostToDevice, ctx->stream));
  FXC_CUDA_TRY(cudaMemcpyAsync(base + off_maps, maps.data(), sizeof(int32_t) * maps.size(),
                               cudaMemcpyHostToDevice, ctx->stream));
  FXC_CUDA_TRY(cudaMemcpyAsync(base + off_tw, tw.data(), sizeof(float2) * (size_t)N,
                               cudaMemcpyHostToDevice, ctx->stream));
  FXC_CUDA_TRY(cudaMemcpyAsync(base + off_perm, perm.data(), sizeof(int) * (size_t)M,
                               cudaMemcpyHostToDevice, ctx->stream));

  // A plan object that only points into the array (its host vectors stay empty).
  fxc_pairplan view;
  view.device = ctx->device;
  view.npairs = npairs;
  view.nchan = nchan;
  view.ntiles = (int64_t)tiles.size();
  view.d_tiles = reinterpret_cast<XcTile*>(base + off_tiles);
  view.d_maps = reinterpret_cast<int32_t*>(base + off_maps);
  view.tensor = nullptr;
  float2* stack = reinterpret_cast<float2*>(base + off_stack);
  int st = xc_stack_launch(ctx, &view, reinterpret_cast<const float2*>(d_spec), nwin, nchan,
                           shape->nspec, spec_pitch, d_mask, scale, stack, pitch, FXC_XC_PLAIN);
  view.d_tiles = nullptr;  // not owned
  view.d_maps = nullptr;
  if (st != FXC_OK) return st;
  return xc_finalize_launch_tables(ctx, stack, npairs, pitch, shape,
                                   reinterpret_cast<const float2*>(base + off_tw),
                                   reinterpret_cast<const int*>(base + off_perm), d_ncf);
}
