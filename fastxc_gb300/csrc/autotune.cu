// Autotuner of the xc stack: picks the method and the contraction layout
// for a shape by timing the candidates on a sample of frequency bins of the
// real input.
//
// Candidates: the plain FP32 kernel (16 x 16 channel tiles, 64 bins per CTA,
// register-tiled complex MACs) and the tcgen05 BF16 hi/lo contraction
// (pack pass + 128 x N channel tiles per bin) in each layout the plan
// admits: whole bin (one CTA per bin over every tile, a bin-major row per
// bin) and tiled (persistent CTAs over (tile, bin) items). Each candidate
// runs twice on the first `sample` bins (the second run is timed with CUDA
// events on the context's stream); the per-bin cost does not depend on the
// bin, so the faster sample is the faster full run. Decisions are cached
// per (device, channels, windows, pairs, pair-tile count) for the process.
#include <map>
#include <mutex>
#include <tuple>

#include "context.cuh"
#include "xc.cuh"

namespace fxc {
namespace {

struct TuneKey {
  int dev, nchan;
  int64_t nwin, npairs, ntiles;
  bool operator<(const TuneKey& o) const {
    return std::tie(dev, nchan, nwin, npairs, ntiles) < std::tie(o.dev, o.nchan, o.nwin, o.npairs, o.ntiles);
  }
};

struct TuneResult {
  int method = FXC_XC_PLAIN;
  int layout = FXC_XC_LAYOUT_AUTO;
  float ms[3] = {-1.f, -1.f, -1.f};  // plain, tensor whole-bin, tensor tiled
};

std::mutex g_mu;
std::map<TuneKey, TuneResult> g_cache;

int tune(fxc_ctx* ctx, const fxc_pairplan* plan, const float* d_spec, int64_t nwin, int32_t nchan, int32_t nspec,
         int64_t spec_pitch, TuneResult* out) {
  const TuneKey key{ctx->device, nchan, nwin, plan->npairs, plan->ntiles};
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      *out = it->second;
      return FXC_OK;
    }
  }
  TuneResult r;
  if (plan->npairs == 0) {
    *out = r;
    return FXC_OK;
  }
  const int sample = std::min<int>(nspec, 512);
  const int64_t pitch = xc_stack_pitch(sample);
  FXC_TRY(ctx->scratch.reserve((size_t)plan->npairs * pitch * sizeof(float2)));
  float2* stack = reinterpret_cast<float2*>(ctx->scratch.ptr);
  const float2* spec = reinterpret_cast<const float2*>(d_spec);
  const int admitted = xc_tensor_layouts(plan);
  const int saved = xc_tensor_layout(plan);
  // (method, layout) per candidate slot
  const int cand[3][2] = {{FXC_XC_PLAIN, FXC_XC_LAYOUT_AUTO},
                          {FXC_XC_TENSOR, FXC_XC_LAYOUT_WHOLE_BIN},
                          {FXC_XC_TENSOR, FXC_XC_LAYOUT_TILED}};
  cudaEvent_t e0, e1;
  FXC_CUDA_TRY(cudaEventCreate(&e0));
  FXC_CUDA_TRY(cudaEventCreate(&e1));
  int rc = FXC_OK;
  for (int c = 0; c < 3 && rc == FXC_OK; ++c) {
    if (cand[c][0] == FXC_XC_TENSOR && !(admitted & (1 << cand[c][1]))) continue;
    if (cand[c][0] == FXC_XC_TENSOR) xc_tensor_set_layout(plan, cand[c][1]);
    for (int rep = 0; rep < 2 && rc == FXC_OK; ++rep) {
      if (rep == 1) cudaEventRecord(e0, ctx->stream);
      rc = xc_stack_launch(ctx, plan, spec, nwin, nchan, sample, spec_pitch, nullptr, 1.0f, stack, pitch,
                           cand[c][0]);
      if (rep == 1) cudaEventRecord(e1, ctx->stream);
    }
    if (rc == FXC_OK && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&r.ms[c], e0, e1);
    if (rc != FXC_OK && cand[c][0] == FXC_XC_TENSOR) {
      // the tensor path is optional: a candidate that does not run is skipped
      r.ms[c] = -1.f;
      rc = FXC_OK;
      clear_error();
    }
  }
  xc_tensor_set_layout(plan, saved);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  FXC_TRY(rc);
  FXC_TRY(ctx_check_device_error(ctx));
  int best = 0;
  for (int c = 1; c < 3; ++c)
    if (r.ms[c] >= 0.f && r.ms[c] < r.ms[best]) best = c;
  r.method = cand[best][0];
  // the tensor layout: the faster of the two that ran (kept for a plain
  // decision too, for a caller that forces the tensor method)
  if (r.ms[1] >= 0.f && (r.ms[2] < 0.f || r.ms[1] <= r.ms[2]))
    r.layout = FXC_XC_LAYOUT_WHOLE_BIN;
  else if (r.ms[2] >= 0.f)
    r.layout = FXC_XC_LAYOUT_TILED;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache[key] = r;
  }
  *out = r;
  return FXC_OK;
}

}  // namespace
}  // namespace fxc

using namespace fxc;

extern "C" {

int fxc_xc_autotune_layout(fxc_ctx* ctx, const fxc_pairplan* plan, const float* d_spec, int64_t nwin,
                           int32_t nchan, int32_t nspec, int64_t spec_pitch, int32_t* method, int32_t* layout,
                           float* ms) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(plan && d_spec && method, "null argument");
  FXC_CHECK_ARG(nwin > 0 && nchan > 0 && nspec > 0 && spec_pitch >= nspec, "invalid shape");
  TuneResult r;
  FXC_TRY(tune(ctx, plan, d_spec, nwin, nchan, nspec, spec_pitch, &r));
  if (r.layout != FXC_XC_LAYOUT_AUTO) xc_tensor_set_layout(plan, r.layout);
  *method = r.method;
  if (layout) *layout = r.layout;
  if (ms)
    for (int c = 0; c < 3; ++c) ms[c] = r.ms[c];
  return FXC_OK;
}

int fxc_xc_autotune(fxc_ctx* ctx, const fxc_pairplan* plan, const float* d_spec, int64_t nwin, int32_t nchan,
                    int32_t nspec, int64_t spec_pitch, int32_t* method, float* ms_plain, float* ms_tensor) {
  float ms[3];
  int32_t layout = 0;
  FXC_TRY(fxc_xc_autotune_layout(ctx, plan, d_spec, nwin, nchan, nspec, spec_pitch, method, &layout, ms));
  if (ms_plain) *ms_plain = ms[0];
  if (ms_tensor) *ms_tensor = layout == FXC_XC_LAYOUT_WHOLE_BIN ? ms[1] : ms[2];
  return FXC_OK;
}

int fxc_pairplan_set_layout(fxc_pairplan* plan, int32_t layout) {
  clear_error();
  FXC_CHECK_ARG(plan != nullptr, "null plan");
  FXC_CHECK_ARG(layout == FXC_XC_LAYOUT_AUTO || layout == FXC_XC_LAYOUT_WHOLE_BIN || layout == FXC_XC_LAYOUT_TILED,
                "unknown layout %d", layout);
  xc_tensor_set_layout(plan, layout);
  return FXC_OK;
}

int fxc_pairplan_layouts(const fxc_pairplan* plan, int64_t nwin, int32_t* admitted, int32_t* effective) {
  clear_error();
  FXC_CHECK_ARG(plan != nullptr && nwin >= 0, "invalid argument");
  if (admitted) *admitted = xc_tensor_layouts(plan);
  if (effective) *effective = xc_tensor_effective_layout(plan, nwin);
  return FXC_OK;
}

}  // extern "C"
