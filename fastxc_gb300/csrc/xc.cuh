// Internal declarations of the xc stage (correlation + stack + finalize).
#pragma once

#include <vector>

#include "context.cuh"

namespace fxc {

constexpr int kXcTile = 16;       // channels per tile side
constexpr int kXcFreqChunk = 64;  // bins per CTA of the plain kernel
constexpr int kTcKbWindows = 32;  // windows per K-block of the packed tensor operands

struct XcTile {
  int32_t a_base;      // first src channel of the tile
  int32_t b_base;      // first rec channel of the tile
  int32_t map_offset;  // offset of the 16x16 pair-index map in the map array
  int32_t npairs;      // pairs mapped into the tile
};

struct XcTensorPlan;

int pairplan_build(const int32_t* src, const int32_t* rec, int64_t npairs, int32_t nchan,
                   std::vector<XcTile>* tiles, std::vector<int32_t>* maps);
int64_t xc_stack_pitch(int nspec);

}  // namespace fxc

struct fxc_pairplan {
  int device = 0;
  int64_t npairs = 0;
  int32_t nchan = 0;
  int64_t ntiles = 0;
  std::vector<int32_t> h_src, h_rec;
  fxc::XcTile* d_tiles = nullptr;
  int32_t* d_maps = nullptr;
  fxc::XcTensorPlan* tensor = nullptr;
};

namespace fxc {

int xc_stack_launch(fxc_ctx* ctx, const fxc_pairplan* plan, const float2* spec, int64_t nwin,
                    int nchan, int nspec, int64_t spec_pitch, const uint8_t* mask, float scale,
                    float2* stack, int64_t stack_pitch, int method, int accumulate = 0);
int xc_finalize_launch_tables(fxc_ctx* ctx, const float2* stack, int64_t npairs,
                              int64_t stack_pitch, const fxc_xc_shape* s, const float2* twn,
                              const int* perm, float* ncf);

int xc_tensor_plan_init(fxc_ctx* ctx, fxc_pairplan* plan);
void xc_tensor_plan_free(fxc_pairplan* plan);
// Contraction layouts (FXC_XC_LAYOUT_*): the admitted ones as a bit mask,
// the plan's preference, and the layout a run of nwin windows takes.
int xc_tensor_layouts(const fxc_pairplan* plan);
int xc_tensor_layout(const fxc_pairplan* plan);
void xc_tensor_set_layout(const fxc_pairplan* plan, int layout);
int xc_tensor_effective_layout(const fxc_pairplan* plan, int64_t nwin);
int xc_stack_tensor_launch(fxc_ctx* ctx, const fxc_pairplan* plan, const float2* spec,
                           int64_t nwin, int nchan, int nspec, int64_t spec_pitch,
                           const uint8_t* mask, float scale, float2* stack, int64_t stack_pitch,
                           int accumulate = 0);
// Packs K-blocks [kb0, kb1) (kb1 < 0: all); spec holds windows from w_base
// on (w_base <= kb0 * 32).
int xc_pack_launch(fxc_ctx* ctx, const float2* spec, int64_t nwin, int nchan, int nspec,
                   int64_t spec_pitch, const uint8_t* mask, uint4* packed, int kb0 = 0, int kb1 = -1,
                   int64_t w_base = 0);
int xc_gemm_launch(fxc_ctx* ctx, const fxc_pairplan* plan, const uint4* packed, int64_t nwin,
                   int nspec, float scale, float2* stack, int64_t stack_pitch, int accumulate = 0);
// Fused pack + whole-bin contraction of FP32 spectra (windows from w_base
// on in spec) into the stack; FXC_ERR_UNSUPPORTED where the plan does not
// take the whole-bin layout.
int xc_gemm_f32_launch(fxc_ctx* ctx, const fxc_pairplan* plan, const float2* spec, int64_t nwin, int nchan,
                       int nspec, int64_t spec_pitch, const uint8_t* mask, int64_t w_base, float scale,
                       float2* stack, int64_t stack_pitch, int accumulate);
int64_t xc_packed_chunks(int32_t nchan, int64_t nwin, int32_t nspec);
int xc_finalize_launch(fxc_ctx* ctx, const float2* stack, int64_t npairs, int64_t stack_pitch,
                       const fxc_xc_shape* s, float* ncf);
// Contraction of packed operands + finalize, the stack in context scratch.
int xc_gemm_finalize_launch(fxc_ctx* ctx, const fxc_pairplan* plan, const uint4* packed, int64_t nwin,
                            int nspec, float scale, const fxc_xc_shape* s, float* ncf);

}  // namespace fxc
