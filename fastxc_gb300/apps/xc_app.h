// Shared by the xc executables (xc_fast, xc_linear).
#pragma once

#include <string.h>

#include <vector>

#include "fastxc_gb300.h"

// Autotunes the stack method on the timestamp's first 512 bins (copied to
// the device for the timing runs only).
inline int autotune_host(fxc_ctx* ctx, fxc_pairplan* plan, const std::vector<float>& payload, int nstep,
                         int32_t nch, int nspec, int* method, int32_t* layout = nullptr) {
  const int sample = nspec < 512 ? nspec : 512;
  const size_t rows = (size_t)nstep * nch;
  std::vector<float> h(rows * sample * 2);
  for (size_t r = 0; r < rows; ++r)
    memcpy(h.data() + r * sample * 2, payload.data() + r * (size_t)nspec * 2, sizeof(float) * 2 * sample);
  void* d = nullptr;
  int rc = fxc_device_alloc(ctx, h.size() * sizeof(float), &d);
  if (rc == FXC_OK) rc = fxc_memcpy(ctx, d, h.data(), h.size() * sizeof(float), FXC_COPY_H2D);
  int32_t m = FXC_XC_PLAIN;
  int32_t lay = FXC_XC_LAYOUT_AUTO;
  if (rc == FXC_OK)
    rc = fxc_xc_autotune_layout(ctx, plan, (const float*)d, nstep, nch, sample, sample, &m, &lay, nullptr);
  if (layout) *layout = lay;
  fxc_device_free(ctx, d);
  *method = m;
  return rc;
}

