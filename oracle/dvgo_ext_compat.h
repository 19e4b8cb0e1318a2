// Force-included (nvcc -include) when the reference's DirectVoxGO torch
// extensions (lib/cuda/render_utils_kernel.cu, total_variation_kernel.cu,
// adam_upd_kernel.cu) are compiled against a PyTorch whose dispatch macros no
// longer accept the deprecated `tensor.type()` argument. It supplies that one
// overload so the reference kernels build unmodified; nothing else changes.
// Test infrastructure only (golden-vector generation).
#pragma once
#include <ATen/ATen.h>

namespace detail {
inline at::ScalarType scalar_type(const at::DeprecatedTypeProperties& t) {
  return t.scalarType();
}
}  // namespace detail
