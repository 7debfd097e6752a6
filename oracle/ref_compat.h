/* ORACLE — test infrastructure only (never part of the product).
 *
 * Forced-include header (nvcc -include) for compiling the reference's own
 * CUDA sources (lib/cuda/*_kernel.cu) with the PyTorch headers of this image.
 * Those sources dispatch on `tensor.type()` (e.g. render_utils_kernel.cu:92,
 * adam_upd_kernel.cu:74), whose conversion for AT_DISPATCH_* was removed from
 * PyTorch 2.x; the overload below restores it so that the files compile as
 * they are.  It changes no device code: only the __global__ kernels of the
 * resulting PTX are ever run (oracle/ref_cuda.py launches them).
 */
#pragma once
#include <torch/extension.h>

namespace detail {
inline at::ScalarType scalar_type(const at::DeprecatedTypeProperties& t) { return t.scalarType(); }
}  // namespace detail
