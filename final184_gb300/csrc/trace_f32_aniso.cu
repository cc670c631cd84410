// trace_f32_aniso.cu -- the cone-trace kernel variants for F32 storage, six-direction anisotropic mips
// (one translation unit per storage format and mip kind, so the variants compile in parallel).
#include "trace_kernel.cuh"

namespace f184 {
const void* trace_kernel_f32_aniso(uint32_t variant) { return kernel_for<F184GI_FMT_F32, true>(variant); }
const void* trace_kernel_count_f32_aniso() { return count_kernel<F184GI_FMT_F32, true>(); }
}  // namespace f184
