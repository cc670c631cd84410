// trace_f16_iso.cu -- the cone-trace kernel variants for F16 storage, isotropic mips
// (one translation unit per storage format and mip kind, so the variants compile in parallel).
#include "trace_kernel.cuh"

namespace f184 {
const void* trace_kernel_f16_iso(uint32_t variant) { return kernel_for<F184GI_FMT_F16, false>(variant); }
const void* trace_kernel_count_f16_iso() { return count_kernel<F184GI_FMT_F16, false>(); }
}  // namespace f184
