// util.cuh -- device utilities shared between passes.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace f184 {

// Exclusive scan of n u32 values (n <= 1M); `total` (device, may be null) receives the sum.
// scratch: scan_scratch_bytes(n) bytes of device memory.
size_t scan_scratch_bytes(uint32_t n);
int exclusive_scan(const uint32_t* in, uint32_t n, uint32_t* out, uint32_t* total, void* scratch, cudaStream_t s);

}  // namespace f184
