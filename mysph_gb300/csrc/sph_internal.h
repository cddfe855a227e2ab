// sph_internal.h — host-side helpers shared by the translation units of
// libsphgpu (not part of the C ABI).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sph {

// Exclusive prefix sum of n uint32 values (out may alias in).  `partials`
// must hold scan_partials(n) uint32 values.  Adds the launches it issues to
// *launches.
int64_t scan_partials(int64_t n);
void exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* partials,
                        cudaStream_t s, int64_t* launches);

// Stable LSD radix sort of (key, value) pairs; scratch layout and size as
// sph_sort_scratch_bytes.  Returns a cudaError_t.
int64_t sort_scratch_bytes(int64_t n, int key_bits);
cudaError_t sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                       uint32_t* vals_out, int64_t n, int key_bits, void* scratch,
                       cudaStream_t s, int64_t* launches);

}  // namespace sph
