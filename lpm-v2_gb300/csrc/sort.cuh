// sort.cuh -- Morton ordering of source particles (device radix sort).
#pragma once

#include "lpm_common.cuh"

namespace lpm {

// Scratch bytes morton_sort needs for ns sources.
size_t morton_sort_bytes(int64_t ns);

// sorted[0..ns) = idx[0..ns) ordered by the Morton code of (x, y, z) * inv_a.  z may be NULL
// (planar particles).  Enqueued on `stream`; no allocation.
int morton_sort(cudaStream_t stream, int64_t ns, const int32_t* idx, const double* x, const double* y,
                const double* z, double inv_a, void* scratch, size_t scratch_bytes, int32_t* sorted);

}  // namespace lpm
