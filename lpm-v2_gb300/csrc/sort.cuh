// sort.cuh -- Hilbert-curve ordering of source particles (device radix sort).
#pragma once

#include "lpm_common.cuh"

namespace lpm {

// Scratch bytes curve_sort needs for ns sources.
size_t curve_sort_bytes(int64_t ns);

// sorted[0..ns) = idx[0..ns) ordered by the Hilbert-curve index of (x, y, z) * inv_a.  z may be NULL
// (planar particles).  Enqueued on `stream`; no allocation.
int curve_sort(cudaStream_t stream, int64_t ns, const int32_t* idx, const double* x, const double* y,
                const double* z, double inv_a, void* scratch, size_t scratch_bytes, int32_t* sorted);

// Hilbert-curve order within groups (ensemble instances): entries are ordered by group first, then
// by the Hilbert-curve index of (x, y, z) * inv_a[group]; idx/grp are the particle and group of each
// entry.  n_groups < 2^33.
size_t grouped_curve_sort_bytes(int64_t ns, int n_groups);
int grouped_curve_sort(cudaStream_t stream, int64_t ns, int n_groups, const int32_t* idx, const int32_t* grp,
                        const double* x, const double* y, const double* z, const double* inv_a, void* scratch,
                        size_t scratch_bytes, int32_t* sorted);

// Planar sources: sorted[0..ns) = idx[0..ns) ordered along a 2-D Hilbert curve over the
// sources' bounding box.
size_t curve_sort2d_bytes(int64_t ns);
int curve_sort2d(cudaStream_t stream, int64_t ns, const int32_t* idx, const double* x, const double* y,
                 void* scratch, size_t scratch_bytes, int32_t* sorted);

// out[0..ns) = the entries of order[0..n) (a permutation of the particles 0..n-1) that are
// listed in idx[0..ns) (the active particles, distinct), in the order of `order`: the active
// particles in the curve order of all of them, without a second sort.  Scratch:
// select_in_order_bytes(n) bytes.
size_t select_in_order_bytes(int64_t n);
int select_in_order(cudaStream_t stream, int64_t n, const int32_t* order, int64_t ns, const int32_t* idx,
                    void* scratch, size_t scratch_bytes, int32_t* out);

}  // namespace lpm
