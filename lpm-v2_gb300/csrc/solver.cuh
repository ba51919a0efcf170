// solver.cuh -- ownership helpers shared by the device-resident solvers and the ensemble.
#pragma once

#include <vector>

#include "lpm_common.cuh"
#include "sums.cuh"

namespace lpm {

// Device allocations owned by one handle, freed together.
struct DeviceArena {
  std::vector<void*> ptrs;
  int alloc(size_t bytes, void** p);
  void free(void* p);  // one allocation (no-op for nullptr)
  void release();
};

// The scratch of one direct sum (source records + split-K partials), sized once so that
// the launches can be captured into a CUDA graph.
struct SumScratch {
  SumPlan plan;
  void* src_buf = nullptr;
  double* partial = nullptr;
  size_t src_cap = 0, partial_cap = 0;  // allocated bytes
  int init(DeviceArena& arena, int kind, int mode, int64_t ns, int64_t nt, int sm_count);
  // Makes the buffers hold plan_sum_max(kind, mode, ns, nt) (growing them if needed) and
  // sets plan to it.
  int fit(DeviceArena& arena, int kind, int mode, int64_t ns, int64_t nt, int sm_count);
};

// Number of kernel nodes in a captured graph: the kernels one replay launches.
int64_t graph_kernel_nodes(cudaGraph_t graph);

// Indices of the active particles, ascending.
std::vector<int32_t> active_list(int64_t n, const int32_t* active);

}  // namespace lpm
