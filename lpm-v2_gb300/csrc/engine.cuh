// engine.cuh -- the tile pipeline shared by every FP32C sweep.
//
// Layout: sources are compacted (active particles only) into an array of fixed-size
// records, padded with inert records to a multiple of the tile size.  A CTA owns a block of
// targets (held in registers) and a contiguous range of source tiles (one split-K chunk).
// Tiles are staged into shared memory by 1-D TMA bulk copies (cp.async.bulk) on a two-stage
// mbarrier pipeline (staged_sweep); every thread then sweeps the tile with broadcast
// shared-memory reads.  Each wait on a tile is bounded (~1 s) and a block-wide
// vote makes all threads leave together if one gives up, so a lost copy cannot hang the GPU.
#pragma once

#include "lpm_common.cuh"

namespace lpm {

// Initialises the two stage barriers of a TMA pipeline (once per CTA).
__device__ __forceinline__ void pipe_init(uint64_t* bars) {
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
}

// Two-stage TMA pipeline over tiles [tile0, tile0 + ntl) of `src`.  body(const Rec* tile)
// is called once per tile by every thread of the block.  `g` counts the tiles this CTA has
// pushed through the pipeline so far (identical in every thread): tile g uses stage g & 1
// and completes phase (g >> 1) & 1 of that stage's barrier, so one CTA can run many sweeps
// (a persistent kernel) on barriers initialised once.  Returns false on a timeout.
template <class Rec, int TILE, class Body>
__device__ __forceinline__ bool staged_sweep(const Rec* __restrict__ src, int64_t tile0,
                                             int64_t ntl, Rec* stage0, Rec* stage1,
                                             uint64_t* bars, uint32_t& g, int* status, Body&& body) {
  constexpr uint32_t kBytes = TILE * sizeof(Rec);
  static_assert(kBytes % 16 == 0, "tile bytes must be a multiple of 16");
  if (threadIdx.x == 0) {
    for (int64_t k = 0; k < ntl && k < 2; ++k) {
      const uint32_t gk = g + static_cast<uint32_t>(k);
      mbar_arrive_expect_tx(&bars[gk & 1u], kBytes);
      tma_load_1d((gk & 1u) ? stage1 : stage0, src + (tile0 + k) * TILE, kBytes, &bars[gk & 1u]);
    }
  }
  bool ok = true;
  int64_t k = 0;
  for (; k < ntl; ++k) {
    const uint32_t gk = g + static_cast<uint32_t>(k);
    const int s = static_cast<int>(gk & 1u);
    const uint32_t phase = (gk >> 1) & 1u;
    const bool mine = mbar_wait_bounded(&bars[s], phase, status);
    if (!__syncthreads_and(mine)) {
      ok = false;
      break;
    }
    body(s ? stage1 : stage0);
    __syncthreads();  // every thread is done with stage s
    if (threadIdx.x == 0 && k + 2 < ntl) {
      mbar_arrive_expect_tx(&bars[s], kBytes);
      tma_load_1d(s ? stage1 : stage0, src + (tile0 + k + 2) * TILE, kBytes, &bars[s]);
    }
  }
  if (!ok && threadIdx.x == 0) {
    // let copies that are still in flight land before the CTA moves on (bounded again)
    for (int64_t kk = k; kk < ntl && kk < k + 2; ++kk) {
      const uint32_t gk = g + static_cast<uint32_t>(kk);
      mbar_wait_bounded(&bars[gk & 1u], (gk >> 1) & 1u, status);
    }
  }
  g += static_cast<uint32_t>(ntl);
  return ok;
}

// Arguments of a compensated FP32 sweep (targets, records, split-K partials).
template <class Op>
struct SweepArgs {
  typename Op::Params p;
  const typename Op::Rec* src;  // padded to n_tiles * TILE records
  int64_t n_tiles;
  int64_t tiles_per_chunk;
  int64_t ib;         // first target (0-based particle index)
  int64_t nt;         // number of targets
  double* partial;    // [gridDim.y][Op::NC][nt]
  int* status;
};

}  // namespace lpm
