// engine.cuh -- the tiled all-pairs sweep shared by every direct sum.
//
// Layout: sources are compacted (active particles only, ascending particle index) into an
// array of fixed-size records, padded with inert records to a multiple of the tile size.
// A CTA owns a block of targets (held in registers) and a contiguous range of source tiles
// (one split-K chunk).  Tiles are staged into shared memory by 1-D TMA bulk copies
// (cp.async.bulk) on a two-stage mbarrier pipeline; every thread then sweeps the tile with
// broadcast shared-memory reads.  Each wait on a tile is bounded (~1 s) and a block-wide
// vote makes all threads leave together if one gives up, so a lost copy cannot hang the GPU.
#pragma once

#include <type_traits>

#include "lpm_common.cuh"

namespace lpm {

// Sources per FP32 partial of an operator: Op::kFlush if it defines one, else a whole tile.
template <class Op, class = void>
struct FlushOf {
  static constexpr int value = 0;
};
template <class Op>
struct FlushOf<Op, std::void_t<decltype(Op::kFlush)>> {
  static constexpr int value = Op::kFlush;
};

// Whether an operator evaluates two targets at once (Op::interact2, packed FP32x2 math).
template <class Op, class = void>
struct PairsOf {
  static constexpr bool value = false;
};
template <class Op>
struct PairsOf<Op, std::void_t<decltype(Op::kPairs)>> {
  static constexpr bool value = Op::kPairs;
};

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

// Arguments of the compensated FP32 sweep.
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

// Compensated FP32 sweep: each thread owns TPT targets; pair terms are summed in FP32 per
// tile (or per Op::kFlush sources) and each partial is added into a (hi, lo) pair with
// TwoSum; the per-chunk result hi + lo is written in FP64 for the cross-chunk reduction.
template <class Op, int THREADS, int TPT, int TILE, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) sweep_fp32c_kernel(SweepArgs<Op> a) {
  using Rec = typename Op::Rec;
  constexpr int NC = Op::NC;
  __shared__ __align__(128) Rec stage[2][TILE];
  __shared__ __align__(8) uint64_t bars[2];

  const int64_t chunk = blockIdx.y;
  const int64_t tile0 = chunk * a.tiles_per_chunk;
  int64_t ntl = a.n_tiles - tile0;
  if (ntl > a.tiles_per_chunk) ntl = a.tiles_per_chunk;
  if (ntl < 0) ntl = 0;

  typename Op::Tgt tg[TPT];
  float hi[TPT][NC], lo[TPT][NC];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT) + threadIdx.x;
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    int64_t il = base + t * THREADS;
    if (il >= a.nt) il = a.nt - 1;  // duplicate a valid target; its result is not stored
    tg[t] = Op::load_target(a.p, a.ib + il);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      hi[t][c] = 0.0f;
      lo[t][c] = 0.0f;
    }
  }

  pipe_init(bars);
  uint32_t g = 0;
  constexpr int FL = (FlushOf<Op>::value > 0 && FlushOf<Op>::value < TILE) ? FlushOf<Op>::value : TILE;
  static_assert(TILE % FL == 0, "flush interval must divide the tile");
  staged_sweep<Rec, TILE>(a.src, tile0, ntl, stage[0], stage[1], bars, g, a.status,
                          [&](const Rec* tile) {
#pragma unroll 1
                            for (int j0 = 0; j0 < TILE; j0 += FL) {
                              float acc[TPT][NC];
#pragma unroll
                              for (int t = 0; t < TPT; ++t)
#pragma unroll
                                for (int c = 0; c < NC; ++c) acc[t][c] = 0.0f;
#pragma unroll 4
                              for (int j = j0; j < j0 + FL; ++j) {
                                const Rec r = tile[j];
                                if constexpr (PairsOf<Op>::value) {
                                  static_assert(TPT % 2 == 0, "targets come in pairs");
#pragma unroll
                                  for (int t = 0; t < TPT; t += 2) Op::interact2(tg[t], tg[t + 1], r, acc[t], acc[t + 1]);
                                } else {
#pragma unroll
                                  for (int t = 0; t < TPT; ++t) Op::interact(tg[t], r, acc[t]);
                                }
                              }
#pragma unroll
                              for (int t = 0; t < TPT; ++t)
#pragma unroll
                                for (int c = 0; c < NC; ++c) comp_add(hi[t][c], lo[t][c], acc[t][c]);
                            }
                          });

#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int64_t il = base + t * THREADS;
    if (il < a.nt) {
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        a.partial[(chunk * NC + c) * a.nt + il] =
            static_cast<double>(hi[t][c]) + static_cast<double>(lo[t][c]);
      }
    }
  }
}

}  // namespace lpm
