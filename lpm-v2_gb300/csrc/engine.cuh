// engine.cuh -- the tile pipelines shared by the direct sums.
//
// Layout: sources are compacted (active particles only) into an array of fixed-size
// records, padded with inert records to a multiple of the tile size.  A CTA owns a block of
// targets (held in registers) and a contiguous range of source tiles (one split-K chunk) --
// or, for the sums with a distance cutoff, a round-robin share of the tiles within reach of
// its targets (sweep_culled_share, at the end of this file).
// Tiles are staged into shared memory by 1-D TMA bulk copies (cp.async.bulk), and every
// thread then sweeps a tile with broadcast shared-memory reads.  Two pipelines:
//  - staged_sweep: two stages, block-synchronous (every warp finishes a tile before its stage
//    is refilled; two block barriers per tile);
//  - warp_sweep / warp_sweep_tiles: S stages, warp-decoupled, over a contiguous range or a
//    list of tiles.  Each stage has a "full" mbarrier (the copy's
//    transaction count) and an "empty" one (one arrival per warp when it is done with the
//    tile).  Thread 0 refills a stage as soon as every warp has released it, so warps that
//    skip a tile's work run ahead by up to S - 1 tiles instead of waiting at a barrier.
// Every wait is bounded (WaitCfg::ns, 1 s by default); a thread that gives up records
// kDevTimeout in the device status word, its warp (or block) leaves the sweep, and copies
// still in flight are waited for (bounded again) before the CTA moves on, so a lost copy
// cannot hang the GPU.
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
                                             uint64_t* bars, uint32_t& g, int* status, const WaitCfg& w,
                                             Body&& body) {
  constexpr uint32_t kBytes = TILE * sizeof(Rec);
  static_assert(kBytes % 16 == 0, "tile bytes must be a multiple of 16");
  if (threadIdx.x == 0) {
    for (int64_t k = 0; k < ntl && k < 2; ++k) {
      const uint32_t gk = g + static_cast<uint32_t>(k);
      if (tile0 + k == w.skip_tile) continue;
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
    const bool mine = mbar_wait_bounded(&bars[s], phase, status, w.ns);
    if (!__syncthreads_and(mine)) {
      ok = false;
      break;
    }
    body(s ? stage1 : stage0);
    __syncthreads();  // every thread is done with stage s
    if (threadIdx.x == 0 && k + 2 < ntl && tile0 + k + 2 != w.skip_tile) {
      mbar_arrive_expect_tx(&bars[s], kBytes);
      tma_load_1d(s ? stage1 : stage0, src + (tile0 + k + 2) * TILE, kBytes, &bars[s]);
    }
  }
  if (!ok && threadIdx.x == 0) {
    // let copies that are still in flight land before the CTA moves on (bounded again)
    for (int64_t kk = k; kk < ntl && kk < k + 2; ++kk) {
      if (tile0 + kk == w.skip_tile) continue;  // never issued
      const uint32_t gk = g + static_cast<uint32_t>(kk);
      mbar_wait_bounded(&bars[gk & 1u], (gk >> 1) & 1u, status, w.ns);
    }
  }
  g += static_cast<uint32_t>(ntl);
  return ok;
}

template <class Rec, int TILE, class Body>
__device__ __forceinline__ bool staged_sweep(const Rec* __restrict__ src, int64_t tile0,
                                             int64_t ntl, Rec* stage0, Rec* stage1,
                                             uint64_t* bars, uint32_t& g, int* status, Body&& body) {
  return staged_sweep<Rec, TILE>(src, tile0, ntl, stage0, stage1, bars, g, status, default_wait(),
                                 static_cast<Body&&>(body));
}

// Shared memory of an S-stage warp-decoupled pipeline.  With NSIDE > 0 each stage also holds
// the tile's NSIDE side records (e.g. its group origins), copied with the tile, so that a warp
// reads them from shared memory rather than waiting on a global load per group.
template <class Rec, int TILE, int S, class Side = Rec, int NSIDE = 0>
struct __align__(128) TilePipe {
  Rec stage[S][TILE];
  Side side[S][NSIDE > 0 ? NSIDE : 1];
  uint64_t full[S];   // completes when tile data has landed (1 arrival + the copies' bytes)
  uint64_t empty[S];  // completes when every warp is done with the stage (one arrival per warp)
};

template <class Rec, int TILE, int S, class Side, int NSIDE>
__device__ __forceinline__ void tile_pipe_init(TilePipe<Rec, TILE, S, Side, NSIDE>& pp) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&pp.full[s], 1);
      mbar_init(&pp.empty[s], blockDim.x / 32);
    }
    fence_mbar_init();
  }
  __syncthreads();
}

// S-stage warp-decoupled sweep over ntl tiles of `src`, the k-th being tile tile_of(k):
// body(const Rec*) runs once per tile in every warp, each warp at its own pace.  `g` counts
// the tiles this CTA has pushed through the pipeline (identical in every thread): tile number
// q uses stage q % S, whose full barrier completes phase (q / S) & 1 for it and whose empty
// barrier completes phase (q / S) & 1 when every warp has released it.  Thread 0 (a consumer
// too) issues the copies: before each of its tiles it refills every stage already released,
// keeping up to S tiles in flight, and it blocks (bounded) on a release only when the tile
// it needs next has not been issued.  Returns false in every thread when any wait gave up;
// the stages' barrier phases are then no longer in step with `g`, so the CTA must not sweep
// again.  With NSIDE > 0 the side records of tile t are side_src[t * NSIDE .. (t + 1) *
// NSIDE) and body(const Rec*, const Side*) gets both; otherwise body(const Rec*).
template <class Rec, int TILE, int S, class Side, int NSIDE, class TileOf, class Body>
__device__ __forceinline__ bool warp_sweep_tiles(const Rec* __restrict__ src, TileOf&& tile_of, int64_t ntl,
                                                 TilePipe<Rec, TILE, S, Side, NSIDE>& pp, uint32_t& g, int* status,
                                                 const WaitCfg& w, const Side* __restrict__ side_src, Body&& body) {
  constexpr uint32_t kBytes = TILE * sizeof(Rec);
  constexpr uint32_t kSideBytes = NSIDE * sizeof(Side);
  static_assert(kBytes % 16 == 0 && kSideBytes % 16 == 0, "copies must be multiples of 16 bytes");
  static_assert(S >= 2, "at least two stages");
  const bool producer = threadIdx.x == 0;
  int64_t next = 0;  // next tile to issue (thread 0)
  bool ok = true;    // thread 0: no wait for a release gave up
  // Issues tile kk if its stage is free: waits (bounded) for the release when `block`,
  // otherwise probes once.  Returns 1 when issued, 0 when not yet free, -1 on a timeout.
  auto issue = [&](int64_t kk, bool block) -> int {
    const uint32_t q = g + static_cast<uint32_t>(kk);
    const uint32_t s = q % S;
    if (q >= static_cast<uint32_t>(S)) {
      const uint32_t ph = ((q - S) / S) & 1u;
      if (block) {
        if (!mbar_wait_bounded(&pp.empty[s], ph, status, w.ns)) return -1;
      } else if (!mbar_try_wait(&pp.empty[s], ph)) {
        return 0;
      }
    }
    const int64_t t = tile_of(kk);
    if (t != w.skip_tile) {
      mbar_arrive_expect_tx(&pp.full[s], kBytes + kSideBytes);
      tma_load_1d(pp.stage[s], src + t * TILE, kBytes, &pp.full[s]);
      if constexpr (NSIDE > 0) tma_load_1d(pp.side[s], side_src + t * NSIDE, kSideBytes, &pp.full[s]);
    }
    return 1;
  };
  int64_t k = 0;
  for (; k < ntl; ++k) {
    if (producer && ok) {
      while (next < ntl && next < k + S) {
        const int r = issue(next, next <= k);
        if (r < 0) ok = false;
        if (r <= 0) break;
        ++next;
      }
    }
    const uint32_t q = g + static_cast<uint32_t>(k);
    const uint32_t s = q % S;
    const bool mine = ok && mbar_wait_bounded(&pp.full[s], (q / S) & 1u, status, w.ns);
    if (!__all_sync(0xffffffffu, mine)) break;
    if constexpr (NSIDE > 0) {
      body(pp.stage[s], pp.side[s]);
    } else {
      body(pp.stage[s]);
    }
    __syncwarp();
    if ((threadIdx.x & 31u) == 0u) mbar_arrive(&pp.empty[s]);
  }
  const bool all = __syncthreads_and(k == ntl);
  if (!all && producer) {
    // copies issued for tiles this warp did not wait for must land before the CTA moves on
    // (bounded again); tiles below k completed, every stage before them too
    for (int64_t kk = k; kk < next; ++kk) {
      if (tile_of(kk) == w.skip_tile) continue;  // never issued
      const uint32_t q = g + static_cast<uint32_t>(kk);
      mbar_wait_bounded(&pp.full[q % S], (q / S) & 1u, status, w.ns);
    }
  }
  g += static_cast<uint32_t>(ntl);
  return all;
}

// The sweep over the contiguous tiles [tile0, tile0 + ntl).
template <class Rec, int TILE, int S, class Side, int NSIDE, class Body>
__device__ __forceinline__ bool warp_sweep(const Rec* __restrict__ src, int64_t tile0, int64_t ntl,
                                           TilePipe<Rec, TILE, S, Side, NSIDE>& pp, uint32_t& g, int* status,
                                           const WaitCfg& w, const Side* __restrict__ side_src, Body&& body) {
  return warp_sweep_tiles(src, [tile0](int64_t k) { return tile0 + k; }, ntl, pp, g, status, w, side_src,
                          static_cast<Body&&>(body));
}

// ---------------------------------------------------------------- tile culling (cutoff sums)
// For the sums with a distance cutoff every CTA of a target block lists the tiles of the whole
// source range that lie within reach of its targets -- one test per tile, of the tile's ball
// (written by the prep kernel) against the ball around the CTA's targets -- and CTA (block, c)
// sweeps the c-th of gridDim.y equal shares of that list (warp_sweep_tiles over it), so the
// work of a block is split evenly among its CTAs wherever its tiles lie.  The test is
// conservative against the warps' own per-group test, so every tile left out is one every
// warp would have skipped: the sums are unchanged, the copies and per-group tests of those
// tiles saved.

// A ball around a CTA's targets: the centroid of the points and the largest distance to it.
struct TargetBall {
  float cx, cy, cz, r;
};

// Every thread passes its NPT points (hi parts of the positions the warps test with); the
// ball is written to `out` (shared memory, so that it holds no registers during the sweep),
// visible to every thread on return.
template <int THREADS, int NPT>
__device__ __forceinline__ void cta_target_ball(const float (&px)[NPT], const float (&py)[NPT], const float (&pz)[NPT],
                                                TargetBall& out) {
  static_assert(THREADS % 32 == 0 && THREADS <= 1024, "whole warps");
  constexpr int NW = THREADS / 32;
  __shared__ float red[4][NW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
  for (int k = 0; k < NPT; ++k) {
    sx += px[k];
    sy += py[k];
    sz += pz[k];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
    sz += __shfl_xor_sync(0xffffffffu, sz, o);
  }
  if (lane == 0) {
    red[0][wid] = sx;
    red[1][wid] = sy;
    red[2][wid] = sz;
  }
  __syncthreads();
  TargetBall b;
  sx = sy = sz = 0.f;
#pragma unroll
  for (int k = 0; k < NW; ++k) {
    sx += red[0][k];
    sy += red[1][k];
    sz += red[2][k];
  }
  constexpr float inv = 1.f / static_cast<float>(THREADS * NPT);
  b.cx = sx * inv;
  b.cy = sy * inv;
  b.cz = sz * inv;
  float m = 0.f;
#pragma unroll
  for (int k = 0; k < NPT; ++k) {
    const float dx = px[k] - b.cx, dy = py[k] - b.cy, dz = pz[k] - b.cz;
    const float d2 = dx * dx + dy * dy + dz * dz;
    m = d2 > m ? d2 : (d2 == d2 ? m : __int_as_float(0x7f800000));  // a NaN point: infinite ball
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) red[3][wid] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    m = 0.f;
#pragma unroll
    for (int k = 0; k < NW; ++k) m = fmaxf(m, red[3][k]);
    b.r = sqrtf(m);
    out = b;
  }
  __syncthreads();
}

// The ball of a tile from its GPT groups' balls (centre hi parts, radius; w < 0 marks an empty
// group): centre the mean of the groups' centres, radius the largest distance to a group's
// centre plus that group's radius, widened by 1e-5 of itself and 1e-6 of the centre's size for
// the rounding of the hi parts.  Every source of the tile lies in it.
template <int GPT>
__device__ __forceinline__ float4 tile_ball_from_groups(const float4 (&grp)[GPT]) {
  float cx = 0.f, cy = 0.f, cz = 0.f, n = 0.f;
#pragma unroll
  for (int g = 0; g < GPT; ++g) {
    if (grp[g].w >= 0.f) {
      cx += grp[g].x;
      cy += grp[g].y;
      cz += grp[g].z;
      n += 1.f;
    }
  }
  if (n > 0.f) {
    cx /= n;
    cy /= n;
    cz /= n;
  }
  float r = 0.f;
#pragma unroll
  for (int g = 0; g < GPT; ++g) {
    if (grp[g].w >= 0.f) {
      const float dx = grp[g].x - cx, dy = grp[g].y - cy, dz = grp[g].z - cz;
      const float e = sqrtf(dx * dx + dy * dy + dz * dz) + grp[g].w;
      r = e > r ? e : (e == e ? r : __int_as_float(0x7f800000));  // NaN: an infinite ball
    }
  }
  r = r * 1.00001f + 1e-6f * (1.f + fabsf(cx) + fabsf(cy) + fabsf(cz));
  return make_float4(cx, cy, cz, r);
}

// Whether a tile's ball is within reach of a CTA's ball: the distance of the centres is below
// the two radii plus c_cut, widened by 1e-4 of that and by 1e-5 of the coordinates' size for
// the rounding of the hi parts (NaN reads as in reach).
__device__ __forceinline__ bool tile_in_reach(const float4& tb, const TargetBall& b, float c_cut) {
  const float dx = tb.x - b.cx, dy = tb.y - b.cy, dz = tb.z - b.cz;
  const float lim = (b.r + tb.w + c_cut) * 1.0001f + 1e-5f * (1.f + fabsf(b.cx) + fabsf(b.cy) + fabsf(b.cz));
  return !(dx * dx + dy * dy + dz * dz >= lim * lim);
}

// One window of THREADS tiles, t0 .. t0 + n - 1 (n <= THREADS), one per thread: counts the
// tiles in reach, and lists (in tile order, into list[0..kept)) those whose rank in the whole
// in-reach list -- rank0 for the window's first -- is share modulo shares.  wcount is shared
// scratch of THREADS / 32 ints.  Every thread gets the same counts.
struct CullCount {
  int in_reach, kept;
};

template <int THREADS, class InReach>
__device__ __forceinline__ CullCount cull_window(int64_t t0, int n, InReach&& in_reach, int64_t rank0, int64_t shares,
                                                 int64_t share, int32_t* list, int* wcount) {
  static_assert(THREADS % 32 == 0 && THREADS <= 1024, "whole warps");
  constexpr int NW = THREADS / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const bool f = static_cast<int>(threadIdx.x) < n && in_reach(t0 + threadIdx.x);
  const unsigned m = __ballot_sync(0xffffffffu, f);
  if (lane == 0) wcount[wid] = __popc(m);
  __syncthreads();
  int before = 0, total = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    const int c = wcount[w];
    before += w < wid ? c : 0;
    total += c;
  }
  const int64_t rank = rank0 + before + __popc(m & ((1u << lane) - 1u));
  // the first rank >= rank0 of this share; the share's ranks follow every `shares`
  const int64_t first = rank0 + ((share - rank0 % shares) % shares + shares) % shares;
  if (f && rank % shares == share) list[(rank - first) / shares] = static_cast<int32_t>(t0 + threadIdx.x);
  const int64_t end = rank0 + total;
  __syncthreads();  // the list is complete and wcount free for the next window
  return CullCount{total, end > first ? static_cast<int>((end - 1 - first) / shares + 1) : 0};
}

// The share of the in-reach tiles for CTA (blockIdx.x, blockIdx.y): every gridDim.y-th tile
// of the block's in-reach list, starting at the blockIdx.y-th (equal counts to within one,
// in one scan of the tile balls).  Lists them a window at a time and calls sweep(list,
// count) for each non-empty window; stops early when sweep returns false (a wait gave up).
// in_reach(t) tests tile t.
template <int THREADS, class InReach, class Sweep>
__device__ __forceinline__ void sweep_culled_share(int64_t n_tiles, InReach&& in_reach, Sweep&& sweep) {
  __shared__ int32_t list[THREADS];
  __shared__ int wcount[THREADS / 32];
  const int64_t shares = gridDim.y, share = blockIdx.y;
  int64_t rank0 = 0;
  for (int64_t w0 = 0; w0 < n_tiles; w0 += THREADS) {
    const int n = static_cast<int>(n_tiles - w0 < THREADS ? n_tiles - w0 : THREADS);
    const CullCount cc = cull_window<THREADS>(w0, n, in_reach, rank0, shares, share, list, wcount);
    rank0 += cc.in_reach;
    if (cc.kept > 0 && !sweep(static_cast<const int32_t*>(list), cc.kept)) break;
  }
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
  WaitCfg wait = default_wait();
};

}  // namespace lpm
