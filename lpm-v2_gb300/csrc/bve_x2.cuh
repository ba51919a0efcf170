// bve_x2.cuh -- the sphere-BVE FP32C sweep on packed FP32x2 arithmetic (FFMA2/FADD2/FMUL2).
//
// Blackwell executes two FP32 lanes per instruction with the packed f32x2 operations
// (__ffma2_rn, __fadd2_rn, __fmul2_rn).  Each takes both halves of the FP32 pipe for two
// cycles, so the pipe's lane rate is that of scalar FFMA, but the packed form needs half
// the issue slots, which keeps the sweep bound by the pipe.  This kernel pairs two targets
// per float2: every thread owns TPT targets as TPT/2 pairs, and each pair
// interacts with one source in 17 packed operations + 2 MUFU.RCP.  Source records are stored
// pre-negated and replicated into both halves of each float2, so shared-memory loads feed
// the packed operations directly.
//
// The arithmetic is that of BveF32 (ops.cuh): d = p_i - p_j from hi/lo positions,
// q = |d|^2 - c_i - c_j, weight S_j / q, D += weight * d, u = D x p_i in the FP64 finish.
#pragma once

#include "engine.cuh"
#include "ops.cuh"

namespace lpm {

struct BveX2 {
  static constexpr int NC = 3;
  struct __align__(16) Rec {
    float4 a;  // -xh, -xh, -yh, -yh
    float4 b;  // -zh, -zh, -xl, -xl
    float4 c;  // -yl, -yl, -zl, -zl
    float4 d;  // -c_j, -c_j, S_j, S_j
  };
  struct Pair {
    float2 xh, yh, zh, xl, yl, zl, nc;
  };
};

__device__ __forceinline__ float2 lo2(const float4& v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4& v) { return make_float2(v.z, v.w); }

template <int THREADS, int TPT, int TILE, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) bve_sweep_x2_kernel(SweepArgs<BveF32> a) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  constexpr int NP = TPT / 2;
  using Rec = BveX2::Rec;
  __shared__ __align__(128) Rec stage[2][TILE];
  __shared__ __align__(8) uint64_t bars[2];

  const int64_t chunk = blockIdx.y;
  const int64_t tile0 = chunk * a.tiles_per_chunk;
  int64_t ntl = a.n_tiles - tile0;
  if (ntl > a.tiles_per_chunk) ntl = a.tiles_per_chunk;
  if (ntl < 0) ntl = 0;

  BveX2::Pair pr[NP];
  float2 hx[NP], hy[NP], hz[NP], lx[NP], ly[NP], lz[NP];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT) + threadIdx.x;
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    int64_t i0 = base + (2 * p) * THREADS, i1 = base + (2 * p + 1) * THREADS;
    if (i0 >= a.nt) i0 = a.nt - 1;  // duplicates of a valid target; results not stored
    if (i1 >= a.nt) i1 = a.nt - 1;
    const BveF32::Tgt t0 = BveF32::load_target(a.p, a.ib + i0);
    const BveF32::Tgt t1 = BveF32::load_target(a.p, a.ib + i1);
    pr[p].xh = make_float2(t0.xh, t1.xh);
    pr[p].yh = make_float2(t0.yh, t1.yh);
    pr[p].zh = make_float2(t0.zh, t1.zh);
    pr[p].xl = make_float2(t0.xl, t1.xl);
    pr[p].yl = make_float2(t0.yl, t1.yl);
    pr[p].zl = make_float2(t0.zl, t1.zl);
    pr[p].nc = make_float2(t0.nc, t1.nc);
    hx[p] = hy[p] = hz[p] = lx[p] = ly[p] = lz[p] = make_float2(0.f, 0.f);
  }

  pipe_init(bars);
  uint32_t g = 0;
  const Rec* src = reinterpret_cast<const Rec*>(a.src);
  staged_sweep<Rec, TILE>(src, tile0, ntl, stage[0], stage[1], bars, g, a.status, [&](const Rec* tile) {
    float2 ax[NP], ay[NP], az[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) ax[p] = ay[p] = az[p] = make_float2(0.f, 0.f);
#pragma unroll 2
    for (int j = 0; j < TILE; ++j) {
      const float4 ra = tile[j].a, rb = tile[j].b, rc = tile[j].c, rd = tile[j].d;
      const float2 nxh = lo2(ra), nyh = hi2(ra), nzh = lo2(rb), nxl = hi2(rb), nyl = lo2(rc), nzl = hi2(rc);
      const float2 ncj = lo2(rd), s2 = hi2(rd);
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const float2 dx = __fadd2_rn(__fadd2_rn(pr[p].xh, nxh), __fadd2_rn(pr[p].xl, nxl));
        const float2 dy = __fadd2_rn(__fadd2_rn(pr[p].yh, nyh), __fadd2_rn(pr[p].yl, nyl));
        const float2 dz = __fadd2_rn(__fadd2_rn(pr[p].zh, nzh), __fadd2_rn(pr[p].zl, nzl));
        float2 q = __fadd2_rn(pr[p].nc, ncj);
        q = __ffma2_rn(dx, dx, q);
        q = __ffma2_rn(dy, dy, q);
        q = __ffma2_rn(dz, dz, q);
        const float2 inv = make_float2(rcp_approx(q.x), rcp_approx(q.y));
        const float2 wgt = __fmul2_rn(s2, inv);
        ax[p] = __ffma2_rn(wgt, dx, ax[p]);
        ay[p] = __ffma2_rn(wgt, dy, ay[p]);
        az[p] = __ffma2_rn(wgt, dz, az[p]);
      }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      comp_add(hx[p].x, lx[p].x, ax[p].x);
      comp_add(hx[p].y, lx[p].y, ax[p].y);
      comp_add(hy[p].x, ly[p].x, ay[p].x);
      comp_add(hy[p].y, ly[p].y, ay[p].y);
      comp_add(hz[p].x, lz[p].x, az[p].x);
      comp_add(hz[p].y, lz[p].y, az[p].y);
    }
  });

#pragma unroll
  for (int p = 0; p < NP; ++p) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t il = base + (2 * p + h) * THREADS;
      if (il < a.nt) {
        const float vx = h ? hx[p].y : hx[p].x, ex = h ? lx[p].y : lx[p].x;
        const float vy = h ? hy[p].y : hy[p].x, ey = h ? ly[p].y : ly[p].x;
        const float vz = h ? hz[p].y : hz[p].x, ez = h ? lz[p].y : lz[p].x;
        a.partial[(chunk * 3 + 0) * a.nt + il] = static_cast<double>(vx) + static_cast<double>(ex);
        a.partial[(chunk * 3 + 1) * a.nt + il] = static_cast<double>(vy) + static_cast<double>(ey);
        a.partial[(chunk * 3 + 2) * a.nt + il] = static_cast<double>(vz) + static_cast<double>(ez);
      }
    }
  }
}

}  // namespace lpm
