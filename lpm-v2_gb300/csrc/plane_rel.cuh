// plane_rel.cuh -- the planar Biot-Savart FP32C sweep on spatially sorted sources in
// group-relative coordinates (7 packed FP32x2 operations per target pair and source).
//
// Reference: planarIncompressibleVelocity, src/PlaneIncompressibleSolver.f90:291-308:
//   u_i = -sum_j S_j (y_i - y_j) / (r^2 + delta^2),  v_i = sum_j S_j (x_i - x_j) / (r^2 + delta^2)
// with S_j = omega_j A_j / (2 pi) (delta = 0 in the reference, delta > 0 the regularised
// extension).  The structure is that of the sphere sweep (bve_rel.cuh): sources in 2-D
// Hilbert-curve order (sort.cu), each group of kGroup sources stored relative to its
// centroid o as rel2(p, o) with the group radius R, and per warp and group a far form
// d = t_hi - s_hi (every target at |t - o| >= 3R: relative error <= ~2^-23) or a near form
// in which each target forms (t_hi, t_lo) = rel2(t, o) with the sources' operations and
// keeps the lo parts (a self pair cancels bit for bit; delta^2 carries a 2^-100 offset so
// that the self weight is finite).  Per target pair and source, far:
//   d (2 FADD2), q = d.d + delta^2 (2 FFMA2), w = S rcp(q) (FMUL2 + 2 MUFU),
//   U += w dy, V += w dx (2 FFMA2);
// near: 4 more FADD2.  Each group's terms are summed in FP32 on their own and added to the
// tile's FP32 partial (2 FADD2 per group), which goes into compensated (hi, lo) pairs; the
// FP64 finish reduces the split-K chunks and sets u = -U, v = V.
#pragma once

#include "bve_x2.cuh"
#include "bve_rel.cuh"
#include "engine.cuh"
#include "ops.cuh"

namespace lpm {

struct PlaneRel {
  struct __align__(16) Rec {
    float4 a;  // -sx_hi, -sx_hi, -sy_hi, -sy_hi
    float4 b;  // S_j, S_j, -sx_lo, -sx_lo
    float4 c;  // -sy_lo, -sy_lo, 0, 0
  };
  struct __align__(16) Origin {
    float4 o;  // o_hi.x, o_hi.y, o_lo.x, o_lo.y
    float4 f;  // R (the group radius about o), S_g hi, S_g lo (S_g = sum of the group's S_j), 0
  };
  struct Pair {
    float2 xh, yh, xl, yl;
  };
  // sources per origin: 128 (the planar velocity, stream-function and SWE sweeps measured 0.2-2 %
  // faster than with 64)
  static constexpr int kGroup = 128;
  static constexpr float kNearFactor = 3.0f;  // near: |t - o| < kNearFactor R
};

struct PlaneRelArgs {
  const double *x, *y;
  float d2;  // delta^2 + 2^-100
  const PlaneRel::Rec* src;
  const PlaneRel::Origin* org;
  int64_t n_tiles, tiles_per_chunk, ib, nt;
  double* partial;  // [chunk][2][nt]
  int* status;
};

template <int THREADS, int TPT, int TILE, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) plane_rel_sweep_kernel(PlaneRelArgs a) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  static_assert(TILE % PlaneRel::kGroup == 0, "whole origin groups per tile");
  constexpr int NP = TPT / 2;
  constexpr int G = PlaneRel::kGroup;
  constexpr int GPT = TILE / G;
  using Rec = PlaneRel::Rec;
  __shared__ __align__(128) Rec stage[2][TILE];
  __shared__ __align__(8) uint64_t bars[2];

  const int64_t chunk = blockIdx.y;
  const int64_t tile0 = chunk * a.tiles_per_chunk;
  int64_t ntl = a.n_tiles - tile0;
  if (ntl > a.tiles_per_chunk) ntl = a.tiles_per_chunk;
  if (ntl < 0) ntl = 0;

  PlaneRel::Pair pr[NP];
  float2 hu[NP], hv[NP], lu[NP], lv[NP];
  const int64_t first = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT);
  const int64_t count = a.nt - first < THREADS * TPT ? a.nt - first : THREADS * TPT;
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    int64_t i0 = (2 * p) * THREADS + threadIdx.x, i1 = (2 * p + 1) * THREADS + threadIdx.x;
    if (i0 >= count) i0 = count - 1;  // duplicates of a valid target; results not stored
    if (i1 >= count) i1 = count - 1;
    float h0, l0, h1, l1;
    split2(a.x[a.ib + first + i0], h0, l0);
    split2(a.x[a.ib + first + i1], h1, l1);
    pr[p].xh = make_float2(h0, h1);
    pr[p].xl = make_float2(l0, l1);
    split2(a.y[a.ib + first + i0], h0, l0);
    split2(a.y[a.ib + first + i1], h1, l1);
    pr[p].yh = make_float2(h0, h1);
    pr[p].yl = make_float2(l0, l1);
    hu[p] = hv[p] = lu[p] = lv[p] = make_float2(0.f, 0.f);
  }
  const float2 d2 = make_float2(a.d2, a.d2);

  pipe_init(bars);
  uint32_t g = 0;
  int64_t tile = tile0;
  staged_sweep<Rec, TILE>(a.src, tile0, ntl, stage[0], stage[1], bars, g, a.status, [&](const Rec* tl) {
    float2 au[NP], av[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) au[p] = av[p] = make_float2(0.f, 0.f);
    const PlaneRel::Origin* og = a.org + tile * GPT;
#pragma unroll 1
    for (int g0 = 0; g0 < TILE; g0 += G) {
      const PlaneRel::Origin o = og[g0 / G];
      const Rec* gr = tl + g0;
      float2 tx[NP], ty[NP];
      bool near = false;
      const float lim = (PlaneRel::kNearFactor * o.f.x) * (PlaneRel::kNearFactor * o.f.x);
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        tx[p] = rel1x2(pr[p].xh, pr[p].xl, o.o.x, o.o.z);
        ty[p] = rel1x2(pr[p].yh, pr[p].yl, o.o.y, o.o.w);
        const float2 n2 = __ffma2_rn(ty[p], ty[p], __fmul2_rn(tx[p], tx[p]));
        near |= (n2.x < lim) | (n2.y < lim);
      }
      // the group's terms are summed on their own and then added to the tile's: a running
      // FP32 sum of a whole tile's terms (both signs, e.g. the two lobes of a dipole) rounds
      // at the size of the tile's partial sum 256 times, a group sum only 64 times
      float2 gu[NP], gv[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) gu[p] = gv[p] = make_float2(0.f, 0.f);
      if (!__any_sync(0xffffffffu, near)) {
        // far group: d = t_hi - s_hi
#pragma unroll 4
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b;
          const float2 nsx = lo2(ra), nsy = hi2(ra), s2 = lo2(rb);
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(tx[p], nsx);
            const float2 dy = __fadd2_rn(ty[p], nsy);
            float2 q = __ffma2_rn(dx, dx, d2);
            q = __ffma2_rn(dy, dy, q);
            const float2 w = __fmul2_rn(s2, make_float2(rcp_approx(q.x), rcp_approx(q.y)));
            gu[p] = __ffma2_rn(w, dy, gu[p]);
            gv[p] = __ffma2_rn(w, dx, gv[p]);
          }
        }
      } else {
        // near group: d = (t_hi - s_hi) + (t_lo - s_lo)
        float2 txh[NP], tyh[NP], txl[NP], tyl[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          rel2x2(pr[p].xh, pr[p].xl, o.o.x, o.o.z, txh[p], txl[p]);
          rel2x2(pr[p].yh, pr[p].yl, o.o.y, o.o.w, tyh[p], tyl[p]);
        }
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c;
          const float2 nsx = lo2(ra), nsy = hi2(ra), s2 = lo2(rb), nlx = hi2(rb), nly = lo2(rc);
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(__fadd2_rn(txh[p], nsx), __fadd2_rn(txl[p], nlx));
            const float2 dy = __fadd2_rn(__fadd2_rn(tyh[p], nsy), __fadd2_rn(tyl[p], nly));
            float2 q = __ffma2_rn(dx, dx, d2);
            q = __ffma2_rn(dy, dy, q);
            const float2 w = __fmul2_rn(s2, make_float2(rcp_approx(q.x), rcp_approx(q.y)));
            gu[p] = __ffma2_rn(w, dy, gu[p]);
            gv[p] = __ffma2_rn(w, dx, gv[p]);
          }
        }
      }
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        au[p] = __fadd2_rn(au[p], gu[p]);
        av[p] = __fadd2_rn(av[p], gv[p]);
      }
    }
    ++tile;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      comp_add(hu[p].x, lu[p].x, au[p].x);
      comp_add(hu[p].y, lu[p].y, au[p].y);
      comp_add(hv[p].x, lv[p].x, av[p].x);
      comp_add(hv[p].y, lv[p].y, av[p].y);
    }
  });

#pragma unroll
  for (int p = 0; p < NP; ++p) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t il = first + (2 * p + h) * THREADS + threadIdx.x;
      if (il < a.nt) {
        a.partial[(chunk * 2 + 0) * a.nt + il] =
            static_cast<double>(h ? hu[p].y : hu[p].x) + static_cast<double>(h ? lu[p].y : lu[p].x);
        a.partial[(chunk * 2 + 1) * a.nt + il] =
            static_cast<double>(h ? hv[p].y : hv[p].x) + static_cast<double>(h ? lv[p].y : lv[p].x);
      }
    }
  }
}

// Records and origins of one tile of TILE sources (one CTA of TILE threads): each group of
// kGroup sources reduces its centroid o, its radius R about o and its total S_g (of the FP32
// strengths), and every record is written as rel2(p_j, o) -- the operations the sweep uses
// for targets.  s_scale = 1/(2 pi) for the velocity, 1/(4 pi) for the stream function.
// `second` (optional): a second strength second_j A_j s_scale into c.zw (the SWE divergence).
template <int TILE>
__global__ void __launch_bounds__(TILE) plane_rel_prep_kernel(const double* x, const double* y, const double* omega,
                                                              const double* area, const int32_t* sorted, int64_t ns,
                                                              double s_scale, PlaneRel::Rec* out,
                                                              PlaneRel::Origin* org, const double* second = nullptr) {
  constexpr int G = PlaneRel::kGroup;
  __shared__ double red[3][TILE];
  __shared__ float fmax_[TILE], cntf[TILE];
  const int64_t t = blockIdx.x;
  const int tid = threadIdx.x;
  const int64_t k = t * TILE + tid;
  const bool valid = k < ns;
  const int32_t j = valid ? sorted[k] : 0;
  const int lane = tid % G;
  const double px = valid ? x[j] : 0.0, py = valid ? y[j] : 0.0;
  const float s = valid ? __double2float_rn(omega[j] * area[j] * s_scale) : 0.f;
  red[0][tid] = px;
  red[1][tid] = py;
  red[2][tid] = s;
  cntf[tid] = valid ? 1.f : 0.f;
  __syncthreads();
  for (int w = G / 2; w > 0; w >>= 1) {
    if (lane < w) {
      red[0][tid] += red[0][tid + w];
      red[1][tid] += red[1][tid + w];
      red[2][tid] += red[2][tid + w];
      cntf[tid] += cntf[tid + w];
    }
    __syncthreads();
  }
  const int g0 = tid - lane;
  const double cnt = cntf[g0] > 0.f ? static_cast<double>(cntf[g0]) : 1.0;
  const double cx = red[0][g0] / cnt, cy = red[1][g0] / cnt;
  fmax_[tid] = valid ? static_cast<float>(sqrt((px - cx) * (px - cx) + (py - cy) * (py - cy))) : 0.f;
  __syncthreads();
  for (int w = G / 2; w > 0; w >>= 1) {
    if (lane < w) fmax_[tid] = fmaxf(fmax_[tid], fmax_[tid + w]);
    __syncthreads();
  }
  float oxh, oxl, oyh, oyl;
  split2(cx, oxh, oxl);
  split2(cy, oyh, oyl);
  PlaneRel::Rec r;
  if (valid) {
    float h, l, sxh, sxl, syh, syl;
    split2(px, h, l);
    rel2(h, l, oxh, oxl, sxh, sxl);
    split2(py, h, l);
    rel2(h, l, oyh, oyl, syh, syl);
    r.a = make_float4(-sxh, -sxh, -syh, -syh);
    r.b = make_float4(s, s, -sxl, -sxl);
    const float s2 = second ? __double2float_rn(second[j] * area[j] * s_scale) : 0.f;
    r.c = make_float4(-syl, -syl, s2, s2);
  } else {
    // inert: at the origin with zero strength (q >= delta^2 + 2^-100 > 0)
    r.a = r.b = r.c = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  out[k] = r;
  if (lane == 0) {
    PlaneRel::Origin o;
    o.o = make_float4(oxh, oyh, oxl, oyl);
    float sgh, sgl;
    split2(red[2][g0], sgh, sgl);
    o.f = make_float4(fmax_[g0], sgh, sgl, 0.f);
    org[t * (TILE / G) + tid / G] = o;
  }
}

}  // namespace lpm

namespace lpm {

// ====================================================================== planar PSE Laplacian
// PSEPlaneLaplacianAtParticles (src/PSEDirectSum.f90:467-500, K8 of the chord distance) and
// the Gaussian 4 exp(-r^2)/pi of the chord, on the planar group-relative layout with the
// group cutoff of the sphere's PSE sweep (pse_rel.cuh): a warp skips a group when every one
// of its targets is farther than R + 7 eps from its centroid, where r^2 >= 49 and a term is
// below 1e-17 of the kernel's peak, far below FP32 resolution of the sum.  Per target pair and evaluated source (far form):
// d (2 FADD2), r^2 (2), exp(-r^2) (1 FMUL2 + 2 MUFU ex2), the K8 polynomial and product
// (3 + 1), f_j - f_i from hi/lo parts (3), the accumulation (2).
struct PlanePseRel {
  struct __align__(16) Rec {
    float4 a;  // -sx_hi, -sx_hi, -sy_hi, -sy_hi
    float4 b;  // A_j, A_j, f_hi, f_hi
    float4 c;  // -sx_lo, -sx_lo, -sy_lo, -sy_lo
    float4 d;  // f_lo, f_lo, 0, 0
  };
  static constexpr int kGroup = 32;  // sources per origin: the group cutoff's granularity
};

struct PlanePseRelArgs {
  const double *x, *y, *f;
  float ks2;    // eps^-2
  float c_cut;  // 7 eps: r^2 = PseRel::kCutR2
  const float4* tball;  // per source tile: centre (hi parts, z = 0) and radius
  const PlanePseRel::Rec* src;
  const PlaneRel::Origin* org;
  int64_t n_tiles, tiles_per_chunk, ib, nt;
  // targets in curve order: position k of the sweep is particle tperm[k] (nullptr: ib + k);
  // partial sums are stored at the particle's own place, (tperm[k] - ib)
  const int32_t* tperm;
  double* partial;  // [chunk][nt]
  int* status;
};

template <bool K8>
__device__ __forceinline__ void plane_pse_pair(float2 dx, float2 dy, float2 ks2, float4 rb, float4 rd, float2 fh,
                                               float2 fl, float2& acc) {
  const float2 r2 = __fmul2_rn(__ffma2_rn(dy, dy, __fmul2_rn(dx, dx)), ks2);
  const float2 ea = __fmul2_rn(r2, make_float2(-1.4426950f, -1.4426950f));
  float2 k = make_float2(ex2_approx(ea.x), ex2_approx(ea.y));  // exp(-r^2)
  if (K8) {
    float2 poly = __ffma2_rn(make_float2(-0.6666666666666666f, -0.6666666666666666f), r2, make_float2(10.0f, 10.0f));
    poly = __ffma2_rn(poly, r2, make_float2(-40.0f, -40.0f));
    poly = __ffma2_rn(poly, r2, make_float2(40.0f, 40.0f));
    k = __fmul2_rn(poly, k);
  }
  const float2 df = __fadd2_rn(__fadd2_rn(hi2(rb), make_float2(-fh.x, -fh.y)), __fadd2_rn(lo2(rd), make_float2(-fl.x, -fl.y)));
  acc = __ffma2_rn(df, __fmul2_rn(lo2(rb), k), acc);
}

// On the warp-decoupled pipeline (S stages of TILE records), like the sphere PSE sweep: a warp
// whose targets reach none of a tile's groups moves on without waiting for the others.
template <bool K8, int THREADS, int TPT, int TILE, int MINB, int S>
__global__ void __launch_bounds__(THREADS, MINB) plane_pse_rel_sweep_kernel(PlanePseRelArgs a) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  constexpr int NP = TPT / 2;
  constexpr int G = PlanePseRel::kGroup;
  constexpr int GPT = TILE / G;
  using Rec = PlanePseRel::Rec;
  __shared__ TilePipe<Rec, TILE, S, PlaneRel::Origin, GPT> pipe;

  const int64_t chunk = blockIdx.y;  // this CTA's share of the target block's in-reach tiles

  PlaneRel::Pair pr[NP];
  float2 fh[NP], fl[NP], hs[NP], ls[NP];
  const int64_t first = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT);
  const int64_t count = a.nt - first < THREADS * TPT ? a.nt - first : THREADS * TPT;
  // each warp takes 32 x TPT consecutive targets of the (curve-ordered) block
  const int64_t wbase = static_cast<int64_t>(threadIdx.x >> 5) * (32 * TPT) + (threadIdx.x & 31);
  int64_t tgt[NP][2];
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    float vh[2][3], vl[2][3];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int64_t il = wbase + (2 * p + h) * 32;
      tgt[p][h] = il < count ? first + il : -1;
      if (il >= count) il = count - 1;  // duplicates of a valid target; results not stored
      const int64_t i = a.tperm ? static_cast<int64_t>(a.tperm[first + il]) : a.ib + first + il;
      if (tgt[p][h] >= 0) tgt[p][h] = i - a.ib;
      split2(a.x[i], vh[h][0], vl[h][0]);
      split2(a.y[i], vh[h][1], vl[h][1]);
      split2(a.f[i], vh[h][2], vl[h][2]);
    }
    pr[p].xh = make_float2(vh[0][0], vh[1][0]);
    pr[p].yh = make_float2(vh[0][1], vh[1][1]);
    pr[p].xl = make_float2(vl[0][0], vl[1][0]);
    pr[p].yl = make_float2(vl[0][1], vl[1][1]);
    fh[p] = make_float2(vh[0][2], vh[1][2]);
    fl[p] = make_float2(vl[0][2], vl[1][2]);
    hs[p] = ls[p] = make_float2(0.f, 0.f);
  }
  const float2 ks2 = make_float2(a.ks2, a.ks2);

  // the CTA's targets (hi parts) for the tile culling (engine.cuh)
  __shared__ TargetBall ball;
  {
    float bx[2 * NP], by[2 * NP], bz[2 * NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      bx[2 * p] = pr[p].xh.x;
      bx[2 * p + 1] = pr[p].xh.y;
      by[2 * p] = pr[p].yh.x;
      by[2 * p + 1] = pr[p].yh.y;
      bz[2 * p] = bz[2 * p + 1] = 0.f;
    }
    cta_target_ball<THREADS, 2 * NP>(bx, by, bz, ball);
  }

  tile_pipe_init(pipe);
  uint32_t g = 0;
  auto tile_body = [&](const Rec* tl, const PlaneRel::Origin* og) {
    float2 acc[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[p] = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int g0 = 0; g0 < TILE; g0 += G) {
      const PlaneRel::Origin o = og[g0 / G];
      const Rec* gr = tl + g0;
      float2 tx[NP], ty[NP];
      const float reach = o.f.x + a.c_cut;
      const float lim = (PlaneRel::kNearFactor * o.f.x) * (PlaneRel::kNearFactor * o.f.x);
      bool in_reach = false, near = false;
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        tx[p] = rel1x2(pr[p].xh, pr[p].xl, o.o.x, o.o.z);
        ty[p] = rel1x2(pr[p].yh, pr[p].yl, o.o.y, o.o.w);
        const float2 n2 = __ffma2_rn(ty[p], ty[p], __fmul2_rn(tx[p], tx[p]));
        in_reach |= (n2.x < reach * reach) | (n2.y < reach * reach);
        near |= (n2.x < lim) | (n2.y < lim);
      }
      if (!__any_sync(0xffffffffu, in_reach)) continue;  // every pair has r^2 > PseRel::kCutR2
      if (!__any_sync(0xffffffffu, near)) {
#pragma unroll 4
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b, rd = gr[j].d;
#pragma unroll
          for (int p = 0; p < NP; ++p)
            plane_pse_pair<K8>(__fadd2_rn(tx[p], lo2(ra)), __fadd2_rn(ty[p], hi2(ra)), ks2, rb, rd, fh[p], fl[p],
                               acc[p]);
        }
      } else {
        float2 txh[NP], tyh[NP], txl[NP], tyl[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          rel2x2(pr[p].xh, pr[p].xl, o.o.x, o.o.z, txh[p], txl[p]);
          rel2x2(pr[p].yh, pr[p].yl, o.o.y, o.o.w, tyh[p], tyl[p]);
        }
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c, rd = gr[j].d;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(__fadd2_rn(txh[p], lo2(ra)), __fadd2_rn(txl[p], lo2(rc)));
            const float2 dy = __fadd2_rn(__fadd2_rn(tyh[p], hi2(ra)), __fadd2_rn(tyl[p], hi2(rc)));
            plane_pse_pair<K8>(dx, dy, ks2, rb, rd, fh[p], fl[p], acc[p]);
          }
        }
      }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      comp_add(hs[p].x, ls[p].x, acc[p].x);
      comp_add(hs[p].y, ls[p].y, acc[p].y);
    }
  };
  // this CTA's balanced share of the in-reach tiles of the whole source range (engine.cuh);
  // gridDim.y CTAs share a target block
  const WaitCfg wait = default_wait();
  sweep_culled_share<THREADS>(
      a.n_tiles, [&](int64_t t) { return tile_in_reach(a.tball[t], ball, a.c_cut); },
      [&](const int32_t* list, int cnt) {
        return warp_sweep_tiles(a.src, [list](int64_t k) { return static_cast<int64_t>(list[k]); }, cnt, pipe, g,
                                a.status, wait, a.org, tile_body);
      });

#pragma unroll
  for (int p = 0; p < NP; ++p) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t il = tgt[p][h];
      if (il >= 0)
        a.partial[chunk * a.nt + il] = static_cast<double>(h ? hs[p].y : hs[p].x) + static_cast<double>(h ? ls[p].y : ls[p].x);
    }
  }
}

// Records and origins for the planar PSE sweep: one CTA of TILE threads per tile; the group
// frame is that of plane_rel_prep_kernel.
template <int TILE>
__global__ void __launch_bounds__(TILE) plane_pse_rel_prep_kernel(const double* x, const double* y, const double* f,
                                                                  const double* area, const int32_t* sorted,
                                                                  int64_t ns, PlanePseRel::Rec* out,
                                                                  PlaneRel::Origin* org, float4* tball) {
  constexpr int G = PlanePseRel::kGroup;
  __shared__ double red[2][TILE];
  __shared__ float fmax_[TILE], cntf[TILE];
  const int64_t t = blockIdx.x;
  const int tid = threadIdx.x;
  const int64_t k = t * TILE + tid;
  const bool valid = k < ns;
  const int32_t j = valid ? sorted[k] : 0;
  const int lane = tid % G;
  const double px = valid ? x[j] : 0.0, py = valid ? y[j] : 0.0;
  red[0][tid] = px;
  red[1][tid] = py;
  cntf[tid] = valid ? 1.f : 0.f;
  __syncthreads();
  for (int w = G / 2; w > 0; w >>= 1) {
    if (lane < w) {
      red[0][tid] += red[0][tid + w];
      red[1][tid] += red[1][tid + w];
      cntf[tid] += cntf[tid + w];
    }
    __syncthreads();
  }
  const int g0 = tid - lane;
  const double cnt = cntf[g0] > 0.f ? static_cast<double>(cntf[g0]) : 1.0;
  const double cx = red[0][g0] / cnt, cy = red[1][g0] / cnt;
  fmax_[tid] = valid ? static_cast<float>(sqrt((px - cx) * (px - cx) + (py - cy) * (py - cy))) : 0.f;
  __syncthreads();
  for (int w = G / 2; w > 0; w >>= 1) {
    if (lane < w) fmax_[tid] = fmaxf(fmax_[tid], fmax_[tid + w]);
    __syncthreads();
  }
  float oxh, oxl, oyh, oyl;
  split2(cx, oxh, oxl);
  split2(cy, oyh, oyl);
  PlanePseRel::Rec r;
  if (valid) {
    float h, l, sxh, sxl, syh, syl, fh, fl;
    split2(px, h, l);
    rel2(h, l, oxh, oxl, sxh, sxl);
    split2(py, h, l);
    rel2(h, l, oyh, oyl, syh, syl);
    split2(f[j], fh, fl);
    const float ar = __double2float_rn(area[j]);
    r.a = make_float4(-sxh, -sxh, -syh, -syh);
    r.b = make_float4(ar, ar, fh, fh);
    r.c = make_float4(-sxl, -sxl, -syl, -syl);
    r.d = make_float4(fl, fl, 0.f, 0.f);
  } else {
    r.a = r.b = r.c = r.d = make_float4(0.f, 0.f, 0.f, 0.f);  // zero area: no contribution
  }
  out[k] = r;
  constexpr int GPT = TILE / G;
  __shared__ float4 grp[GPT];  // the groups' balls for the tile's ball (w < 0: empty group)
  if (lane == 0) {
    PlaneRel::Origin o;
    o.o = make_float4(oxh, oyh, oxl, oyl);
    o.f = make_float4(fmax_[g0], 0.f, 0.f, 0.f);
    org[t * GPT + tid / G] = o;
    grp[tid / G] = valid ? make_float4(oxh, oyh, 0.f, fmax_[g0]) : make_float4(0.f, 0.f, 0.f, -1.f);
  }
  __syncthreads();
  if (tid == 0) tball[t] = tile_ball_from_groups<GPT>(grp);
}

// ====================================================================== planar SWE integrals
// SWEPlaneRHSIntegrals, src/SWEPlaneSolver.f90:457-571, velocity and velocity-gradient part
// (the surface-height Laplacian is the planar PSE sweep above).  With W = vort_j A_j / (2 pi),
// D = div_j A_j / (2 pi) (records: b.xy = W, c.zw = D) and s = 1/r^2, the reference's terms are
//   u += s P, v += s Q,  P = D dx - W dy, Q = W dx + D dy,
//   ux += D s - 2 s dx (s P),  uy += -W s - 2 s dy (s P),
//   vx +=  W s - 2 s dx (s Q), vy += D s - 2 s dy (s Q)
// (1/(pi r^4) = 2 s^2 / (2 pi)).  Each gradient term is formed per pair before it is summed, so
// the cancellation between the D s and the s^2 terms happens per pair, as in the reference.
// Far groups: 23 packed operations and 2 MUFU per target pair and source; near groups add the
// lo parts and give the self pair s = 0.  Partials: [chunk][6][nt] (u, v, ux, uy, vx, vy).
template <int THREADS, int TPT, int TILE, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) plane_swe_rel_sweep_kernel(PlaneRelArgs a) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  static_assert(TILE % PlaneRel::kGroup == 0, "whole origin groups per tile");
  constexpr int NP = TPT / 2;
  constexpr int G = PlaneRel::kGroup;
  constexpr int GPT = TILE / G;
  constexpr int NC = 6;
  using Rec = PlaneRel::Rec;
  __shared__ __align__(128) Rec stage[2][TILE];
  __shared__ __align__(8) uint64_t bars[2];

  const int64_t chunk = blockIdx.y;
  const int64_t tile0 = chunk * a.tiles_per_chunk;
  int64_t ntl = a.n_tiles - tile0;
  if (ntl > a.tiles_per_chunk) ntl = a.tiles_per_chunk;
  if (ntl < 0) ntl = 0;

  PlaneRel::Pair pr[NP];
  float2 hs[NP][NC], ls[NP][NC];
  const int64_t first = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT);
  const int64_t count = a.nt - first < THREADS * TPT ? a.nt - first : THREADS * TPT;
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    int64_t i0 = (2 * p) * THREADS + threadIdx.x, i1 = (2 * p + 1) * THREADS + threadIdx.x;
    if (i0 >= count) i0 = count - 1;  // duplicates of a valid target; results not stored
    if (i1 >= count) i1 = count - 1;
    float h0, l0, h1, l1;
    split2(a.x[a.ib + first + i0], h0, l0);
    split2(a.x[a.ib + first + i1], h1, l1);
    pr[p].xh = make_float2(h0, h1);
    pr[p].xl = make_float2(l0, l1);
    split2(a.y[a.ib + first + i0], h0, l0);
    split2(a.y[a.ib + first + i1], h1, l1);
    pr[p].yh = make_float2(h0, h1);
    pr[p].yl = make_float2(l0, l1);
#pragma unroll
    for (int c = 0; c < NC; ++c) hs[p][c] = ls[p][c] = make_float2(0.f, 0.f);
  }
  const float2 m2 = make_float2(-2.0f, -2.0f);

  pipe_init(bars);
  uint32_t g = 0;
  int64_t tile = tile0;
  staged_sweep<Rec, TILE>(a.src, tile0, ntl, stage[0], stage[1], bars, g, a.status, [&](const Rec* tl) {
    float2 acc[NP][NC];
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[p][c] = make_float2(0.f, 0.f);
    // one pair's terms from d = (dx, dy) and s = 1/r^2 (0 for the self pair)
    auto terms = [&](float2 (&ac)[NC], float2 dx, float2 dy, float2 sv, float2 w, float2 dd) {
      const float2 pp = __ffma2_rn(dd, dx, __fmul2_rn(make_float2(-w.x, -w.y), dy));
      const float2 qq = __ffma2_rn(w, dx, __fmul2_rn(dd, dy));
      const float2 sp = __fmul2_rn(sv, pp), sq = __fmul2_rn(sv, qq);
      const float2 ds = __fmul2_rn(dd, sv), ws = __fmul2_rn(w, sv);
      const float2 s2 = __fmul2_rn(sv, m2);
      const float2 t1 = __fmul2_rn(s2, dx), t2 = __fmul2_rn(s2, dy);
      ac[0] = __fadd2_rn(ac[0], sp);
      ac[1] = __fadd2_rn(ac[1], sq);
      ac[2] = __fadd2_rn(ac[2], __ffma2_rn(t1, sp, ds));
      ac[3] = __fadd2_rn(ac[3], __ffma2_rn(t2, sp, make_float2(-ws.x, -ws.y)));
      ac[4] = __fadd2_rn(ac[4], __ffma2_rn(t1, sq, ws));
      ac[5] = __fadd2_rn(ac[5], __ffma2_rn(t2, sq, ds));
    };
    const PlaneRel::Origin* og = a.org + tile * GPT;
#pragma unroll 1
    for (int g0 = 0; g0 < TILE; g0 += G) {
      const PlaneRel::Origin o = og[g0 / G];
      const Rec* gr = tl + g0;
      float2 tx[NP], ty[NP];
      bool near = false;
      const float lim = fmaxf((PlaneRel::kNearFactor * o.f.x) * (PlaneRel::kNearFactor * o.f.x),
                              7.888609052210118e-31f);
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        tx[p] = rel1x2(pr[p].xh, pr[p].xl, o.o.x, o.o.z);
        ty[p] = rel1x2(pr[p].yh, pr[p].yl, o.o.y, o.o.w);
        const float2 n2 = __ffma2_rn(ty[p], ty[p], __fmul2_rn(tx[p], tx[p]));
        near |= !(n2.x > lim) | !(n2.y > lim);
      }
      if (!__any_sync(0xffffffffu, near)) {
        // far group: d = t_hi - s_hi, r^2 > 0
#pragma unroll 2
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(tx[p], lo2(ra));
            const float2 dy = __fadd2_rn(ty[p], hi2(ra));
            const float2 r2 = __ffma2_rn(dy, dy, __fmul2_rn(dx, dx));
            terms(acc[p], dx, dy, make_float2(rcp_approx(r2.x), rcp_approx(r2.y)), lo2(rb), hi2(rc));
          }
        }
      } else {
        // near group: d = (t_hi - s_hi) + (t_lo - s_lo); the self pair has d = 0 exactly
        float2 txh[NP], tyh[NP], txl[NP], tyl[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          rel2x2(pr[p].xh, pr[p].xl, o.o.x, o.o.z, txh[p], txl[p]);
          rel2x2(pr[p].yh, pr[p].yl, o.o.y, o.o.w, tyh[p], tyl[p]);
        }
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(__fadd2_rn(txh[p], lo2(ra)), __fadd2_rn(txl[p], hi2(rb)));
            const float2 dy = __fadd2_rn(__fadd2_rn(tyh[p], hi2(ra)), __fadd2_rn(tyl[p], lo2(rc)));
            const float2 r2 = __ffma2_rn(dy, dy, __fmul2_rn(dx, dx));
            const float2 sv = make_float2(r2.x > 0.f ? rcp_approx(r2.x) : 0.f, r2.y > 0.f ? rcp_approx(r2.y) : 0.f);
            terms(acc[p], dx, dy, sv, lo2(rb), hi2(rc));
          }
        }
      }
    }
    ++tile;
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        comp_add(hs[p][c].x, ls[p][c].x, acc[p][c].x);
        comp_add(hs[p][c].y, ls[p][c].y, acc[p][c].y);
      }
  });

#pragma unroll
  for (int p = 0; p < NP; ++p) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t il = first + (2 * p + h) * THREADS + threadIdx.x;
      if (il < a.nt) {
#pragma unroll
        for (int c = 0; c < NC; ++c)
          a.partial[(chunk * NC + c) * a.nt + il] = static_cast<double>(h ? hs[p][c].y : hs[p][c].x) +
                                                    static_cast<double>(h ? ls[p][c].y : ls[p][c].x);
      }
    }
  }
}

}  // namespace lpm
