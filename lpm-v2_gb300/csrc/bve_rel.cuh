// bve_rel.cuh -- the sphere-BVE FP32C sweep on spatially sorted sources in group-relative
// coordinates (10-11 packed FP32x2 operations per target pair and source).
//
// Sources are in Hilbert-curve order (sort.cu), so a group of kGroup consecutive sources
// covers one connected patch of the sphere.  Each source is stored relative to the centroid
// o of its group as a two-float offset (s_hi, s_lo) = rel2(p, o) (p - o to ~2^-48), and the
// group record holds o and the group radius R (the largest |p_j - o|).  The precision is
// chosen per warp and group:
//  - far (every target of the warp at |t - o| >= 3R): d = t_hi - s_hi with t_hi = fl(t - o),
//    one subtraction per component.  The roundings of t_hi and s_hi are <= 2^-24 |t - o|
//    and 2^-24 R, and |d| >= |t - o| - R >= 2R, so the relative error of d is at most
//    ~2^-23 whatever the point distribution;
//  - near (some target of the warp inside 3R, which includes the group's own sources and any
//    target at a source's position): the target forms (t_hi, t_lo) = rel2(t, o) with
//    exactly the operations of the sources, and d = (t_hi - s_hi) + (t_lo - s_lo) keeps ~48
//    bits; a self pair cancels bit for bit.
// A compact group (R <= a/2 and R <= 64 x its smallest spacing h, i.e. a patch of a
// quasi-uniform point set) takes the far form for every target: the group record carries
// R = 0, and its records use rel2_fast, the target's far-form operations, so a self pair
// still cancels bit for bit.  For a target near such a group the roundings are an absolute
// 2^-24 R inside the near-field sum sum_j S_j / |d_j|^2, which grows only like ln(1/h) on a
// quasi-uniform set, so the velocity error scales with R, not R/h (1.0e-7 relative at
// icosahedral nest 8).  Groups that fail the test (clustered or sparse points) keep the
// near/far choice, whose error bound holds for any point distribution.
// Particle order along the mesh or the curve keeps a warp's targets close together, so a
// warp meets few near groups (at icosahedral nest 8 about one group in a thousand).
// A group whose sources all lie on the sphere to within |c_j| <= 2^-30 h^2 (h its smallest
// spacing; always the case once positions are renormalised) drops c_j: q is then
// fma(dz,dz, fma(dy,dy, fma(dx,dx, -c_i))), one operation less per pair.
// Then  q = |d|^2 - c_i - c_j,  w = S_j / q,  D += w d  with c = |p|^2 - 1 and
// S_j = -zeta_j A_j / (2 pi a) as in BveF32; u = D x p_i in FP64.
// A group whose warp is far (every target at |t - o| >= 3R, compact or not) takes the
// expanded form: with B_j = |s_j|^2 - c_j and S_j s_j stored per source,
//   q/2 = (|t|^2 - c_i)/2 + B_j/2 - t.s_j,  W = sum_j S_j / (q/2),  V = sum_j S_j s_j / (q/2),
//   D += (t W - V) / 2  (once per group),
// 8 packed FP32x2 operations and 2 MUFU per target pair and source: the FMA and MUFU pipes
// are then about equally loaded.  |t|^2 + |s|^2 - 2 t.s cancels by at most
// ((|t| + R) / (|t| - R))^2 <= 4 at the 3R boundary, so q stays within a few ulps.  A compact
// group with a target of the warp near it keeps d = t_hi - s_hi (10-11 operations; it
// contains the self pairs), any other near group the two-float form (17).  Forming the
// targets' offsets and the near test cost about 15 per pair and group.
// Targets keep their original order (only sources are sorted), so no scatter is needed.
#pragma once

#include "bve_x2.cuh"
#include "engine.cuh"
#include "ops.cuh"

namespace lpm {

struct BveRel {
  struct __align__(16) Rec {
    float4 a;  // -sx_hi, -sx_hi, -sy_hi, -sy_hi
    float4 b;  // -sz_hi, -sz_hi, S_j, S_j
    float4 c;  // B_j / 2, B_j / 2, -S_j sx_hi, -S_j sx_hi   (B_j = |s_hi|^2 - c_j)
    float4 d;  // -S_j sy_hi, -S_j sy_hi, -S_j sz_hi, -S_j sz_hi
    float4 e;  // -sx_lo, -sy_lo, -sz_lo, -c_j             (near and compact-near forms)
  };
  struct __align__(16) Origin {
    float4 hi;  // o_hi.x, o_hi.y, o_hi.z, R (the group radius about o; -R for a compact group)
    float4 lo;  // o_lo.x, o_lo.y, o_lo.z, 1 if every c_j of the group is negligible
  };
  // sources per origin: 128 measured 4.4 % faster than 64 for the BVE sweep (half the per-group
  // work per source) at the same accuracy; the stream-function sweeps share the layout
  static constexpr int kGroup = 128;
  static constexpr float kNearFactor = 3.0f;  // near: |t - o| < kNearFactor R
  static constexpr float kCompactRadius = 0.5f;  // compact: R <= kCompactRadius (unit sphere)
  static constexpr float kCompactRatio = 64.0f;  // and R <= kCompactRatio h
};

// Offset of a hi/lo value from a hi/lo origin, rounded once: fl(p - o) to ~2^-24 relative
// (the far form needs no more).
__device__ __forceinline__ float2 rel1x2(float2 ph, float2 pl, float oh, float ol) {
  return __fadd2_rn(__fadd2_rn(ph, make_float2(-oh, -oh)), __fadd2_rn(pl, make_float2(-ol, -ol)));
}

// The same offset as two floats from single roundings: r_hi = rel1 (the far form's target
// offset), r_lo the rounding of its last addition only.  Records of compact groups use it,
// so that a target at a source's position reproduces that source's r_hi bit for bit.
__device__ __forceinline__ void rel2_fast(float ph, float pl, float oh, float ol, float& rh, float& rl) {
  const float a = __fadd_rn(ph, -oh);
  const float b = __fadd_rn(pl, -ol);
  rh = __fadd_rn(a, b);
  rl = __fadd_rn(__fadd_rn(a, -rh), b);
}

// Two-float offset (r_hi, r_lo) of a hi/lo value from a hi/lo origin, r_hi + r_lo = p - o to
// ~2^-48 relative: the TwoSum of (p_hi, -o_hi) keeps the rounding of the leading difference
// (it is not exact when o is far from p), then the small terms are added and renormalised.
__device__ __forceinline__ void rel2(float ph, float pl, float oh, float ol, float& rh, float& rl) {
  const float s = __fadd_rn(ph, -oh);
  const float v = __fadd_rn(s, -ph);
  const float e = __fadd_rn(__fadd_rn(ph, -__fadd_rn(s, -v)), __fadd_rn(-oh, -v));
  const float r = __fadd_rn(e, __fadd_rn(pl, -ol));
  rh = __fadd_rn(s, r);
  rl = __fadd_rn(r, -__fadd_rn(rh, -s));
}

__device__ __forceinline__ void rel2x2(float2 ph, float2 pl, float oh, float ol, float2& rh, float2& rl) {
  const float2 noh = make_float2(-oh, -oh);
  const float2 s = __fadd2_rn(ph, noh);
  const float2 v = __fadd2_rn(s, make_float2(-ph.x, -ph.y));
  const float2 sv = __fadd2_rn(s, make_float2(-v.x, -v.y));
  const float2 e = __fadd2_rn(__fadd2_rn(ph, make_float2(-sv.x, -sv.y)), __fadd2_rn(noh, make_float2(-v.x, -v.y)));
  const float2 r = __fadd2_rn(e, __fadd2_rn(pl, make_float2(-ol, -ol)));
  rh = __fadd2_rn(s, r);
  const float2 d = __fadd2_rn(rh, make_float2(-s.x, -s.y));
  rl = __fadd2_rn(r, make_float2(-d.x, -d.y));
}

// Target pairs of a sweep: thread t holds targets first + t + (2p + h) * threads, clamped
// to the `count` valid ones (duplicates are computed but not stored).
template <int NP>
__device__ __forceinline__ void bve_load_pairs(const BveF32::Params& prm, int64_t first, int64_t count,
                                               int threads, BveX2::Pair (&pr)[NP]) {
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    int64_t i0 = (2 * p) * threads + threadIdx.x, i1 = (2 * p + 1) * threads + threadIdx.x;
    if (i0 >= count) i0 = count - 1;
    if (i1 >= count) i1 = count - 1;
    const BveF32::Tgt t0 = BveF32::load_target(prm, first + i0);
    const BveF32::Tgt t1 = BveF32::load_target(prm, first + i1);
    pr[p].xh = make_float2(t0.xh, t1.xh);
    pr[p].yh = make_float2(t0.yh, t1.yh);
    pr[p].zh = make_float2(t0.zh, t1.zh);
    pr[p].xl = make_float2(t0.xl, t1.xl);
    pr[p].yl = make_float2(t0.yl, t1.yl);
    pr[p].zl = make_float2(t0.zl, t1.zl);
    pr[p].nc = make_float2(t0.nc, t1.nc);
  }
}

// Whether any target of the warp lies within kNearFactor R of a group origin (t = t_hi,
// the offsets from it).  Every lane of the warp must call it.
template <int NP>
__device__ __forceinline__ bool warp_near(const float2 (&tx)[NP], const float2 (&ty)[NP], const float2 (&tz)[NP],
                                          float r) {
  const float lim = (BveRel::kNearFactor * r) * (BveRel::kNearFactor * r);
  bool near = false;
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    const float2 n2 = __ffma2_rn(tz[p], tz[p], __ffma2_rn(ty[p], ty[p], __fmul2_rn(tx[p], tx[p])));
    near |= (n2.x < lim) | (n2.y < lim);
  }
  return __any_sync(0xffffffffu, near);
}

// One staged tile against NP target pairs: FP32 partials of D added into (ax, ay, az).  The far
// loop is unrolled UNROLL times (4 measured 0.2 % faster than 2 for the 128 x 8 sweep).
template <int NP, int TILE, int UNROLL = 4>
__device__ __forceinline__ void bve_rel_tile(const BveRel::Rec* __restrict__ tl, const BveRel::Origin* __restrict__ og,
                                             const BveX2::Pair (&pr)[NP], float2 (&ax)[NP], float2 (&ay)[NP],
                                             float2 (&az)[NP]) {
  constexpr int G = BveRel::kGroup;
#pragma unroll 1
  for (int g0 = 0; g0 < TILE; g0 += G) {
    const BveRel::Origin o = og[g0 / G];
    const BveRel::Rec* gr = tl + g0;
    float2 tx[NP], ty[NP], tz[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      tx[p] = rel1x2(pr[p].xh, pr[p].xl, o.hi.x, o.lo.x);
      ty[p] = rel1x2(pr[p].yh, pr[p].yl, o.hi.y, o.lo.y);
      tz[p] = rel1x2(pr[p].zh, pr[p].zl, o.hi.z, o.lo.z);
    }
    if (!warp_near<NP>(tx, ty, tz, fabsf(o.hi.w))) {
      // far group, expanded form: h = q/2 = (|t|^2 - c_i)/2 + B_j/2 - t.s_j, D += (t W - V)/2
      float2 ct[NP], ww[NP], vx[NP], vy[NP], vz[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        ct[p] = __fmul2_rn(__ffma2_rn(tz[p], tz[p], __ffma2_rn(ty[p], ty[p], __ffma2_rn(tx[p], tx[p], pr[p].nc))),
                           make_float2(0.5f, 0.5f));
        ww[p] = vx[p] = vy[p] = vz[p] = make_float2(0.f, 0.f);
      }
#pragma unroll UNROLL
      for (int j = 0; j < G; ++j) {
        const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c, rd = gr[j].d;
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          // records hold -s, so t.(-s) = -t.s
          float2 h = __fadd2_rn(ct[p], lo2(rc));
          h = __ffma2_rn(tx[p], lo2(ra), h);
          h = __ffma2_rn(ty[p], hi2(ra), h);
          h = __ffma2_rn(tz[p], lo2(rb), h);
          const float2 inv = make_float2(rcp_approx(h.x), rcp_approx(h.y));
          ww[p] = __ffma2_rn(hi2(rb), inv, ww[p]);
          vx[p] = __ffma2_rn(hi2(rc), inv, vx[p]);
          vy[p] = __ffma2_rn(lo2(rd), inv, vy[p]);
          vz[p] = __ffma2_rn(hi2(rd), inv, vz[p]);
        }
      }
#pragma unroll
      for (int p = 0; p < NP; ++p) {  // V holds -sum S s / h: D += (t W + V) / 2
        const float2 half = make_float2(0.5f, 0.5f);
        ax[p] = __ffma2_rn(__ffma2_rn(tx[p], ww[p], vx[p]), half, ax[p]);
        ay[p] = __ffma2_rn(__ffma2_rn(ty[p], ww[p], vy[p]), half, ay[p]);
        az[p] = __ffma2_rn(__ffma2_rn(tz[p], ww[p], vz[p]), half, az[p]);
      }
    } else if (o.hi.w < 0.f) {
      // compact group near the warp (it may hold the targets themselves): d = t_hi - s_hi with
      // the records' rel2_fast offsets, so a self pair cancels bit for bit
      if (o.lo.w != 0.f) {
        // every source of the group on the sphere: c_j dropped
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b;
          const float2 nsx = lo2(ra), nsy = hi2(ra), nsz = lo2(rb), s2 = hi2(rb);
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(tx[p], nsx);
            const float2 dy = __fadd2_rn(ty[p], nsy);
            const float2 dz = __fadd2_rn(tz[p], nsz);
            float2 q = __ffma2_rn(dx, dx, pr[p].nc);
            q = __ffma2_rn(dy, dy, q);
            q = __ffma2_rn(dz, dz, q);
            const float2 inv = make_float2(rcp_approx(q.x), rcp_approx(q.y));
            const float2 wgt = __fmul2_rn(s2, inv);
            ax[p] = __ffma2_rn(wgt, dx, ax[p]);
            ay[p] = __ffma2_rn(wgt, dy, ay[p]);
            az[p] = __ffma2_rn(wgt, dz, az[p]);
          }
        }
      } else {
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b;
          const float ncj1 = gr[j].e.w;
          const float2 nsx = lo2(ra), nsy = hi2(ra), nsz = lo2(rb), ncj = make_float2(ncj1, ncj1), s2 = hi2(rb);
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(tx[p], nsx);
            const float2 dy = __fadd2_rn(ty[p], nsy);
            const float2 dz = __fadd2_rn(tz[p], nsz);
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
      }
    } else {
      // near group: d = (t_hi - s_hi) + (t_lo - s_lo)
      float2 txh[NP], tyh[NP], tzh[NP], txl[NP], tyl[NP], tzl[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        rel2x2(pr[p].xh, pr[p].xl, o.hi.x, o.lo.x, txh[p], txl[p]);
        rel2x2(pr[p].yh, pr[p].yl, o.hi.y, o.lo.y, tyh[p], tyl[p]);
        rel2x2(pr[p].zh, pr[p].zl, o.hi.z, o.lo.z, tzh[p], tzl[p]);
      }
      for (int j = 0; j < G; ++j) {
        const float4 ra = gr[j].a, rb = gr[j].b, re = gr[j].e;
        const float2 nsx = lo2(ra), nsy = hi2(ra), nsz = lo2(rb), s2 = hi2(rb);
        const float2 nlx = make_float2(re.x, re.x), nly = make_float2(re.y, re.y), nlz = make_float2(re.z, re.z);
        const float2 ncj = make_float2(re.w, re.w);
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const float2 dx = __fadd2_rn(__fadd2_rn(txh[p], nsx), __fadd2_rn(txl[p], nlx));
          const float2 dy = __fadd2_rn(__fadd2_rn(tyh[p], nsy), __fadd2_rn(tyl[p], nly));
          const float2 dz = __fadd2_rn(__fadd2_rn(tzh[p], nsz), __fadd2_rn(tzl[p], nlz));
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
    }
  }
}

// Adds the FP32 tile partials into the compensated (hi, lo) accumulators.
template <int NP>
__device__ __forceinline__ void bve_merge_pairs(const float2 (&ax)[NP], const float2 (&ay)[NP], const float2 (&az)[NP],
                                                float2 (&hx)[NP], float2 (&hy)[NP], float2 (&hz)[NP],
                                                float2 (&lx)[NP], float2 (&ly)[NP], float2 (&lz)[NP]) {
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    comp_add(hx[p].x, lx[p].x, ax[p].x);
    comp_add(hx[p].y, lx[p].y, ax[p].y);
    comp_add(hy[p].x, ly[p].x, ay[p].x);
    comp_add(hy[p].y, ly[p].y, ay[p].y);
    comp_add(hz[p].x, lz[p].x, az[p].x);
    comp_add(hz[p].y, lz[p].y, az[p].y);
  }
}

template <int THREADS, int TPT, int TILE, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) bve_rel_sweep_kernel(SweepArgs<BveF32> a,
                                                                      const BveRel::Origin* __restrict__ org) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  static_assert(TILE % BveRel::kGroup == 0, "whole origin groups per tile");
  constexpr int NP = TPT / 2;
  constexpr int GPT = TILE / BveRel::kGroup;
  using Rec = BveRel::Rec;
  __shared__ __align__(128) Rec stage[2][TILE];
  __shared__ __align__(8) uint64_t bars[2];

  const int64_t chunk = blockIdx.y;
  const int64_t tile0 = chunk * a.tiles_per_chunk;
  int64_t ntl = a.n_tiles - tile0;
  if (ntl > a.tiles_per_chunk) ntl = a.tiles_per_chunk;
  if (ntl < 0) ntl = 0;

  BveX2::Pair pr[NP];
  float2 hx[NP], hy[NP], hz[NP], lx[NP], ly[NP], lz[NP];
  const int64_t first = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT);
  const int64_t count = a.nt - first < THREADS * TPT ? a.nt - first : THREADS * TPT;
  bve_load_pairs<NP>(a.p, a.ib + first, count, THREADS, pr);
#pragma unroll
  for (int p = 0; p < NP; ++p) hx[p] = hy[p] = hz[p] = lx[p] = ly[p] = lz[p] = make_float2(0.f, 0.f);

  pipe_init(bars);
  uint32_t g = 0;
  int64_t tile = tile0;
  const Rec* src = reinterpret_cast<const Rec*>(a.src);
  staged_sweep<Rec, TILE>(src, tile0, ntl, stage[0], stage[1], bars, g, a.status, a.wait, [&](const Rec* tl) {
    float2 ax[NP], ay[NP], az[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) ax[p] = ay[p] = az[p] = make_float2(0.f, 0.f);
    bve_rel_tile<NP, TILE>(tl, org + tile * GPT, pr, ax, ay, az);
    ++tile;
    bve_merge_pairs<NP>(ax, ay, az, hx, hy, hz, lx, ly, lz);
  });

#pragma unroll
  for (int p = 0; p < NP; ++p) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t il = first + (2 * p + h) * THREADS + threadIdx.x;
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

// The frame of the thread's group of G sources within a tile of TILE (one CTA of TILE
// threads, every thread one source): the centroid o as hi/lo floats, the radius R about o,
// whether the group is compact (R <= a/2 and R <= 64 x the smallest distance h between
// consecutive sources) and whether every |c_j| <= 2^-30 h^2 (c_j negligible in q).  (px, py,
// pz) is the unit-scaled position and cj = |p|^2 - 1 (both meaningful only if `valid`).
struct GroupFrame {
  float oxh, oxl, oyh, oyl, ozh, ozl;
  float radius;
  bool compact, on_sphere;
};

template <int TILE, int G>
__device__ __forceinline__ GroupFrame sphere_group_frame(bool valid, double px, double py, double pz, double cj) {
  __shared__ double sp[3][TILE];
  __shared__ double red[3][TILE];
  __shared__ float fmax_[TILE], fmin_[TILE], cmax_[TILE], cntf[TILE];
  const int tid = threadIdx.x;
  const int lane = tid % G;  // position in the group
  if (!valid) px = py = pz = cj = 0.0;
  sp[0][tid] = px;
  sp[1][tid] = py;
  sp[2][tid] = pz;
  red[0][tid] = px;
  red[1][tid] = py;
  red[2][tid] = pz;
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
  const int g0 = tid - lane;  // first thread of the group
  const double cnt = cntf[g0] > 0.f ? static_cast<double>(cntf[g0]) : 1.0;
  const double cx = red[0][g0] / cnt, cy = red[1][g0] / cnt, cz = red[2][g0] / cnt;
  float rad = 0.f, spc = 3.4e38f;
  if (valid) {
    const double dx = px - cx, dy = py - cy, dz = pz - cz;
    rad = static_cast<float>(sqrt(dx * dx + dy * dy + dz * dz));
    if (lane > 0) {
      const double ex = px - sp[0][tid - 1], ey = py - sp[1][tid - 1], ez = pz - sp[2][tid - 1];
      spc = static_cast<float>(sqrt(ex * ex + ey * ey + ez * ez));
    }
  }
  fmax_[tid] = rad;
  fmin_[tid] = spc;
  cmax_[tid] = static_cast<float>(fabs(cj));
  __syncthreads();
  for (int w = G / 2; w > 0; w >>= 1) {
    if (lane < w) {
      fmax_[tid] = fmaxf(fmax_[tid], fmax_[tid + w]);
      fmin_[tid] = fminf(fmin_[tid], fmin_[tid + w]);
      cmax_[tid] = fmaxf(cmax_[tid], cmax_[tid + w]);
    }
    __syncthreads();
  }
  GroupFrame f;
  f.radius = fmax_[g0];
  const float gspc = fmin_[g0], gcmax = cmax_[g0];
  f.compact = f.radius <= BveRel::kCompactRadius && f.radius <= BveRel::kCompactRatio * gspc;
  // on the sphere: dropping every c_j moves q by <= 2^-30 h^2 relative to the smallest |d|^2
  f.on_sphere = gcmax <= 9.313225746154785e-10f * gspc * gspc;
  split2(cx, f.oxh, f.oxl);
  split2(cy, f.oyh, f.oyl);
  split2(cz, f.ozh, f.ozl);
  return f;
}

// Offsets of a unit-scaled position from its group's centroid: rel2_fast for a compact
// group (the target's far-form operations), rel2 otherwise.
__device__ __forceinline__ void group_offsets(const GroupFrame& f, double px, double py, double pz, float (&hi)[3],
                                              float (&lo)[3]) {
  const double p[3] = {px, py, pz};
  const float oh[3] = {f.oxh, f.oyh, f.ozh}, ol[3] = {f.oxl, f.oyl, f.ozl};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float h, l;
    split2(p[c], h, l);
    if (f.compact) {
      rel2_fast(h, l, oh[c], ol[c], hi[c], lo[c]);
    } else {
      rel2(h, l, oh[c], ol[c], hi[c], lo[c]);
    }
  }
}

// The group record: centroid, radius (0 for a compact group: never near), on-sphere flag.
__device__ __forceinline__ BveRel::Origin group_origin(const GroupFrame& f) {
  BveRel::Origin o;
  o.hi = make_float4(f.oxh, f.oyh, f.ozh, f.compact ? 0.f : f.radius);
  o.lo = make_float4(f.oxl, f.oyl, f.ozl, f.on_sphere ? 1.f : 0.f);
  return o;
}

// Records and origins of one tile of TILE sources (one CTA of TILE threads; every thread
// one record).  `j` is the thread's particle (meaningful only if `valid`), `inv_a` and
// `s_scale` the tile's sphere scale.  Every record is written as the offset of p_j from its
// group's centroid -- the operations the sweep uses for targets.
template <int TILE>
__device__ __forceinline__ void bve_rel_prep_tile(const double* x, const double* y, const double* z,
                                                  const double* zeta, const double* area, bool valid, int32_t j,
                                                  double inv_a, double s_scale, BveRel::Rec* out,
                                                  BveRel::Origin* og) {
  double px = 0.0, py = 0.0, pz = 0.0, cj = 0.0;
  if (valid) {
    px = x[j] * inv_a;
    py = y[j] * inv_a;
    pz = z[j] * inv_a;
    cj = fma(px, px, fma(py, py, fma(pz, pz, -1.0)));
  }
  const GroupFrame f = sphere_group_frame<TILE, BveRel::kGroup>(valid, px, py, pz, cj);
  BveRel::Rec r;
  if (valid) {
    float hi[3], lo[3];
    group_offsets(f, px, py, pz, hi, lo);
    const float nc = __double2float_rn(-cj);
    const double sd = zeta[j] * area[j] * s_scale;
    const float s = __double2float_rn(sd);
    const double h0 = hi[0], h1 = hi[1], h2 = hi[2];
    const float b = __double2float_rn(0.5 * fma(h0, h0, fma(h1, h1, fma(h2, h2, -cj))));  // (|s_hi|^2 - c_j) / 2
    r.a = make_float4(-hi[0], -hi[0], -hi[1], -hi[1]);
    r.b = make_float4(-hi[2], -hi[2], s, s);
    const float sx = __double2float_rn(-sd * h0), sy = __double2float_rn(-sd * h1), sz = __double2float_rn(-sd * h2);
    r.c = make_float4(b, b, sx, sx);
    r.d = make_float4(sy, sy, sz, sz);
    r.e = make_float4(-lo[0], -lo[1], -lo[2], nc);
  } else {
    // inert: at the origin with zero strength and zero -c (weight 0 times a finite value;
    // q > 0 through the target's 2^-100 offset when the target sits on o)
    r.a = r.b = r.c = r.d = r.e = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  *out = r;
  if (threadIdx.x % BveRel::kGroup == 0) {
    BveRel::Origin o = group_origin(f);
    o.hi.w = f.compact ? -f.radius : f.radius;  // the sign marks a compact group
    og[threadIdx.x / BveRel::kGroup] = o;
  }
}

// Tile-relative records of the Hilbert-sorted source list `sorted` (ns entries, records
// ns..npad-1 inert) and the group origins: one CTA of TILE threads per tile.
template <int TILE>
__global__ void __launch_bounds__(TILE) bve_rel_prep_kernel(const double* x, const double* y, const double* z,
                                                            const double* zeta, const double* area,
                                                            const int32_t* sorted, int64_t ns, double inv_a,
                                                            double s_scale, BveRel::Rec* out, BveRel::Origin* org) {
  const int64_t t = blockIdx.x;
  const int64_t k = t * TILE + threadIdx.x;
  const bool valid = k < ns;
  const int32_t j = valid ? sorted[k] : 0;
  bve_rel_prep_tile<TILE>(x, y, z, zeta, area, valid, j, inv_a, s_scale, out + k,
                          org + t * (TILE / BveRel::kGroup));
}

}  // namespace lpm
