// pse_rel.cuh -- the sphere PSE Laplacian in FP32C on the group-relative layout of the BVE
// sweep (bve_rel.cuh), with a group-level cutoff.
//
// Reference: PSESphereLaplacianAtParticles, src/PSEDirectSum.f90:502-535:
//   L_i = eps^-4 sum_{j active} (f_j - f_i) A_j K(r_ij),  r = dist / eps,
// K = K8 of the great-circle distance (bivariateLaplacianKernel8, :622-627), or the Gaussian
// 4 exp(-r^2)/pi of the chord distance.  Both carry exp(-r^2): a pair with r^2 >= 100 adds
// less than 1e-37 of a near pair's term, below FP32 resolution of any sum it enters.  A warp
// therefore skips a whole group of 64 sources when every one of its targets is farther than
// R + c_cut from the group's centroid (R the group radius, c_cut = 10 eps / a the chord at
// which r^2 = 100; the great-circle distance is never shorter than the chord).  The result
// equals the all-pairs sum to FP32 rounding; the skipped pairs are counted as done.
//
// Positions are unit directions p / |p| for the great circle (the angle between them is what
// SphereDistance's atan2 measures) and x / a for the chord, Hilbert-sorted and stored as
// hi/lo offsets from their group's centroid,
// with the compact / far / near precision choice of the BVE sweep.  Per target pair and
// evaluated source (far form, K8): d (3 FADD2), v = |d|^2 (3), the asin^2 series for the
// angle (4), r^2 (2), exp(-r^2) (1 FMUL2 + 2 MUFU ex2), the K8 polynomial (3) and product
// (1), f_j - f_i from hi/lo parts (3), the weight and the accumulation (2).  The series is
// taken only when eps / a <= 0.06 (PseF32<kPseK8GeoSeries>); the launcher uses the generic
// atan2 sweep otherwise.
#pragma once

#include "bve_rel.cuh"
#include "ops.cuh"

namespace lpm {

struct PseRel {
  struct __align__(16) Rec {
    float4 a;  // -sx_hi, -sx_hi, -sy_hi, -sy_hi
    float4 b;  // -sz_hi, -sz_hi, A_j, A_j
    float4 c;  // f_hi, f_hi, f_lo, f_lo
    float4 d;  // -sx_lo, -sx_lo, -sy_lo, -sy_lo
    float4 e;  // -sz_lo, -sz_lo, 0, 0
  };
  struct Pair {
    float2 xh, yh, zh, xl, yl, zl, fh, fl;
  };
  static constexpr float kCutR2 = 100.0f;  // r^2 beyond which a pair is negligible
};

struct PseRelArgs {
  const double *x, *y, *z, *f;
  double inv_a;
  float ks2;    // (a / eps)^2: r^2 = v ks2 (chord) or theta^2 ks2 (great circle)
  float c_cut;  // chord at which r^2 = kCutR2
  const PseRel::Rec* src;
  const BveRel::Origin* org;  // hi.w: near radius (0 for a compact group), lo.w: group radius
  int64_t n_tiles, tiles_per_chunk, ib, nt;
  double* partial;  // [chunk][nt]
  int* status;
};

// One pair term for target pairs: (f_j - f_i) A_j K(r) with d the offsets' difference.
template <int KIND>
__device__ __forceinline__ float2 pse_pair(float2 dx, float2 dy, float2 dz, float2 ks2, float2 a2, float2 fjh,
                                           float2 fjl, const PseRel::Pair& t) {
  const float2 v = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
  float2 r2;
  if (KIND == kPseK8GeoSeries) {
    float2 sr = __ffma2_rn(v, make_float2(3.1746032e-4f, 3.1746032e-4f), make_float2(1.7857143e-3f, 1.7857143e-3f));
    sr = __ffma2_rn(sr, v, make_float2(1.1111111e-2f, 1.1111111e-2f));
    sr = __ffma2_rn(sr, v, make_float2(8.3333336e-2f, 8.3333336e-2f));
    sr = __ffma2_rn(sr, v, make_float2(1.0f, 1.0f));
    r2 = __fmul2_rn(__fmul2_rn(v, ks2), sr);
  } else {
    r2 = __fmul2_rn(v, ks2);
  }
  const float2 ea = __fmul2_rn(r2, make_float2(-1.4426950f, -1.4426950f));
  float2 k = make_float2(ex2_approx(ea.x), ex2_approx(ea.y));
  if (KIND != kPseGaussChord) {
    float2 poly = __ffma2_rn(make_float2(-0.6666666666666666f, -0.6666666666666666f), r2, make_float2(10.0f, 10.0f));
    poly = __ffma2_rn(poly, r2, make_float2(-40.0f, -40.0f));
    poly = __ffma2_rn(poly, r2, make_float2(40.0f, 40.0f));
    k = __fmul2_rn(poly, k);
  }
  // f_j - f_i = (f_j,hi - f_i,hi) + (f_j,lo - f_i,lo)
  const float2 df = __fadd2_rn(__fadd2_rn(fjh, make_float2(-t.fh.x, -t.fh.y)),
                               __fadd2_rn(fjl, make_float2(-t.fl.x, -t.fl.y)));
  return __fmul2_rn(df, __fmul2_rn(a2, k));
}

template <int KIND, int THREADS, int TPT, int TILE, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) pse_rel_sweep_kernel(PseRelArgs a) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  constexpr int NP = TPT / 2;
  constexpr int G = BveRel::kGroup;
  constexpr int GPT = TILE / G;
  using Rec = PseRel::Rec;
  __shared__ __align__(128) Rec stage[2][TILE];
  __shared__ __align__(8) uint64_t bars[2];

  const int64_t chunk = blockIdx.y;
  const int64_t tile0 = chunk * a.tiles_per_chunk;
  int64_t ntl = a.n_tiles - tile0;
  if (ntl > a.tiles_per_chunk) ntl = a.tiles_per_chunk;
  if (ntl < 0) ntl = 0;

  PseRel::Pair pr[NP];
  float2 hs[NP], ls[NP];
  const int64_t first = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT);
  const int64_t count = a.nt - first < THREADS * TPT ? a.nt - first : THREADS * TPT;
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    float vh[2][4], vl[2][4];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int64_t il = (2 * p + h) * THREADS + threadIdx.x;
      if (il >= count) il = count - 1;  // duplicates of a valid target; results not stored
      const int64_t i = a.ib + first + il;
      double px, py, pz;
      PseF32<KIND>::position(a.x, a.y, a.z, i, a.inv_a, px, py, pz);
      split2(px, vh[h][0], vl[h][0]);
      split2(py, vh[h][1], vl[h][1]);
      split2(pz, vh[h][2], vl[h][2]);
      split2(a.f[i], vh[h][3], vl[h][3]);
    }
    pr[p].xh = make_float2(vh[0][0], vh[1][0]);
    pr[p].yh = make_float2(vh[0][1], vh[1][1]);
    pr[p].zh = make_float2(vh[0][2], vh[1][2]);
    pr[p].fh = make_float2(vh[0][3], vh[1][3]);
    pr[p].xl = make_float2(vl[0][0], vl[1][0]);
    pr[p].yl = make_float2(vl[0][1], vl[1][1]);
    pr[p].zl = make_float2(vl[0][2], vl[1][2]);
    pr[p].fl = make_float2(vl[0][3], vl[1][3]);
    hs[p] = ls[p] = make_float2(0.f, 0.f);
  }
  const float2 ks2 = make_float2(a.ks2, a.ks2);

  pipe_init(bars);
  uint32_t g = 0;
  int64_t tile = tile0;
  staged_sweep<Rec, TILE>(a.src, tile0, ntl, stage[0], stage[1], bars, g, a.status, [&](const Rec* tl) {
    float2 acc[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[p] = make_float2(0.f, 0.f);
    const BveRel::Origin* og = a.org + tile * GPT;
#pragma unroll 1
    for (int g0 = 0; g0 < TILE; g0 += G) {
      const BveRel::Origin o = og[g0 / G];
      const Rec* gr = tl + g0;
      float2 tx[NP], ty[NP], tz[NP];
      const float reach = o.lo.w + a.c_cut;
      bool in_reach = false;
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        tx[p] = rel1x2(pr[p].xh, pr[p].xl, o.hi.x, o.lo.x);
        ty[p] = rel1x2(pr[p].yh, pr[p].yl, o.hi.y, o.lo.y);
        tz[p] = rel1x2(pr[p].zh, pr[p].zl, o.hi.z, o.lo.z);
        const float2 n2 = __ffma2_rn(tz[p], tz[p], __ffma2_rn(ty[p], ty[p], __fmul2_rn(tx[p], tx[p])));
        in_reach |= (n2.x < reach * reach) | (n2.y < reach * reach);
      }
      if (!__any_sync(0xffffffffu, in_reach)) continue;  // every pair has r^2 > 100
      if (o.hi.w == 0.f || !warp_near<NP>(tx, ty, tz, o.hi.w)) {
        // compact or far group: d = t_hi - s_hi
#pragma unroll 4
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c;
          const float2 nsx = lo2(ra), nsy = hi2(ra), nsz = lo2(rb), a2 = hi2(rb), fjh = lo2(rc), fjl = hi2(rc);
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(tx[p], nsx);
            const float2 dy = __fadd2_rn(ty[p], nsy);
            const float2 dz = __fadd2_rn(tz[p], nsz);
            acc[p] = __fadd2_rn(acc[p], pse_pair<KIND>(dx, dy, dz, ks2, a2, fjh, fjl, pr[p]));
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
          const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c, rd = gr[j].d, re = gr[j].e;
          const float2 nsx = lo2(ra), nsy = hi2(ra), nsz = lo2(rb), a2 = hi2(rb), fjh = lo2(rc), fjl = hi2(rc);
          const float2 nlx = lo2(rd), nly = hi2(rd), nlz = lo2(re);
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(__fadd2_rn(txh[p], nsx), __fadd2_rn(txl[p], nlx));
            const float2 dy = __fadd2_rn(__fadd2_rn(tyh[p], nsy), __fadd2_rn(tyl[p], nly));
            const float2 dz = __fadd2_rn(__fadd2_rn(tzh[p], nsz), __fadd2_rn(tzl[p], nlz));
            acc[p] = __fadd2_rn(acc[p], pse_pair<KIND>(dx, dy, dz, ks2, a2, fjh, fjl, pr[p]));
          }
        }
      }
    }
    ++tile;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      comp_add(hs[p].x, ls[p].x, acc[p].x);
      comp_add(hs[p].y, ls[p].y, acc[p].y);
    }
  });

#pragma unroll
  for (int p = 0; p < NP; ++p) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t il = first + (2 * p + h) * THREADS + threadIdx.x;
      if (il < a.nt)
        a.partial[chunk * a.nt + il] = static_cast<double>(h ? hs[p].y : hs[p].x) + static_cast<double>(h ? ls[p].y : ls[p].x);
    }
  }
}

// Records and group origins of the sorted sources (one CTA of TILE threads per tile).
template <int KIND, int TILE>
__global__ void __launch_bounds__(TILE) pse_rel_prep_kernel(const double* x, const double* y, const double* z,
                                                            const double* f, const double* area,
                                                            const int32_t* sorted, int64_t ns, double inv_a,
                                                            PseRel::Rec* out, BveRel::Origin* org) {
  const int64_t t = blockIdx.x;
  const int64_t k = t * TILE + threadIdx.x;
  const bool valid = k < ns;
  const int32_t j = valid ? sorted[k] : 0;
  double px = 0.0, py = 0.0, pz = 0.0;
  if (valid) PseF32<KIND>::position(x, y, z, j, inv_a, px, py, pz);
  const GroupFrame fr = sphere_group_frame<TILE>(valid, px, py, pz, 0.0);
  PseRel::Rec r;
  if (valid) {
    float hi[3], lo[3], fh, fl;
    group_offsets(fr, px, py, pz, hi, lo);
    split2(f[j], fh, fl);
    const float ar = __double2float_rn(area[j]);
    r.a = make_float4(-hi[0], -hi[0], -hi[1], -hi[1]);
    r.b = make_float4(-hi[2], -hi[2], ar, ar);
    r.c = make_float4(fh, fh, fl, fl);
    r.d = make_float4(-lo[0], -lo[0], -lo[1], -lo[1]);
    r.e = make_float4(-lo[2], -lo[2], 0.f, 0.f);
  } else {
    r.a = r.b = r.c = r.d = r.e = make_float4(0.f, 0.f, 0.f, 0.f);  // zero area: no contribution
  }
  out[k] = r;
  if (threadIdx.x % BveRel::kGroup == 0) {
    BveRel::Origin o = group_origin(fr);
    o.lo.w = fr.radius;  // the cutoff test needs the radius of every group
    org[t * (TILE / BveRel::kGroup) + threadIdx.x / BveRel::kGroup] = o;
  }
}

}  // namespace lpm
