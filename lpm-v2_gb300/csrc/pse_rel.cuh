// pse_rel.cuh -- the sphere PSE operators in FP32C on the group-relative layout of the BVE
// sweep (bve_rel.cuh), with a group-level cutoff: the Laplacian (K8 of the great-circle
// distance, or the Gaussian of the chord), the gradient and the divergence (K1, the first-
// derivative kernel, of the great-circle distance).
//
// Reference, src/PSEDirectSum.f90 (kernels :611-640):
//   PSESphereLaplacianAtParticles (:502-535)  L_i = eps^-4 sum_j (f_j - f_i) A_j K8(r)
//   PSESphereGradientAtParticles  (:220-267)  G_i = eps^-4 P_i sum_j (f_j + f_i) (x_i - x_j) A_j K1(r)
//   PSESphereDivergenceAtParticles (:537-579) D_i = eps^-4 sum_j (P_i (x_i - x_j)) . (V_j + V_i) A_j K1(r)
// with r = distance / eps and P_i = I - x_i x_i^T (SphereProjection).  Every kernel carries
// exp(-r^2): at r^2 >= 49 every kernel (K8, K1 times r, the Gaussian) is below 1e-17 of its
// peak (K8: |40 - 40 r^2 + 10 r^4 - 2/3 r^6| e^-49 / 40 = 7e-19), far below FP32 -- and
// FP64 -- resolution of any sum it enters.  A warp therefore skips a whole group of 32
// sources when every one of its targets is farther than R + c_cut from the group's centroid
// (R the group radius, c_cut = 7 eps / a the chord at which r^2 = 49; the great-circle
// distance is never shorter than the chord).  The result equals the all-pairs sum to FP32
// rounding; the skipped pairs are counted as done.
//
// Positions are unit directions p / |p| for the great-circle kernels (the angle between them
// is what SphereDistance's atan2 measures; then x_i - x_j = a d and x_i . d = |d|^2 / 2 on
// the sphere) and x / a for the chord kernel, Hilbert-sorted and stored as hi/lo offsets from
// their group's centroid, with the compact / far / near precision choice of the BVE sweep.
// The angle: theta^2 from the chord v = |d|^2 by the asin^2 series when eps / a <= 0.06
// (kPseAngleSeries), else 4 asin^2(sqrt(v) / 2).  Per target pair and evaluated
// source (far form, series angle): d (3 FADD2), v (3), theta^2 (4), r^2 (2), exp(-r^2)
// (1 FMUL2 + 2 MUFU ex2), the kernel polynomial (3) and product (1), then the operator's
// terms (Laplacian: f_j - f_i from hi/lo parts, 3 + 2; gradient: 1 + 1 + 3; divergence:
// V_j + V_i, the projection and the dot product, 3 + 4 + 3 + 1).
#pragma once

#include "bve_rel.cuh"
#include "ops.cuh"

namespace lpm {

enum PseRelOp { kPseOpLapK8 = 0, kPseOpLapGauss = 1, kPseOpGrad = 2, kPseOpDiv = 3 };
enum PseRelAngle { kPseAngleSeries = 0, kPseAngleAsin = 1, kPseAngleChord = 2 };

struct PseRel {
  // Laplacian and gradient: c = (f_hi, f_hi, f_lo, f_lo), e = (-sz_lo, -sz_lo, 0, 0);
  // divergence: c = (vx, vx, vy, vy), e = (-sz_lo, -sz_lo, vz, vz).
  struct __align__(16) Rec {
    float4 a;  // -sx_hi, -sx_hi, -sy_hi, -sy_hi
    float4 b;  // -sz_hi, -sz_hi, A_j, A_j
    float4 c;
    float4 d;  // -sx_lo, -sx_lo, -sy_lo, -sy_lo
    float4 e;
  };
  // target pair: position hi/lo, and (f_hi, f_lo, -) or (vx, vy, vz)
  struct Pair {
    float2 xh, yh, zh, xl, yl, zl, e0, e1, e2;
  };
  static constexpr float kCutR2 = 49.0f;  // r^2 beyond which a pair is negligible
  // sources per origin: the group cutoff's granularity (larger groups reach farther; 32 ran
  // 2-9 % faster than 64 with the r^2 >= 49 cutoff and the tile culling, 128 12 % slower)
  static constexpr int kGroup = 32;
};

struct PseRelArgs {
  const double *x, *y, *z, *f, *vy, *vz;  // f is vx for the divergence
  double inv_a;
  float ks2;      // (a / eps)^2
  float c_cut;    // chord at which r^2 = kCutR2
  const float4* tball;  // per source tile: centre (unit-scaled hi parts) and radius
  float half_a2;  // a^2 / 2 (divergence: P d = d - (a^2 |d|^2 / 2) p_i)
  const PseRel::Rec* src;
  const BveRel::Origin* org;  // hi.w: near radius (0 for a compact group), lo.w: group radius
  int64_t n_tiles, tiles_per_chunk, ib, nt;
  // targets in curve order: position k of the sweep is particle tperm[k] (nullptr: ib + k);
  // partial sums are stored at the particle's own place, (tperm[k] - ib)
  const int32_t* tperm;
  double* partial;  // [chunk][comps][nt]
  int* status;
  WaitCfg wait;  // limits of the bounded waits (the test hook may shorten them and skip a tile)
};

template <int OP>
struct PseRelComps {
  static constexpr int value = OP == kPseOpGrad ? 3 : 1;
};

// Position of particle i as the operator uses it.
template <int ANG>
__device__ __forceinline__ void pse_position(const double* x, const double* y, const double* z, int64_t i,
                                             double inv_a, double& px, double& py, double& pz) {
  px = x[i] * inv_a;
  py = y[i] * inv_a;
  pz = z[i] * inv_a;
  if (ANG != kPseAngleChord) {
    const double s = 1.0 / sqrt(fma(px, px, fma(py, py, pz * pz)));
    px *= s;
    py *= s;
    pz *= s;
  }
}

template <int ANG>
__device__ __forceinline__ float2 pse_r2(float2 v, float2 ks2) {
  if (ANG == kPseAngleSeries) {
    float2 sr = __ffma2_rn(v, make_float2(3.1746032e-4f, 3.1746032e-4f), make_float2(1.7857143e-3f, 1.7857143e-3f));
    sr = __ffma2_rn(sr, v, make_float2(1.1111111e-2f, 1.1111111e-2f));
    sr = __ffma2_rn(sr, v, make_float2(8.3333336e-2f, 8.3333336e-2f));
    sr = __ffma2_rn(sr, v, make_float2(1.0f, 1.0f));
    return __fmul2_rn(__fmul2_rn(v, ks2), sr);
  } else if (ANG == kPseAngleAsin) {
    const float h0 = asinf(fminf(0.5f * sqrtf(v.x), 1.0f)), h1 = asinf(fminf(0.5f * sqrtf(v.y), 1.0f));
    return __fmul2_rn(make_float2(4.0f * h0 * h0, 4.0f * h1 * h1), ks2);
  } else {
    return __fmul2_rn(v, ks2);
  }
}

// One pair term for a target pair with d the offsets' difference; accumulates into acc.
template <int OP, int ANG>
__device__ __forceinline__ void pse_pair(float2 dx, float2 dy, float2 dz, float2 ks2, float half_a2, float4 rb,
                                         float4 rc, float4 re, const PseRel::Pair& t, float2* acc) {
  const float2 v = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
  const float2 r2 = pse_r2<ANG>(v, ks2);
  const float2 ea = __fmul2_rn(r2, make_float2(-1.4426950f, -1.4426950f));
  float2 k = make_float2(ex2_approx(ea.x), ex2_approx(ea.y));  // exp(-r^2)
  if (OP == kPseOpLapK8) {
    float2 poly = __ffma2_rn(make_float2(-0.6666666666666666f, -0.6666666666666666f), r2, make_float2(10.0f, 10.0f));
    poly = __ffma2_rn(poly, r2, make_float2(-40.0f, -40.0f));
    poly = __ffma2_rn(poly, r2, make_float2(40.0f, 40.0f));
    k = __fmul2_rn(poly, k);
  } else if (OP == kPseOpGrad || OP == kPseOpDiv) {
    float2 poly = __ffma2_rn(make_float2(0.33333334f, 0.33333334f), r2, make_float2(-5.0f, -5.0f));
    poly = __ffma2_rn(poly, r2, make_float2(20.0f, 20.0f));
    poly = __ffma2_rn(poly, r2, make_float2(-20.0f, -20.0f));
    k = __fmul2_rn(poly, k);
  }
  const float2 wk = __fmul2_rn(hi2(rb), k);  // A_j K
  if (OP == kPseOpLapK8 || OP == kPseOpLapGauss) {
    // f_j - f_i = (f_j,hi - f_i,hi) + (f_j,lo - f_i,lo)
    const float2 df = __fadd2_rn(__fadd2_rn(lo2(rc), make_float2(-t.e0.x, -t.e0.y)),
                                 __fadd2_rn(hi2(rc), make_float2(-t.e1.x, -t.e1.y)));
    acc[0] = __ffma2_rn(df, wk, acc[0]);
  } else if (OP == kPseOpGrad) {
    const float2 w = __fmul2_rn(__fadd2_rn(lo2(rc), t.e0), wk);  // (f_j + f_i) A_j K1
    acc[0] = __ffma2_rn(w, dx, acc[0]);
    acc[1] = __ffma2_rn(w, dy, acc[1]);
    acc[2] = __ffma2_rn(w, dz, acc[2]);
  } else {
    // (P_i d) . (V_j + V_i) with P_i d = d - (a^2 v / 2) p_i
    const float2 c = __fmul2_rn(v, make_float2(-half_a2, -half_a2));
    const float2 gx = __ffma2_rn(c, t.xh, dx), gy = __ffma2_rn(c, t.yh, dy), gz = __ffma2_rn(c, t.zh, dz);
    const float2 wx = __fadd2_rn(lo2(rc), t.e0), wy = __fadd2_rn(hi2(rc), t.e1), wz = __fadd2_rn(hi2(re), t.e2);
    const float2 dot = __ffma2_rn(gz, wz, __ffma2_rn(gy, wy, __fmul2_rn(gx, wx)));
    acc[0] = __ffma2_rn(dot, wk, acc[0]);
  }
}

// The sweep runs on the warp-decoupled pipeline (S stages of TILE records): most groups are
// out of reach of most warps, and a warp that skips a tile's groups moves on to the next
// tile instead of waiting at a block barrier for the warps that evaluate it.
template <int OP, int ANG, int THREADS, int TPT, int TILE, int MINB, int S>
__global__ void __launch_bounds__(THREADS, MINB) pse_rel_sweep_kernel(PseRelArgs a) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  constexpr int NP = TPT / 2;
  constexpr int NC = PseRelComps<OP>::value;
  constexpr int G = PseRel::kGroup;
  constexpr int GPT = TILE / G;
  using Rec = PseRel::Rec;
  __shared__ TilePipe<Rec, TILE, S, BveRel::Origin, GPT> pipe;

  const int64_t chunk = blockIdx.y;  // this CTA's share of the target block's in-reach tiles

  PseRel::Pair pr[NP];
  float2 hs[NP][NC], ls[NP][NC];
  const int64_t first = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT);
  const int64_t count = a.nt - first < THREADS * TPT ? a.nt - first : THREADS * TPT;
  // each warp takes 32 x TPT consecutive targets of the (curve-ordered) block, so that its
  // targets are close together and the group cutoff passes over as many groups as it can
  const int64_t wbase = static_cast<int64_t>(threadIdx.x >> 5) * (32 * TPT) + (threadIdx.x & 31);
  int64_t tgt[NP][2];
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    float vh[2][3], vl[2][3], ex[2][3];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int64_t il = wbase + (2 * p + h) * 32;
      tgt[p][h] = il < count ? first + il : -1;
      if (il >= count) il = count - 1;  // duplicates of a valid target; results not stored
      const int64_t i = a.tperm ? static_cast<int64_t>(a.tperm[first + il]) : a.ib + first + il;
      if (tgt[p][h] >= 0) tgt[p][h] = i - a.ib;
      double px, py, pz;
      pse_position<ANG>(a.x, a.y, a.z, i, a.inv_a, px, py, pz);
      split2(px, vh[h][0], vl[h][0]);
      split2(py, vh[h][1], vl[h][1]);
      split2(pz, vh[h][2], vl[h][2]);
      if (OP == kPseOpDiv) {
        ex[h][0] = __double2float_rn(a.f[i]);
        ex[h][1] = __double2float_rn(a.vy[i]);
        ex[h][2] = __double2float_rn(a.vz[i]);
      } else {
        split2(a.f[i], ex[h][0], ex[h][1]);
        ex[h][2] = 0.f;
      }
    }
    pr[p].xh = make_float2(vh[0][0], vh[1][0]);
    pr[p].yh = make_float2(vh[0][1], vh[1][1]);
    pr[p].zh = make_float2(vh[0][2], vh[1][2]);
    pr[p].xl = make_float2(vl[0][0], vl[1][0]);
    pr[p].yl = make_float2(vl[0][1], vl[1][1]);
    pr[p].zl = make_float2(vl[0][2], vl[1][2]);
    pr[p].e0 = make_float2(ex[0][0], ex[1][0]);
    pr[p].e1 = make_float2(ex[0][1], ex[1][1]);
    pr[p].e2 = make_float2(ex[0][2], ex[1][2]);
#pragma unroll
    for (int c = 0; c < NC; ++c) hs[p][c] = ls[p][c] = make_float2(0.f, 0.f);
  }
  const float2 ks2 = make_float2(a.ks2, a.ks2);

  // the ball around the CTA's targets (unit-scaled hi parts) for the tile culling
  __shared__ TargetBall ball;
  {
    float bx[2 * NP], by[2 * NP], bz[2 * NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      bx[2 * p] = pr[p].xh.x;
      bx[2 * p + 1] = pr[p].xh.y;
      by[2 * p] = pr[p].yh.x;
      by[2 * p + 1] = pr[p].yh.y;
      bz[2 * p] = pr[p].zh.x;
      bz[2 * p + 1] = pr[p].zh.y;
    }
    cta_target_ball<THREADS, 2 * NP>(bx, by, bz, ball);
  }

  tile_pipe_init(pipe);
  uint32_t g = 0;
  auto tile_body = [&](const Rec* tl, const BveRel::Origin* og) {
    float2 acc[NP][NC];
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[p][c] = make_float2(0.f, 0.f);
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
      if (!__any_sync(0xffffffffu, in_reach)) continue;  // every pair has r^2 > kCutR2
      if (o.hi.w == 0.f || !warp_near<NP>(tx, ty, tz, o.hi.w)) {
        // compact or far group: d = t_hi - s_hi
#pragma unroll 4
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c, re = gr[j].e;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(tx[p], lo2(ra));
            const float2 dy = __fadd2_rn(ty[p], hi2(ra));
            const float2 dz = __fadd2_rn(tz[p], lo2(rb));
            pse_pair<OP, ANG>(dx, dy, dz, ks2, a.half_a2, rb, rc, re, pr[p], acc[p]);
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
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(__fadd2_rn(txh[p], lo2(ra)), __fadd2_rn(txl[p], lo2(rd)));
            const float2 dy = __fadd2_rn(__fadd2_rn(tyh[p], hi2(ra)), __fadd2_rn(tyl[p], hi2(rd)));
            const float2 dz = __fadd2_rn(__fadd2_rn(tzh[p], lo2(rb)), __fadd2_rn(tzl[p], lo2(re)));
            pse_pair<OP, ANG>(dx, dy, dz, ks2, a.half_a2, rb, rc, re, pr[p], acc[p]);
          }
        }
      }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        comp_add(hs[p][c].x, ls[p][c].x, acc[p][c].x);
        comp_add(hs[p][c].y, ls[p][c].y, acc[p][c].y);
      }
  };
  // this CTA's balanced share of the in-reach tiles of the whole source range (engine.cuh);
  // gridDim.y CTAs share a target block.  (The gradient and divergence sweeps spill 64-144
  // bytes with it, at 128 registers, and still run 1.4-2x faster than over every tile of a
  // chunk.)
  sweep_culled_share<THREADS>(
      a.n_tiles, [&](int64_t t) { return tile_in_reach(a.tball[t], ball, a.c_cut); },
      [&](const int32_t* list, int cnt) {
        return warp_sweep_tiles(a.src, [list](int64_t k) { return static_cast<int64_t>(list[k]); }, cnt, pipe, g,
                                a.status, a.wait, a.org, tile_body);
      });

#pragma unroll
  for (int p = 0; p < NP; ++p) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t il = tgt[p][h];
      if (il >= 0) {
#pragma unroll
        for (int c = 0; c < NC; ++c)
          a.partial[(chunk * NC + c) * a.nt + il] =
              static_cast<double>(h ? hs[p][c].y : hs[p][c].x) + static_cast<double>(h ? ls[p][c].y : ls[p][c].x);
      }
    }
  }
}

// Records and group origins of the sorted sources (one CTA of TILE threads per tile).  For the
// divergence f is vx and vy, vz the other components.
template <int OP, int ANG, int TILE>
__global__ void __launch_bounds__(TILE) pse_rel_prep_kernel(const double* x, const double* y, const double* z,
                                                            const double* f, const double* vy, const double* vz,
                                                            const double* area, const int32_t* sorted, int64_t ns,
                                                            double inv_a, PseRel::Rec* out, BveRel::Origin* org,
                                                            float4* tball) {
  const int64_t t = blockIdx.x;
  const int64_t k = t * TILE + threadIdx.x;
  const bool valid = k < ns;
  const int32_t j = valid ? sorted[k] : 0;
  double px = 0.0, py = 0.0, pz = 0.0;
  if (valid) pse_position<ANG>(x, y, z, j, inv_a, px, py, pz);
  const GroupFrame fr = sphere_group_frame<TILE, PseRel::kGroup>(valid, px, py, pz, 0.0);
  PseRel::Rec r;
  if (valid) {
    float hi[3], lo[3];
    group_offsets(fr, px, py, pz, hi, lo);
    const float ar = __double2float_rn(area[j]);
    r.a = make_float4(-hi[0], -hi[0], -hi[1], -hi[1]);
    r.b = make_float4(-hi[2], -hi[2], ar, ar);
    r.d = make_float4(-lo[0], -lo[0], -lo[1], -lo[1]);
    if (OP == kPseOpDiv) {
      const float vxf = __double2float_rn(f[j]), vyf = __double2float_rn(vy[j]), vzf = __double2float_rn(vz[j]);
      r.c = make_float4(vxf, vxf, vyf, vyf);
      r.e = make_float4(-lo[2], -lo[2], vzf, vzf);
    } else {
      float fh, fl;
      split2(f[j], fh, fl);
      r.c = make_float4(fh, fh, fl, fl);
      r.e = make_float4(-lo[2], -lo[2], 0.f, 0.f);
    }
  } else {
    r.a = r.b = r.c = r.d = r.e = make_float4(0.f, 0.f, 0.f, 0.f);  // zero area: no contribution
  }
  out[k] = r;
  constexpr int GPT = TILE / PseRel::kGroup;
  __shared__ float4 grp[GPT];  // the groups' balls for the tile's ball (w < 0: empty group)
  if (threadIdx.x % PseRel::kGroup == 0) {
    BveRel::Origin o = group_origin(fr);
    o.lo.w = fr.radius;  // the cutoff test needs the radius of every group
    org[t * GPT + threadIdx.x / PseRel::kGroup] = o;
    grp[threadIdx.x / PseRel::kGroup] = valid ? make_float4(o.hi.x, o.hi.y, o.hi.z, fr.radius)
                                              : make_float4(0.f, 0.f, 0.f, -1.f);
  }
  __syncthreads();
  if (threadIdx.x == 0) tball[t] = tile_ball_from_groups<GPT>(grp);
}

// Gradient finish: chunk sums of sum_j (f_j + f_i) A_j K1 d, projected with P_i = I - x_i x_i^T
// (physical x_i) and scaled by a / (pi eps^4).
__global__ void pse_grad_finish_kernel(const double* partial, int64_t nsplit, int64_t nt, int64_t ib, const double* x,
                                       const double* y, const double* z, double scale, double* gx, double* gy,
                                       double* gz) {
  const int64_t il = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (il >= nt) return;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int64_t c = 0; c < nsplit; ++c) {
    s0 += partial[(c * 3 + 0) * nt + il];
    s1 += partial[(c * 3 + 1) * nt + il];
    s2 += partial[(c * 3 + 2) * nt + il];
  }
  const int64_t i = ib + il;
  const double xi = x[i], yi = y[i], zi = z[i];
  const double xg = xi * s0 + yi * s1 + zi * s2;
  gx[il] = (s0 - xi * xg) * scale;
  gy[il] = (s1 - yi * xg) * scale;
  gz[il] = (s2 - zi * xg) * scale;
}

}  // namespace lpm
