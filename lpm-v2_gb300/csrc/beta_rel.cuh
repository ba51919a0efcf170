// beta_rel.cuh -- the beta-plane (x-periodic) velocity and stream functions in FP32C on 2-D
// Hilbert-ordered sources in groups of 64, with complex far forms (the stream functions'
// follow the velocity kernel below).
//
// Reference: BetaPlaneVelocity, src/BetaPlaneSolver.f90:227-268:
//   s_j = 0.5 zeta_j A_j / (cosh(2 pi dy) - cos(2 pi dx)),  u -= sinh(2 pi dy) s_j,
//   v += sin(2 pi dx) s_j,   dx = x_i - x_j, dy = y_i - y_j,  j != i.
// With z = x + i y, S_j = 0.5 zeta_j A_j and cot(a + ib) = (sin 2a - i sinh 2b) / (cosh 2b - cos 2a),
// the pair term is v + i u = S_j cot(pi (z_i - z_j)).  With e = exp(2 pi i (z - z_o)) taken
// relative to the centroid z_o of the source's group, cot(pi (z_i - z_j)) = i (e_i + e_j) /
// (e_i - e_j) = i (1 + 2 e_j / (e_i - e_j)), so a group contributes
//   v + i u = i (S_g + 2 G),  G = sum_j S_j e_j / (e_i - e_j),  S_g = sum_j S_j:
// u += S_g + 2 Re G, v -= 2 Im G.  Per target pair and source: e_i - e_j (2 FADD2), |.|^2 (2),
// 2 MUFU, S_j e_j conj(e_i - e_j) (4) and the accumulation (2) -- 10 packed operations and 2
// MUFU against about 28 packed operations for the direct form.  e_j is formed in FP64 by the prep kernel; e_i once per target
// and group with expf and sincospif.  The periodicity in x is in e itself.
// An error delta in e_i moves e_i - e_j by delta |e_i|, i.e. by delta / (2 pi |z_i - z_j|)
// relative, so the complex form is kept for targets beyond max(4 R, 0.02) of the group
// (|z_i - z_j| >= 3 R): a warp with any target nearer (in the periodic distance) sums that
// group with the direct, cancellation-free form of BetaF32 (csrc/ops.cuh), which also drops
// the self pair.
// Each tile's FP32 partial goes into compensated (hi, lo) pairs; partials [chunk][2][nt].
#pragma once

#include "bve_rel.cuh"
#include "engine.cuh"
#include "ops.cuh"
#include "stream_rel.cuh"

namespace lpm {

struct BetaRel {
  struct __align__(16) Rec {
    float4 a;  // x_hi, y_hi, x_lo, y_lo                 (direct form)
    float4 b;  // S, 0, 0, 0                             (S = zeta A / 2)
    float4 c;  // e.re, e.re, e.im, e.im                 (e = exp(2 pi i (z - z_o)))
    float4 d;  // (S e).re, (S e).re, (S e).im, (S e).im
  };
  struct __align__(16) Origin {
    float4 o;  // x_o hi, y_o hi, x_o lo, y_o lo
    float4 f;  // R (the group radius about z_o), S_g, 0, 0
  };
  static constexpr int kGroup = 64;
  static constexpr float kNearFactor = 4.0f;    // direct form for targets within 4 R
  static constexpr float kMaxFarRadius = 2.0f;  // wider groups: direct form for all targets
};

struct BetaRelArgs {
  const double *x, *y;
  const BetaRel::Rec* src;
  const BetaRel::Origin* org;
  int64_t n_tiles, tiles_per_chunk, ib, nt;
  double* partial;  // [chunk][2][nt]
  int* status;
};

template <int THREADS, int TPT, int TILE, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) beta_rel_sweep_kernel(BetaRelArgs a) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  static_assert(TILE % BetaRel::kGroup == 0, "whole origin groups per tile");
  constexpr int NP = TPT / 2;
  constexpr int G = BetaRel::kGroup;
  constexpr int GPT = TILE / G;
  using Rec = BetaRel::Rec;
  __shared__ __align__(128) Rec stage[2][TILE];
  __shared__ __align__(8) uint64_t bars[2];

  const int64_t chunk = blockIdx.y;
  const int64_t tile0 = chunk * a.tiles_per_chunk;
  int64_t ntl = a.n_tiles - tile0;
  if (ntl > a.tiles_per_chunk) ntl = a.tiles_per_chunk;
  if (ntl < 0) ntl = 0;

  BetaTgt tg[2 * NP];
  float hu[2 * NP], lu[2 * NP], hv[2 * NP], lv[2 * NP];
  const int64_t first = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT);
  const int64_t count = a.nt - first < THREADS * TPT ? a.nt - first : THREADS * TPT;
#pragma unroll
  for (int t = 0; t < 2 * NP; ++t) {
    int64_t il = t * THREADS + threadIdx.x;
    if (il >= count) il = count - 1;  // duplicates of a valid target; results not stored
    split2(a.x[a.ib + first + il], tg[t].xh, tg[t].xl);
    split2(a.y[a.ib + first + il], tg[t].yh, tg[t].yl);
    hu[t] = lu[t] = hv[t] = lv[t] = 0.f;
  }

  pipe_init(bars);
  uint32_t g = 0;
  int64_t tile = tile0;
  staged_sweep<Rec, TILE>(a.src, tile0, ntl, stage[0], stage[1], bars, g, a.status, [&](const Rec* tl) {
    float au[2 * NP], av[2 * NP];
#pragma unroll
    for (int t = 0; t < 2 * NP; ++t) au[t] = av[t] = 0.f;
    const BetaRel::Origin* og = a.org + tile * GPT;
#pragma unroll 1
    for (int g0 = 0; g0 < TILE; g0 += G) {
      const BetaRel::Origin o = og[g0 / G];
      const Rec* gr = tl + g0;
      // offsets from the centroid, x wrapped into [-1/2, 1/2]
      float2 dx[NP], dy[NP];
      bool near = false;
      // (every target within 0.02 of the centroid takes the direct form too: the error of e_i
      // weighs 1 / (2 pi |z_i - z_j|) in the complex one)
      const float lim = fmaxf((BetaRel::kNearFactor * o.f.x) * (BetaRel::kNearFactor * o.f.x), 4e-4f);
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const BetaTgt& t0 = tg[2 * p];
        const BetaTgt& t1 = tg[2 * p + 1];
        // the wrapped x offset keeps the rounding of its hi difference (the phase of e_i needs
        // it to ~2^-24 of the wrapped value), as beta_deltas2 does for a source
        const float4 oa = make_float4(o.o.x, o.o.y, o.o.z, o.o.w);
        beta_deltas2(t0, t1, oa, dx[p], dy[p]);
        const float2 n2 = __ffma2_rn(dy[p], dy[p], __fmul2_rn(dx[p], dx[p]));
        near |= !(n2.x > lim) | !(n2.y > lim);
      }
      if (!__any_sync(0xffffffffu, near)) {
        // complex far form: G = sum S_j e_j / (e_i - e_j)
        float2 er[NP], ei[NP], gre[NP], gim[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          float s0, c0, s1, c1;
          sincospif(2.0f * dx[p].x, &s0, &c0);
          sincospif(2.0f * dx[p].y, &s1, &c1);
          // |y_i - y_o| is clamped to 6, so |e_i|^2 <= e^(24 pi) stays finite; a far group has
          // R <= 2, so the clamp moves a term by at most e^(2 pi (2 - 6)) ~ 1e-11 of S_j
          const float m0 = expf(-6.2831853f * fminf(fmaxf(dy[p].x, -6.0f), 6.0f));
          const float m1 = expf(-6.2831853f * fminf(fmaxf(dy[p].y, -6.0f), 6.0f));
          er[p] = make_float2(m0 * c0, m1 * c1);
          ei[p] = make_float2(m0 * s0, m1 * s1);
          gre[p] = gim[p] = make_float2(0.f, 0.f);
        }
#pragma unroll 2
        for (int j = 0; j < G; ++j) {
          const float4 rc = gr[j].c, rd = gr[j].d;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 br = __fadd2_rn(er[p], make_float2(-rc.x, -rc.y));
            const float2 bi = __fadd2_rn(ei[p], make_float2(-rc.z, -rc.w));
            const float2 mm = __ffma2_rn(bi, bi, __fmul2_rn(br, br));
            const float2 inv = make_float2(rcp_approx(mm.x), rcp_approx(mm.y));
            // S e_j conj(b) = (Ser br + Sei bi) + i (Sei br - Ser bi)
            const float2 nr = __ffma2_rn(hi2(rd), bi, __fmul2_rn(lo2(rd), br));
            const float2 ni = __ffma2_rn(make_float2(-rd.x, -rd.y), bi, __fmul2_rn(hi2(rd), br));
            gre[p] = __ffma2_rn(nr, inv, gre[p]);
            gim[p] = __ffma2_rn(ni, inv, gim[p]);
          }
        }
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          au[2 * p] += o.f.y + 2.0f * gre[p].x;
          au[2 * p + 1] += o.f.y + 2.0f * gre[p].y;
          av[2 * p] -= 2.0f * gim[p].x;
          av[2 * p + 1] -= 2.0f * gim[p].y;
        }
      } else {
        // direct form (cancellation-free half angles), the self pair a zero term
        for (int j = 0; j < G; ++j) {
          BetaF32::Rec r;
          r.a = gr[j].a;
          r.b = gr[j].b;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            float a0[2] = {au[2 * p], av[2 * p]}, a1[2] = {au[2 * p + 1], av[2 * p + 1]};
            BetaF32::interact2(tg[2 * p], tg[2 * p + 1], r, a0, a1);
            au[2 * p] = a0[0];
            av[2 * p] = a0[1];
            au[2 * p + 1] = a1[0];
            av[2 * p + 1] = a1[1];
          }
        }
      }
    }
    ++tile;
#pragma unroll
    for (int t = 0; t < 2 * NP; ++t) {
      comp_add(hu[t], lu[t], au[t]);
      comp_add(hv[t], lv[t], av[t]);
    }
  });

#pragma unroll
  for (int p = 0; p < NP; ++p) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int t = 2 * p + h;
      const int64_t il = first + t * THREADS + threadIdx.x;
      if (il < a.nt) {
        a.partial[(chunk * 2 + 0) * a.nt + il] = static_cast<double>(hu[t]) + static_cast<double>(lu[t]);
        a.partial[(chunk * 2 + 1) * a.nt + il] = static_cast<double>(hv[t]) + static_cast<double>(lv[t]);
      }
    }
  }
}

// Records and origins of one tile of TILE sources (one CTA of TILE threads): each group of
// kGroup sources reduces its centroid z_o, its radius R about z_o and S_g; e_j = exp(2 pi i
// (z_j - z_o)) and S_j e_j are formed in FP64 and rounded.
template <int TILE>
__global__ void __launch_bounds__(TILE) beta_rel_prep_kernel(const double* x, const double* y, const double* zeta,
                                                             const double* area, const int32_t* sorted, int64_t ns,
                                                             BetaRel::Rec* out, BetaRel::Origin* org) {
  constexpr int G = BetaRel::kGroup;
  __shared__ double red[3][TILE];
  __shared__ float fmax_[TILE], cntf[TILE];
  const int64_t t = blockIdx.x;
  const int tid = threadIdx.x;
  const int64_t k = t * TILE + tid;
  const bool valid = k < ns;
  const int32_t j = valid ? sorted[k] : 0;
  const int lane = tid % G;
  const double px = valid ? x[j] : 0.0, py = valid ? y[j] : 0.0;
  const float sf = valid ? __double2float_rn(0.5 * zeta[j] * area[j]) : 0.f;
  red[0][tid] = px;
  red[1][tid] = py;
  red[2][tid] = sf;
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
  BetaRel::Rec r;
  if (valid) {
    float h, l;
    split2(px, h, l);
    r.a.x = h;
    r.a.z = l;
    split2(py, h, l);
    r.a.y = h;
    r.a.w = l;
    r.b = make_float4(sf, 0.f, 0.f, 0.f);
    double sn, cs;
    sincospi(2.0 * (px - cx), &sn, &cs);
    const double m = exp(-2.0 * 3.1415926535897932384626433832795 * (py - cy));
    const double ere = m * cs, eim = m * sn;
    const float fre = __double2float_rn(ere), fim = __double2float_rn(eim);
    const float sre = __double2float_rn(static_cast<double>(sf) * ere), sim = __double2float_rn(static_cast<double>(sf) * eim);
    r.c = make_float4(fre, fre, fim, fim);
    r.d = make_float4(sre, sre, sim, sim);
  } else {
    // inert: zero strength at the centroid (e = 1; a target there is near: direct form, S = 0)
    r.a = make_float4(static_cast<float>(cx), static_cast<float>(cy), 0.f, 0.f);
    r.b = make_float4(0.f, 0.f, 0.f, 0.f);
    r.c = make_float4(1.f, 1.f, 0.f, 0.f);
    r.d = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  out[k] = r;
  if (lane == 0) {
    BetaRel::Origin o;
    float oxh, oxl, oyh, oyl;
    split2(cx, oxh, oxl);
    split2(cy, oyh, oyl);
    o.o = make_float4(oxh, oyh, oxl, oyl);
    // a group wider than 2 (|e_j| up to e^(2 pi R)) is summed with the direct form by every
    // target: its R is replaced by a value whose near limit (4 R)^2 is infinite
    const float rg = fmax_[g0] <= BetaRel::kMaxFarRadius ? fmax_[g0] : 3e37f;
    o.f = make_float4(rg, __double2float_rn(red[2][g0]), 0.f, 0.f);
    org[t * (TILE / G) + tid / G] = o;
  }
}

// Offsets of two targets from a float origin (x_o, y_o) as float-float pairs: the x offset
// wrapped into [-1/2, 1/2] (t_hi = (x_hi - x_o) - rint(x_hi - x_o) is exact), each hi part
// carrying the rounding of its difference (TwoSum) and the target's lo part.
__device__ __forceinline__ void beta_offsets_ff(const BetaTgt& t0, const BetaTgt& t1, float xo, float yo, float2& xh,
                                                float2& xl, float2& yh, float2& yl) {
  const float2 kM = make_float2(12582912.0f, 12582912.0f), kNM = make_float2(-12582912.0f, -12582912.0f);
  const float2 nxo = make_float2(-xo, -xo), nyo = make_float2(-yo, -yo);
  const float2 tx = make_float2(t0.xh, t1.xh), ty = make_float2(t0.yh, t1.yh);
  // TwoSum(tx, -xo) and TwoSum(ty, -yo)
  const float2 dx = __fadd2_rn(tx, nxo), dy = __fadd2_rn(ty, nyo);
  const float2 bx = __fadd2_rn(dx, make_float2(-tx.x, -tx.y)), by = __fadd2_rn(dy, make_float2(-ty.x, -ty.y));
  const float2 ex = __fadd2_rn(__fadd2_rn(tx, make_float2(-(dx.x - bx.x), -(dx.y - bx.y))),
                               __fadd2_rn(nxo, make_float2(-bx.x, -bx.y)));
  const float2 ey = __fadd2_rn(__fadd2_rn(ty, make_float2(-(dy.x - by.x), -(dy.y - by.y))),
                               __fadd2_rn(nyo, make_float2(-by.x, -by.y)));
  const float2 nn = __fadd2_rn(__fadd2_rn(dx, kM), kNM);
  const float2 th = __fadd2_rn(dx, make_float2(-nn.x, -nn.y));
  const float2 tl = __fadd2_rn(ex, make_float2(t0.xl, t1.xl));
  const float2 ul = __fadd2_rn(ey, make_float2(t0.yl, t1.yl));
  // renormalise (Fast2Sum: |lo| is below an ulp of the difference or the hi part is 0)
  xh = __fadd2_rn(th, tl);
  xl = __fadd2_rn(tl, make_float2(-(xh.x - th.x), -(xh.y - th.y)));
  yh = __fadd2_rn(dy, ul);
  yl = __fadd2_rn(ul, make_float2(-(yh.x - dy.x), -(yh.y - dy.y)));
}

// ============================================================ beta-plane stream functions
// The beta plane's SetStreamFunctionsOnMesh, src/BetaPlaneSolver.f90 (the x-periodic kernel
// g = ln(cosh 2 pi dy - cos 2 pi dx) / (4 pi), psi_rel += g zeta_j A_j, psi_abs += g
// (zeta_j + f_j) A_j, j != i) on the same groups.  With e as above,
//   |e_i - e_j|^2 = 2 |e_i| |e_j| (cosh 2 pi dy - cos 2 pi dx),  ln|e| = -2 pi (y - y_o),
// so a far group adds  sum_j w_j ln|e_i - e_j|^2 + W (2 pi (y_i - y_o)) + C,
//   W = sum_j w_j,  C = sum_j w_j (2 pi (y_j - y_o) - ln 2)   (w = q A / (4 pi); W, C per group).
// Per target pair and source: e_i - e_j (2 FADD2), |.|^2 (2), the accurate log of
// ln_q2_shift (csrc/stream_rel.cuh) and two accumulations.  The log is taken less s ln 2,
// s the exponent of |e_i - 1|^2 (exact, it only moves the exponent), so the 64 terms of a
// group are O(1) and their FP32 sum loses nothing to the group's common log; W s ln 2 goes
// back in once per group.  The far form needs |y_i - y_o| <= 6 besides the distance test (no
// clamp: the log keeps the linear growth in |dy|); other warps take BetaStreamF32's direct
// form, flushed every 8 sources.  The origin is the centroid rounded to float (no lo part),
// the same point the prep kernel forms e_j about.
struct BetaStreamRel {
  struct __align__(16) Rec {
    float4 a;  // x_hi, y_hi, x_lo, y_lo                 (direct form)
    float4 b;  // w_rel, w_abs, 0, 0                     (w = q A / (4 pi))
    float4 c;  // e.re, e.re, e.im, e.im
  };
  struct __align__(16) Origin {
    float4 o;  // x_o, y_o (floats), R, W_rel
    float4 f;  // W_abs, C_rel, C_abs, 0
  };
  static constexpr int kGroup = 64;
  static constexpr float kNearFactor = BetaRel::kNearFactor;
  static constexpr float kMaxFarRadius = BetaRel::kMaxFarRadius;
  static constexpr float kMaxFarDy = 6.0f;  // |y_i - y_o| for the complex form (|e_i|^2 <= e^(24 pi))
};

struct BetaStreamRelArgs {
  const double *x, *y;
  const BetaStreamRel::Rec* src;
  const BetaStreamRel::Origin* org;
  int64_t n_tiles, tiles_per_chunk, ib, nt;
  double* partial;  // [chunk][2][nt]
  int* status;
};

template <int THREADS, int TPT, int TILE, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) beta_stream_rel_sweep_kernel(BetaStreamRelArgs a) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  static_assert(TILE % BetaStreamRel::kGroup == 0, "whole origin groups per tile");
  constexpr int NP = TPT / 2;
  constexpr int G = BetaStreamRel::kGroup;
  constexpr int GPT = TILE / G;
  // the direct form's terms are flushed every 8 sources: sorted sources bring runs of
  // same-sign terms of up to ~40 w each (2 pi |dy| for |dy| <= 6)
  constexpr int FL = 8;
  static_assert(G % FL == 0, "whole flushes per group");
  using Rec = BetaStreamRel::Rec;
  __shared__ __align__(128) Rec stage[2][TILE];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ __align__(8) float2 ln_tab[32];

  const int64_t chunk = blockIdx.y;
  const int64_t tile0 = chunk * a.tiles_per_chunk;
  int64_t ntl = a.n_tiles - tile0;
  if (ntl > a.tiles_per_chunk) ntl = a.tiles_per_chunk;
  if (ntl < 0) ntl = 0;

  BetaTgt tg[2 * NP];
  float hr[2 * NP], lr[2 * NP], ha[2 * NP], la[2 * NP];
  const int64_t first = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT);
  const int64_t count = a.nt - first < THREADS * TPT ? a.nt - first : THREADS * TPT;
#pragma unroll
  for (int t = 0; t < 2 * NP; ++t) {
    int64_t il = t * THREADS + threadIdx.x;
    if (il >= count) il = count - 1;  // duplicates of a valid target; results not stored
    split2(a.x[a.ib + first + il], tg[t].xh, tg[t].xl);
    split2(a.y[a.ib + first + il], tg[t].yh, tg[t].yl);
    hr[t] = lr[t] = ha[t] = la[t] = 0.f;
  }

  ln_tab_load(ln_tab);
  pipe_init(bars);
  uint32_t g = 0;
  int64_t tile = tile0;
  staged_sweep<Rec, TILE>(a.src, tile0, ntl, stage[0], stage[1], bars, g, a.status, [&](const Rec* tl) {
    const BetaStreamRel::Origin* og = a.org + tile * GPT;
#pragma unroll 1
    for (int g0 = 0; g0 < TILE; g0 += G) {
      const BetaStreamRel::Origin o = og[g0 / G];
      const Rec* gr = tl + g0;
      float2 dx[NP], dxl[NP], dy[NP], dyl[NP];
      bool near = false;
      const float lim =
          fmaxf((BetaStreamRel::kNearFactor * o.o.z) * (BetaStreamRel::kNearFactor * o.o.z), 4e-4f);
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        beta_offsets_ff(tg[2 * p], tg[2 * p + 1], o.o.x, o.o.y, dx[p], dxl[p], dy[p], dyl[p]);
        const float2 n2 = __ffma2_rn(dy[p], dy[p], __fmul2_rn(dx[p], dx[p]));
        const float2 ady = bits_abs(dy[p]);
        near |= !(n2.x > lim) | !(n2.y > lim) | !(ady.x <= BetaStreamRel::kMaxFarDy) |
                !(ady.y <= BetaStreamRel::kMaxFarDy);
      }
      float2 ar[NP], aa[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) ar[p] = aa[p] = make_float2(0.f, 0.f);
      if (!__any_sync(0xffffffffu, near)) {
        // e_i from A = 2 pi (y_i - y_o) and 2 pi (x_i - x_o) as float-float values: an error in
        // them is common to the group's 64 terms (it is 2^-24 |A| for A rounded once)
        constexpr float k2PiH = 6.2831854820251465f, k2PiL = -1.7484556025237907e-07f;
        constexpr float kLn2H = 0.693145751953125f, kLn2L = 1.4286068202862268e-06f;
        float2 er[NP], ei[NP], bias[NP], kh[NP], kl[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          float s0, c0, s1, c1;
          sincospif(2.0f * dx[p].x, &s0, &c0);
          sincospif(2.0f * dx[p].y, &s1, &c1);
          // rotate by 2 pi x_lo (|x_lo| <= 2^-25: first order is exact to float)
          const float2 dl = __fmul2_rn(make_float2(k2PiH, k2PiH), dxl[p]);
          const float2 cc = __ffma2_rn(make_float2(-s0, -s1), dl, make_float2(c0, c1));
          const float2 ss = __ffma2_rn(make_float2(c0, c1), dl, make_float2(s0, s1));
          const float2 ah = __fmul2_rn(make_float2(k2PiH, k2PiH), dy[p]);
          const float2 al = __fadd2_rn(make_float2(fmaf(k2PiH, dy[p].x, -ah.x), fmaf(k2PiH, dy[p].y, -ah.y)),
                                       __ffma2_rn(make_float2(k2PiH, k2PiH), dyl[p],
                                                  __fmul2_rn(make_float2(k2PiL, k2PiL), dy[p])));
          // |e_i| = e^(-A) = e^(-ah) (1 - al), |al| < 2^-20
          const float2 m = __fmul2_rn(make_float2(expf(-ah.x), expf(-ah.y)),
                                      __fadd2_rn(make_float2(1.0f, 1.0f), make_float2(-al.x, -al.y)));
          er[p] = __fmul2_rn(m, cc);
          ei[p] = __fmul2_rn(m, ss);
          // s = the exponent of |e_i - 1|^2 (a normal float: |z_i - z_o| >= 0.02)
          const float2 d1 = __fadd2_rn(er[p], make_float2(-1.0f, -1.0f));
          const float2 m2 = __ffma2_rn(ei[p], ei[p], __fmul2_rn(d1, d1));
          const int e0 = static_cast<int>(__float_as_uint(m2.x) >> 23) - 127;
          const int e1 = static_cast<int>(__float_as_uint(m2.y) >> 23) - 127;
          bias[p] = shift_bias(e0, e1);
          // the group's constant per unit weight, s ln 2 + A, as kh + kl (s ln2_hi is exact)
          const float2 sl = __fmul2_rn(make_float2(static_cast<float>(e0), static_cast<float>(e1)),
                                       make_float2(kLn2H, kLn2H));
          kh[p] = __fadd2_rn(sl, ah);
          const float2 bb = __fadd2_rn(kh[p], make_float2(-sl.x, -sl.y));
          const float2 te = __fadd2_rn(__fadd2_rn(sl, make_float2(-(kh[p].x - bb.x), -(kh[p].y - bb.y))),
                                       __fadd2_rn(ah, make_float2(-bb.x, -bb.y)));
          kl[p] = __fadd2_rn(__fadd2_rn(te, al), __fmul2_rn(make_float2(static_cast<float>(e0), static_cast<float>(e1)),
                                                            make_float2(kLn2L, kLn2L)));
        }
#pragma unroll 2
        for (int j = 0; j < G; ++j) {
          const float4 rb = gr[j].b, rc = gr[j].c;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 br = __fadd2_rn(er[p], make_float2(-rc.x, -rc.y));
            const float2 bi = __fadd2_rn(ei[p], make_float2(-rc.z, -rc.w));
            const float2 mm = __ffma2_rn(bi, bi, __fmul2_rn(br, br));
            const float2 lg = ln_q2_shift(mm, bias[p], ln_tab);
            ar[p] = __ffma2_rn(make_float2(rb.x, rb.x), lg, ar[p]);
            aa[p] = __ffma2_rn(make_float2(rb.y, rb.y), lg, aa[p]);
          }
        }
        // W (kh + kl) + C + the terms: W kh by TwoProduct, every part compensated
        const float wr = o.o.w, wa = o.f.x;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const int t = 2 * p + h;
            const float k_h = h ? kh[p].y : kh[p].x, k_l = h ? kl[p].y : kl[p].x;
            const float pr = wr * k_h, pa = wa * k_h;
            comp_add(hr[t], lr[t], pr);
            comp_add(hr[t], lr[t], o.f.y);
            comp_add(hr[t], lr[t], fmaf(wr, k_l, fmaf(wr, k_h, -pr)) + (h ? ar[p].y : ar[p].x));
            comp_add(ha[t], la[t], pa);
            comp_add(ha[t], la[t], o.f.z);
            comp_add(ha[t], la[t], fmaf(wa, k_l, fmaf(wa, k_h, -pa)) + (h ? aa[p].y : aa[p].x));
          }
        }
      } else {
        // direct form, the self pair a zero term, flushed every FL sources
#pragma unroll 1
        for (int j0 = 0; j0 < G; j0 += FL) {
          for (int j = j0; j < j0 + FL; ++j) {
            BetaStreamF32::Rec r;
            r.a = gr[j].a;
            r.b = gr[j].b;
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              float a0[2] = {ar[p].x, aa[p].x}, a1[2] = {ar[p].y, aa[p].y};
              BetaStreamF32::interact2(tg[2 * p], tg[2 * p + 1], r, a0, a1, ln_tab);
              ar[p] = make_float2(a0[0], a1[0]);
              aa[p] = make_float2(a0[1], a1[1]);
            }
          }
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            comp_add(hr[2 * p], lr[2 * p], ar[p].x);
            comp_add(hr[2 * p + 1], lr[2 * p + 1], ar[p].y);
            comp_add(ha[2 * p], la[2 * p], aa[p].x);
            comp_add(ha[2 * p + 1], la[2 * p + 1], aa[p].y);
            ar[p] = aa[p] = make_float2(0.f, 0.f);
          }
        }
      }
    }
    ++tile;
  });

#pragma unroll
  for (int p = 0; p < NP; ++p) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int t = 2 * p + h;
      const int64_t il = first + t * THREADS + threadIdx.x;
      if (il < a.nt) {
        a.partial[(chunk * 2 + 0) * a.nt + il] = static_cast<double>(hr[t]) + static_cast<double>(lr[t]);
        a.partial[(chunk * 2 + 1) * a.nt + il] = static_cast<double>(ha[t]) + static_cast<double>(la[t]);
      }
    }
  }
}

// Records and origins of one tile for the stream functions: the group centroid rounded to
// float is the origin; e_j, W and C are formed in FP64 about it.
template <int TILE>
__global__ void __launch_bounds__(TILE) beta_stream_rel_prep_kernel(const double* x, const double* y,
                                                                    const double* qr, const double* qa,
                                                                    const double* area, const int32_t* sorted,
                                                                    int64_t ns, BetaStreamRel::Rec* out,
                                                                    BetaStreamRel::Origin* org) {
  constexpr int G = BetaStreamRel::kGroup;
  constexpr double kTwoPi = 6.283185307179586476925286766559;
  constexpr double kLn2 = 0.69314718055994530941723212145818;
  __shared__ double red[4][TILE];
  __shared__ float fmax_[TILE], cntf[TILE];
  const int64_t t = blockIdx.x;
  const int tid = threadIdx.x;
  const int64_t k = t * TILE + tid;
  const bool valid = k < ns;
  const int32_t j = valid ? sorted[k] : 0;
  const int lane = tid % G;
  const int g0 = tid - lane;
  const double px = valid ? x[j] : 0.0, py = valid ? y[j] : 0.0;
  const float wr = valid ? __double2float_rn(qr[j] * area[j] * kInv4Pi) : 0.f;
  const float wa = valid ? __double2float_rn(qa[j] * area[j] * kInv4Pi) : 0.f;
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
  const double cnt = cntf[g0] > 0.f ? static_cast<double>(cntf[g0]) : 1.0;
  // the origin: the centroid rounded to float, exactly the point the sweep subtracts
  const double cx = static_cast<double>(__double2float_rn(red[0][g0] / cnt));
  const double cy = static_cast<double>(__double2float_rn(red[1][g0] / cnt));
  fmax_[tid] = valid ? static_cast<float>(sqrt((px - cx) * (px - cx) + (py - cy) * (py - cy))) : 0.f;
  __syncthreads();
  // W and C of both strengths (the weights as rounded into the records)
  const double c_arg = kTwoPi * (py - cy) - kLn2;
  red[0][tid] = wr;
  red[1][tid] = wa;
  red[2][tid] = static_cast<double>(wr) * c_arg;
  red[3][tid] = static_cast<double>(wa) * c_arg;
  __syncthreads();
  for (int w = G / 2; w > 0; w >>= 1) {
    if (lane < w) {
      fmax_[tid] = fmaxf(fmax_[tid], fmax_[tid + w]);
#pragma unroll
      for (int c = 0; c < 4; ++c) red[c][tid] += red[c][tid + w];
    }
    __syncthreads();
  }
  BetaStreamRel::Rec r;
  if (valid) {
    float h, l;
    split2(px, h, l);
    r.a.x = h;
    r.a.z = l;
    split2(py, h, l);
    r.a.y = h;
    r.a.w = l;
    r.b = make_float4(wr, wa, 0.f, 0.f);
    double sn, cs;
    sincospi(2.0 * (px - cx), &sn, &cs);
    const double m = exp(-kTwoPi * (py - cy));
    const float fre = __double2float_rn(m * cs), fim = __double2float_rn(m * sn);
    r.c = make_float4(fre, fre, fim, fim);
  } else {
    // inert: zero strength at the origin
    r.a = make_float4(static_cast<float>(cx), static_cast<float>(cy), 0.f, 0.f);
    r.b = make_float4(0.f, 0.f, 0.f, 0.f);
    r.c = make_float4(1.f, 1.f, 0.f, 0.f);
  }
  out[k] = r;
  if (lane == 0) {
    BetaStreamRel::Origin o;
    const float rg = fmax_[g0] <= BetaStreamRel::kMaxFarRadius ? fmax_[g0] : 3e37f;
    o.o = make_float4(static_cast<float>(cx), static_cast<float>(cy), rg, __double2float_rn(red[0][g0]));
    o.f = make_float4(__double2float_rn(red[1][g0]), __double2float_rn(red[2][g0]), __double2float_rn(red[3][g0]),
                      0.f);
    org[t * (TILE / G) + tid / G] = o;
  }
}

}  // namespace lpm
