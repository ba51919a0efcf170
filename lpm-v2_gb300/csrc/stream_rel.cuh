// stream_rel.cuh -- the sphere stream functions in FP32C on the group-relative layout of the
// BVE sweep (bve_rel.cuh): Hilbert-sorted sources, offsets from each group's centroid, the
// compact / far / near precision choice, and target pairs in packed FP32x2 arithmetic.
//
// Reference: SetStreamFunctionsOnMesh, src/SphereBVE.f90:445-485:
//   psi_i = -1/(4 pi) sum_{j != i} ln(a^2 - x_i.x_j) zeta_j A_j   (relative and absolute zeta)
// With p = x / a and c = |p|^2 - 1, a^2 - x_i.x_j = (a^2 / 2) q_ij with q_ij = |d|^2 - c_i - c_j
// (exact), so
//   psi_i = sum_{j != i} S_j ln q_ij - ln(a^2 / 2) / (4 pi) sum_{j != i} zeta_j A_j,
// S_j = -zeta_j A_j / (4 pi).  The sweep forms the first sum; the finish adds the second from
// a fixed-order FP64 total minus the target's own term.  Per target pair and source, far
// warp (every target beyond 3R of the group's centroid): the expanded form of the BVE sweep,
// h = q/2 = (|t|^2 - c_i)/2 + B_j/2 - t.s_j (4 packed), ln q = ln h + ln 2 (ln_q2_shift:
// integer exponent split, a table load per lane, 9 packed) and the two accumulations; no
// select, since q > 0.  A compact group near the warp takes d = t_hi - s_hi with the
// self-pair select and the clamp to >= 2^-126, any other near group the two-float form.  The
// FP32 partials are flushed into compensated (hi, lo) pairs every 32 sources, because the
// terms cancel to a much smaller psi.  The sphere sweep runs on the warp-decoupled pipeline
// (engine.cuh, the group origins copied with each tile): warps meet near and far groups at
// different rates, and it measured 3.5 % faster than the block-synchronous one.
#pragma once

#include "bve_rel.cuh"
#include "ln_table.cuh"
#include "ops.cuh"
#include "plane_rel.cuh"

namespace lpm {

struct StreamRel {
  struct __align__(16) Rec {
    float4 a;  // -sx_hi, -sx_hi, -sy_hi, -sy_hi
    float4 b;  // -sz_hi, -sz_hi, -c_j, -c_j
    float4 c;  // S_rel, S_rel, S_abs, S_abs
    float4 d;  // -sx_lo, -sx_lo, -sy_lo, -sy_lo
    float4 e;  // -sz_lo, -sz_lo, B_j / 2, B_j / 2   (B_j = |s_hi|^2 - c_j)
  };
  static constexpr int kFlush = 32;
};

// Natural log of two positive normal floats (the sweeps clamp them): per lane q = 2^k m with
// m in [sqrt(1/2), sqrt(2)) (an integer split; 0x3f3504f3 = fl(sqrt(1/2))).  Bits 19..23 of
// m pick (inv, ln c) from a 32-entry table in shared memory (ln_table.cuh: 1/c for c the
// midpoint of the key's interval, with ln c exact to ~2e-4 ulp in float -- Gal's accurate
// tables).  Then, packed, r = m inv - 1 (one FMA, |r| <= 0.0305, exact to 2^-30),
// ln(1 + r) = r + r^2 (-1/2 + r/3 - r^2/4 + r^3/5) (truncated at r^6/6 < 2e-10), and
// ln q = (k ln 2 + ln c) + ln(1 + r): 9 packed operations and two 8-byte shared loads (keys
// 6 and 22 alone share banks), no MUFU; good to about 1 ulp of the larger part.
// The exponent split of a positive normal float with bits b: q = 2^k m, m in [sqrt(1/2),
// sqrt(2)) (0x3f3504f3 = fl(sqrt(1/2))); returns k and writes the bits of m.  Inline PTX
// keeps the integer sequence as written: the same four operations in C++, fed straight
// from a packed FFMA2 result in the planar stream sweep's far loop, gave (nvcc 13.0,
// sm_103a) logs as if k were b - 0x3f3504f3, unshifted.
__device__ __forceinline__ int exp_split(int b, int& mb) {
  int k;
  asm("{\n\t.reg .s32 t;\n\tsub.s32 t, %2, 0x3f3504f3;\n\tshr.s32 %0, t, 23;\n\tshl.b32 t, %0, 23;\n\t"
      "sub.s32 %1, %2, t;\n\t}"
      : "=r"(k), "=r"(mb)
      : "r"(b));
  return k;
}

// ln_q2_shift(q, shift_bias(s0, s1)) is (ln q.x - s0 ln 2, ln q.y - s1 ln 2) for small
// integers s: the shift only moves the exponent k (the float k - s is exact), so it costs
// nothing -- it replaces the constant of the magic-number conversion of k.
__device__ __forceinline__ float2 shift_bias(int s0, int s1) {
  return make_float2(-12582912.0f - static_cast<float>(s0), -12582912.0f - static_cast<float>(s1));
}

// The table into shared memory (threads 0..31; the caller's next __syncthreads publishes it).
__device__ __forceinline__ void ln_tab_load(float2* tab) {
  if (threadIdx.x < 32) tab[threadIdx.x] = make_float2(kLnTabInv[threadIdx.x], kLnTabLog[threadIdx.x]);
}

__device__ __forceinline__ float2 ln_q2_shift(float2 q, float2 bias, const float2* tab) {
  int m0, m1;
  const int k0 = exp_split(__float_as_int(q.x), m0), k1 = exp_split(__float_as_int(q.y), m1);
  const float2 e0 = tab[(m0 >> 19) & 31], e1 = tab[(m1 >> 19) & 31];
  const float2 m = make_float2(__int_as_float(m0), __int_as_float(m1));
  const float2 kf = __fadd2_rn(make_float2(__int_as_float(k0 + 0x4b400000), __int_as_float(k1 + 0x4b400000)), bias);
  const float2 r = __ffma2_rn(m, make_float2(e0.x, e1.x), make_float2(-1.0f, -1.0f));
  float2 p = __ffma2_rn(make_float2(0.2f, 0.2f), r, make_float2(-0.25f, -0.25f));
  p = __ffma2_rn(p, r, make_float2(0.33333334f, 0.33333334f));
  p = __ffma2_rn(p, r, make_float2(-0.5f, -0.5f));
  const float2 b = __ffma2_rn(__fmul2_rn(r, r), p, r);
  const float2 a = __ffma2_rn(kf, make_float2(0.69314718f, 0.69314718f), make_float2(e0.y, e1.y));
  return __fadd2_rn(a, b);
}

__device__ __forceinline__ float2 ln_q2(float2 q, const float2* tab) { return ln_q2_shift(q, shift_bias(0, 0), tab); }

// The log argument of a pair: q clamped to >= 2^-126, or 1 (a zero term) when d = 0.
__device__ __forceinline__ float2 stream_arg(float2 u, float2 q) {
  return make_float2(u.x != 0.0f ? fmaxf(q.x, kLogFloor) : 1.0f, u.y != 0.0f ? fmaxf(q.y, kLogFloor) : 1.0f);
}

template <int NP>
__device__ __forceinline__ void stream_flush(float2 (&ar)[NP], float2 (&aa)[NP], float2 (&hr)[NP], float2 (&lr)[NP],
                                             float2 (&ha)[NP], float2 (&la)[NP]) {
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    comp_add(hr[p].x, lr[p].x, ar[p].x);
    comp_add(hr[p].y, lr[p].y, ar[p].y);
    comp_add(ha[p].x, la[p].x, aa[p].x);
    comp_add(ha[p].y, la[p].y, aa[p].y);
    ar[p] = aa[p] = make_float2(0.f, 0.f);
  }
}

template <int THREADS, int TPT, int TILE, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) stream_rel_sweep_kernel(SweepArgs<BveF32> a,
                                                                         const StreamRel::Rec* __restrict__ src,
                                                                         const BveRel::Origin* __restrict__ org) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  constexpr int NP = TPT / 2;
  constexpr int G = BveRel::kGroup;
  constexpr int GPT = TILE / G;
  constexpr int FL = StreamRel::kFlush;
  static_assert(G % FL == 0, "flush interval must divide the group");
  using Rec = StreamRel::Rec;
  __shared__ TilePipe<Rec, TILE, 2, BveRel::Origin, GPT> pipe;
  __shared__ __align__(8) float2 ln_tab[32];

  const int64_t chunk = blockIdx.y;
  const int64_t tile0 = chunk * a.tiles_per_chunk;
  int64_t ntl = a.n_tiles - tile0;
  if (ntl > a.tiles_per_chunk) ntl = a.tiles_per_chunk;
  if (ntl < 0) ntl = 0;

  BveX2::Pair pr[NP];
  float2 hr[NP], lr[NP], ha[NP], la[NP], ar[NP], aa[NP];
  const int64_t first = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT);
  const int64_t count = a.nt - first < THREADS * TPT ? a.nt - first : THREADS * TPT;
  bve_load_pairs<NP>(a.p, a.ib + first, count, THREADS, pr);
#pragma unroll
  for (int p = 0; p < NP; ++p) hr[p] = lr[p] = ha[p] = la[p] = ar[p] = aa[p] = make_float2(0.f, 0.f);

  ln_tab_load(ln_tab);
  tile_pipe_init(pipe);
  uint32_t g = 0;
  warp_sweep(src, tile0, ntl, pipe, g, a.status, default_wait(), org, [&](const Rec* tl, const BveRel::Origin* og) {
#pragma unroll 1
    for (int g0 = 0; g0 < TILE; g0 += G) {
      const BveRel::Origin o = og[g0 / G];
      const Rec* gr = tl + g0;
      float2 tx[NP], ty[NP], tz[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        tx[p] = rel1x2(pr[p].xh, pr[p].xl, o.hi.x, o.lo.x);
        ty[p] = rel1x2(pr[p].yh, pr[p].yl, o.hi.y, o.lo.y);
        tz[p] = rel1x2(pr[p].zh, pr[p].zl, o.hi.z, o.lo.z);
      }
      // far: every target of the warp beyond 3R (and off the centroid of a zero-radius group)
      const float rg = fabsf(o.hi.w);
      const float lim = fmaxf((BveRel::kNearFactor * rg) * (BveRel::kNearFactor * rg), 7.888609052210118e-31f);
      bool nearw = false;
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const float2 n2 = __ffma2_rn(tz[p], tz[p], __ffma2_rn(ty[p], ty[p], __fmul2_rn(tx[p], tx[p])));
        nearw |= !(n2.x > lim) | !(n2.y > lim);
      }
      if (!__any_sync(0xffffffffu, nearw)) {
        // expanded form: h = q/2 = (|t|^2 - c_i)/2 + B_j/2 - t.s_j > 0, ln q = ln h + ln 2
        float2 ct[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p)
          ct[p] = __fmul2_rn(__ffma2_rn(tz[p], tz[p], __ffma2_rn(ty[p], ty[p], __ffma2_rn(tx[p], tx[p], pr[p].nc))),
                             make_float2(0.5f, 0.5f));
        const float2 bias = shift_bias(-1, -1);
#pragma unroll 1
        for (int j0 = 0; j0 < G; j0 += FL) {
#pragma unroll 2
          for (int j = j0; j < j0 + FL; ++j) {
            const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c, re = gr[j].e;
            const float2 sr = lo2(rc), sa = hi2(rc);
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              float2 h = __fadd2_rn(ct[p], hi2(re));
              h = __ffma2_rn(tx[p], lo2(ra), h);
              h = __ffma2_rn(ty[p], hi2(ra), h);
              h = __ffma2_rn(tz[p], lo2(rb), h);
              const float2 lg = ln_q2_shift(h, bias, ln_tab);
              ar[p] = __ffma2_rn(sr, lg, ar[p]);
              aa[p] = __ffma2_rn(sa, lg, aa[p]);
            }
          }
          stream_flush<NP>(ar, aa, hr, lr, ha, la);
        }
      } else if (o.hi.w < 0.f) {
        // compact group near the warp: d = t_hi - s_hi (rel2_fast records: a self pair gives d = 0)
#pragma unroll 1
        for (int j0 = 0; j0 < G; j0 += FL) {
          for (int j = j0; j < j0 + FL; ++j) {
            const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c;
            const float2 nsx = lo2(ra), nsy = hi2(ra), nsz = lo2(rb), ncj = hi2(rb), sr = lo2(rc), sa = hi2(rc);
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              const float2 dx = __fadd2_rn(tx[p], nsx);
              const float2 dy = __fadd2_rn(ty[p], nsy);
              const float2 dz = __fadd2_rn(tz[p], nsz);
              const float2 u = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
              const float2 q = __fadd2_rn(u, __fadd2_rn(pr[p].nc, ncj));
              const float2 lg = ln_q2(stream_arg(u, q), ln_tab);
              ar[p] = __ffma2_rn(sr, lg, ar[p]);
              aa[p] = __ffma2_rn(sa, lg, aa[p]);
            }
          }
          stream_flush<NP>(ar, aa, hr, lr, ha, la);
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
#pragma unroll 1
        for (int j0 = 0; j0 < G; j0 += FL) {
          for (int j = j0; j < j0 + FL; ++j) {
            const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c, rd = gr[j].d, re = gr[j].e;
            const float2 nsx = lo2(ra), nsy = hi2(ra), nsz = lo2(rb), ncj = hi2(rb), sr = lo2(rc), sa = hi2(rc);
            const float2 nlx = lo2(rd), nly = hi2(rd), nlz = lo2(re);
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              const float2 dx = __fadd2_rn(__fadd2_rn(txh[p], nsx), __fadd2_rn(txl[p], nlx));
              const float2 dy = __fadd2_rn(__fadd2_rn(tyh[p], nsy), __fadd2_rn(tyl[p], nly));
              const float2 dz = __fadd2_rn(__fadd2_rn(tzh[p], nsz), __fadd2_rn(tzl[p], nlz));
              const float2 u = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
              const float2 q = __fadd2_rn(u, __fadd2_rn(pr[p].nc, ncj));
              const float2 lg = ln_q2(stream_arg(u, q), ln_tab);
              ar[p] = __ffma2_rn(sr, lg, ar[p]);
              aa[p] = __ffma2_rn(sa, lg, aa[p]);
            }
          }
          stream_flush<NP>(ar, aa, hr, lr, ha, la);
        }
      }
    }
  });

#pragma unroll
  for (int p = 0; p < NP; ++p) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t il = first + (2 * p + h) * THREADS + threadIdx.x;
      if (il < a.nt) {
        a.partial[(chunk * 2 + 0) * a.nt + il] =
            static_cast<double>(h ? hr[p].y : hr[p].x) + static_cast<double>(h ? lr[p].y : lr[p].x);
        a.partial[(chunk * 2 + 1) * a.nt + il] =
            static_cast<double>(h ? ha[p].y : ha[p].x) + static_cast<double>(h ? la[p].y : la[p].x);
      }
    }
  }
}

// Records and group origins of the sorted sources (one CTA of TILE threads per tile); a
// source that is also a target (ib <= j < ib + nt) leaves its zeta A in
// self_w[c * nt + j - ib] (zeroed before) for the finish to take out of the total.
template <int TILE>
__global__ void __launch_bounds__(TILE) stream_rel_prep_kernel(const double* x, const double* y, const double* z,
                                                               const double* qr, const double* qa, const double* area,
                                                               const int32_t* sorted, int64_t ns, double inv_a,
                                                               int64_t ib, int64_t nt, StreamRel::Rec* out,
                                                               BveRel::Origin* org, double* self_w,
                                                               double scale_r = -kInv4Pi, double scale_a = -kInv4Pi) {
  const int64_t t = blockIdx.x;
  const int64_t k = t * TILE + threadIdx.x;
  const bool valid = k < ns;
  const int32_t j = valid ? sorted[k] : 0;
  double px = 0.0, py = 0.0, pz = 0.0, cj = 0.0;
  if (valid) {
    px = x[j] * inv_a;
    py = y[j] * inv_a;
    pz = z[j] * inv_a;
    cj = fma(px, px, fma(py, py, fma(pz, pz, -1.0)));
  }
  const GroupFrame f = sphere_group_frame<TILE, BveRel::kGroup>(valid, px, py, pz, cj);
  StreamRel::Rec r;
  if (valid) {
    float hi[3], lo[3];
    group_offsets(f, px, py, pz, hi, lo);
    const float nc = __double2float_rn(-cj);
    const double wr = qr[j] * area[j], wa = qa[j] * area[j];
    const float sr = __double2float_rn(wr * scale_r), sa = __double2float_rn(wa * scale_a);
    r.a = make_float4(-hi[0], -hi[0], -hi[1], -hi[1]);
    r.b = make_float4(-hi[2], -hi[2], nc, nc);
    r.c = make_float4(sr, sr, sa, sa);
    r.d = make_float4(-lo[0], -lo[0], -lo[1], -lo[1]);
    const double h0 = hi[0], h1 = hi[1], h2 = hi[2];
    const float b = __double2float_rn(0.5 * fma(h0, h0, fma(h1, h1, fma(h2, h2, -cj))));
    r.e = make_float4(-lo[2], -lo[2], b, b);
    if (self_w && j >= ib && j < ib + nt) {
      self_w[j - ib] = wr;
      self_w[nt + j - ib] = wa;
    }
  } else {
    // inert: zero strength at the centroid (q = |t - o|^2 - c_i > 0 unless the target sits
    // on o, where d = 0 gives a zero term)
    r.a = r.b = r.c = r.d = r.e = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  out[k] = r;
  if (threadIdx.x % BveRel::kGroup == 0) {
    BveRel::Origin o = group_origin(f);
    o.hi.w = f.compact ? -f.radius : f.radius;  // the sign marks a compact group
    org[t * (TILE / BveRel::kGroup) + threadIdx.x / BveRel::kGroup] = o;
  }
}

// ====================================================================== planar stream function
// SetStreamFunctionOnMesh, src/PlanarIncompressible.f90:470-505: psi_i = sum_{j != i}
// ln(|x_i - x_j|^2) omega_j A_j / (4 pi), on the planar group-relative layout (plane_rel.cuh;
// plane_rel_prep_kernel writes S_j = omega_j A_j / (4 pi) and each group's total S_g).
//
// The terms are centred per target and group: with a power of two 2^k near
// max(|t - o|^2, R^2) (k from the exponent split of ln_q2),
//   sum_j S_j ln u_j = sum_j S_j (ln u_j - k ln 2) + k ln 2 S_g,
// so the FP32 partials hold terms of size |S_j| (|ln(u_j 2^-k)| <= ~1.2 for a far group)
// instead of |S_j ln u_j|, and the second part is carried exactly: S_g k as a product of
// a (hi, lo) float pair and a small integer into its own compensated pair, times ln 2 in
// FP64 at the end.  ln_q2_shift applies the shift for free.  A far group (every target of the
// warp at |t - o| > 3R, so u_j > 0) needs no select; in a near group the self pair (u = 0,
// the lo parts cancel bit for bit) takes q = 1, whose centred term -k ln 2 cancels the
// target's own share of k ln 2 S_g.  Per target pair and source (far form): d (2 FADD2),
// |d|^2 (2), ln (ln_q2_shift: integer split, a table load per lane, 9 packed) and the
// accumulation (1 FFMA2).  Near partials are flushed every 16 sources, far ones per group.
template <int THREADS, int TPT, int TILE, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) plane_stream_rel_sweep_kernel(PlaneRelArgs a) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  constexpr int NP = TPT / 2;
  constexpr int G = PlaneRel::kGroup;
  constexpr int GPT = TILE / G;
  constexpr int FLN = 16;
  static_assert(G % FLN == 0, "flush interval must divide the group");
  using Rec = PlaneRel::Rec;
  __shared__ __align__(128) Rec stage[2][TILE];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ __align__(8) float2 ln_tab[32];

  const int64_t chunk = blockIdx.y;
  const int64_t tile0 = chunk * a.tiles_per_chunk;
  int64_t ntl = a.n_tiles - tile0;
  if (ntl > a.tiles_per_chunk) ntl = a.tiles_per_chunk;
  if (ntl < 0) ntl = 0;

  PlaneRel::Pair pr[NP];
  float2 hs[NP], ls[NP], hk[NP], lk[NP];
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
    hs[p] = ls[p] = hk[p] = lk[p] = make_float2(0.f, 0.f);
  }
  constexpr float kTiny = 7.888609052210118e-31f;  // 2^-100: centring and near floor
  constexpr float kHuge = 1.2676506002282294e30f;  // 2^100

  ln_tab_load(ln_tab);
  pipe_init(bars);
  uint32_t g = 0;
  int64_t tile = tile0;
  staged_sweep<Rec, TILE>(a.src, tile0, ntl, stage[0], stage[1], bars, g, a.status, [&](const Rec* tl) {
    const PlaneRel::Origin* og = a.org + tile * GPT;
#pragma unroll 1
    for (int g0 = 0; g0 < TILE; g0 += G) {
      const PlaneRel::Origin o = og[g0 / G];
      const Rec* gr = tl + g0;
      float2 tx[NP], ty[NP];
      float2 bias[NP];
      bool near = false;
      const float r2 = o.f.x * o.f.x;
      const float lim = fmaxf(PlaneRel::kNearFactor * PlaneRel::kNearFactor * r2, kTiny);
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        tx[p] = rel1x2(pr[p].xh, pr[p].xl, o.o.x, o.o.z);
        ty[p] = rel1x2(pr[p].yh, pr[p].yl, o.o.y, o.o.w);
        const float2 n2 = __ffma2_rn(ty[p], ty[p], __fmul2_rn(tx[p], tx[p]));
        near |= !(n2.x > lim) | !(n2.y > lim);
        // the centring shift k: the exponent of max(|t - o|^2, R^2) clamped to [2^-100, 2^100]
        const float c0 = fminf(fmaxf(fmaxf(n2.x, r2), kTiny), kHuge);
        const float c1 = fminf(fmaxf(fmaxf(n2.y, r2), kTiny), kHuge);
        int mb;
        const int sh0 = exp_split(__float_as_int(c0), mb);
        const int sh1 = exp_split(__float_as_int(c1), mb);
        bias[p] = shift_bias(sh0, sh1);
        // k S_g into (hk, lk): S_hi k is exact as a product and its error term
        const float2 kf = make_float2(static_cast<float>(sh0), static_cast<float>(sh1));
        const float2 ph = __fmul2_rn(make_float2(o.f.y, o.f.y), kf);
        const float2 pe = __ffma2_rn(make_float2(o.f.y, o.f.y), kf, make_float2(-ph.x, -ph.y));
        comp_add(hk[p].x, lk[p].x, ph.x);
        comp_add(hk[p].y, lk[p].y, ph.y);
        lk[p] = __ffma2_rn(make_float2(o.f.z, o.f.z), kf, __fadd2_rn(lk[p], pe));
      }
      if (!__any_sync(0xffffffffu, near)) {
        // far group: d = t_hi - s_hi, u > 0
        float2 acc[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) acc[p] = make_float2(0.f, 0.f);
#pragma unroll 4
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(tx[p], lo2(ra));
            const float2 dy = __fadd2_rn(ty[p], hi2(ra));
            const float2 u = __ffma2_rn(dy, dy, __fmul2_rn(dx, dx));
            acc[p] = __ffma2_rn(lo2(rb), ln_q2_shift(u, bias[p], ln_tab), acc[p]);
          }
        }
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          comp_add(hs[p].x, ls[p].x, acc[p].x);
          comp_add(hs[p].y, ls[p].y, acc[p].y);
        }
      } else {
        // near group: d = (t_hi - s_hi) + (t_lo - s_lo)
        float2 txh[NP], tyh[NP], txl[NP], tyl[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          rel2x2(pr[p].xh, pr[p].xl, o.o.x, o.o.z, txh[p], txl[p]);
          rel2x2(pr[p].yh, pr[p].yl, o.o.y, o.o.w, tyh[p], tyl[p]);
        }
#pragma unroll 1
        for (int j0 = 0; j0 < G; j0 += FLN) {
          float2 acc[NP];
#pragma unroll
          for (int p = 0; p < NP; ++p) acc[p] = make_float2(0.f, 0.f);
          for (int j = j0; j < j0 + FLN; ++j) {
            const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c;
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              const float2 dx = __fadd2_rn(__fadd2_rn(txh[p], lo2(ra)), __fadd2_rn(txl[p], hi2(rb)));
              const float2 dy = __fadd2_rn(__fadd2_rn(tyh[p], hi2(ra)), __fadd2_rn(tyl[p], lo2(rc)));
              const float2 u = __ffma2_rn(dy, dy, __fmul2_rn(dx, dx));
              acc[p] = __ffma2_rn(lo2(rb), ln_q2_shift(stream_arg(u, u), bias[p], ln_tab), acc[p]);
            }
          }
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            comp_add(hs[p].x, ls[p].x, acc[p].x);
            comp_add(hs[p].y, ls[p].y, acc[p].y);
          }
        }
      }
    }
    ++tile;
  });

  constexpr double kLn2 = 0.69314718055994530942;
#pragma unroll
  for (int p = 0; p < NP; ++p) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t il = first + (2 * p + h) * THREADS + threadIdx.x;
      if (il < a.nt) {
        const double c = static_cast<double>(h ? hk[p].y : hk[p].x) + static_cast<double>(h ? lk[p].y : lk[p].x);
        a.partial[chunk * a.nt + il] =
            (static_cast<double>(h ? hs[p].y : hs[p].x) + static_cast<double>(h ? ls[p].y : ls[p].x)) + kLn2 * c;
      }
    }
  }
}

// ====================================================================== sphere SWE velocity
// SWESphereRHSIntegrals, src/SphereSWESolver.f90:299-372, velocity part, on the stream
// functions' layout (two strengths per record: S_r = -zeta_j A_j / (2 pi a^2) and
// S_p = div_j A_j / (2 pi a^2), written by stream_rel_prep_kernel).  With p = x/a, d = p_i - p_j
// and a^2 - x_i.x_j = (a^2/2) q, q = |d|^2 - c_i - c_j, the reference's
//   u -= (x_i x x_j) zeta_j A_j / (4 pi a^2 (a^2 - x_i.x_j)) + x_j a div_j A_j / (4 pi a^2 (a^2 - x_i.x_j))
// is u = Dr x p_i + Dp - p_i W with Dr = sum (S_r/q) d, Dp = sum (S_p/q) d, W = sum S_p/q
// (x_i x x_j = a^2 d x p_i and p_j = p_i - d).  The self pair (d = 0 exactly, in a near or a
// compact group) gets 1/q = 0.  Per target pair and source (far form): d (3 FADD2), |d|^2
// (3), q (1), the select and 2 MUFU, two weights (2), 7 accumulations.  Partials:
// [chunk][7][nt] (Dr, Dp, W).
template <int THREADS, int TPT, int TILE, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) sphere_swe_rel_sweep_kernel(SweepArgs<BveF32> a,
                                                                             const StreamRel::Rec* __restrict__ src,
                                                                             const BveRel::Origin* __restrict__ org) {
  static_assert(TPT % 2 == 0, "targets come in pairs");
  constexpr int NP = TPT / 2;
  constexpr int G = BveRel::kGroup;
  constexpr int GPT = TILE / G;
  constexpr int NC = 7;
  using Rec = StreamRel::Rec;
  __shared__ __align__(128) Rec stage[2][TILE];
  __shared__ __align__(8) uint64_t bars[2];

  const int64_t chunk = blockIdx.y;
  const int64_t tile0 = chunk * a.tiles_per_chunk;
  int64_t ntl = a.n_tiles - tile0;
  if (ntl > a.tiles_per_chunk) ntl = a.tiles_per_chunk;
  if (ntl < 0) ntl = 0;

  BveX2::Pair pr[NP];
  float2 hs[NP][NC], ls[NP][NC];
  const int64_t first = static_cast<int64_t>(blockIdx.x) * (THREADS * TPT);
  const int64_t count = a.nt - first < THREADS * TPT ? a.nt - first : THREADS * TPT;
  bve_load_pairs<NP>(a.p, a.ib + first, count, THREADS, pr);
#pragma unroll
  for (int p = 0; p < NP; ++p)
#pragma unroll
    for (int c = 0; c < NC; ++c) hs[p][c] = ls[p][c] = make_float2(0.f, 0.f);

  pipe_init(bars);
  uint32_t g = 0;
  int64_t tile = tile0;
  staged_sweep<Rec, TILE>(src, tile0, ntl, stage[0], stage[1], bars, g, a.status, [&](const Rec* tl) {
    float2 ac[NP][NC];
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
      for (int c = 0; c < NC; ++c) ac[p][c] = make_float2(0.f, 0.f);
    auto terms = [&](float2 (&acc)[NC], float2 dx, float2 dy, float2 dz, float2 q, float2 u, float2 sr, float2 sp) {
      const float2 inv = make_float2(u.x != 0.f ? rcp_approx(q.x) : 0.f, u.y != 0.f ? rcp_approx(q.y) : 0.f);
      const float2 wr = __fmul2_rn(sr, inv), wp = __fmul2_rn(sp, inv);
      acc[0] = __ffma2_rn(wr, dx, acc[0]);
      acc[1] = __ffma2_rn(wr, dy, acc[1]);
      acc[2] = __ffma2_rn(wr, dz, acc[2]);
      acc[3] = __ffma2_rn(wp, dx, acc[3]);
      acc[4] = __ffma2_rn(wp, dy, acc[4]);
      acc[5] = __ffma2_rn(wp, dz, acc[5]);
      acc[6] = __fadd2_rn(wp, acc[6]);
    };
    const BveRel::Origin* og = org + tile * GPT;
#pragma unroll 1
    for (int g0 = 0; g0 < TILE; g0 += G) {
      const BveRel::Origin o = og[g0 / G];
      const Rec* gr = tl + g0;
      float2 tx[NP], ty[NP], tz[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        tx[p] = rel1x2(pr[p].xh, pr[p].xl, o.hi.x, o.lo.x);
        ty[p] = rel1x2(pr[p].yh, pr[p].yl, o.hi.y, o.lo.y);
        tz[p] = rel1x2(pr[p].zh, pr[p].zl, o.hi.z, o.lo.z);
      }
      if (o.hi.w <= 0.f || !warp_near<NP>(tx, ty, tz, o.hi.w)) {  // -R: compact, taken as far
        // compact or far group: d = t_hi - s_hi
#pragma unroll 2
        for (int j = 0; j < G; ++j) {
          const float4 ra = gr[j].a, rb = gr[j].b, rc = gr[j].c;
          const float2 nsx = lo2(ra), nsy = hi2(ra), nsz = lo2(rb), ncj = hi2(rb), sr = lo2(rc), sp = hi2(rc);
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(tx[p], nsx);
            const float2 dy = __fadd2_rn(ty[p], nsy);
            const float2 dz = __fadd2_rn(tz[p], nsz);
            const float2 u = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
            terms(ac[p], dx, dy, dz, __fadd2_rn(u, __fadd2_rn(pr[p].nc, ncj)), u, sr, sp);
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
          const float2 nsx = lo2(ra), nsy = hi2(ra), nsz = lo2(rb), ncj = hi2(rb), sr = lo2(rc), sp = hi2(rc);
          const float2 nlx = lo2(rd), nly = hi2(rd), nlz = lo2(re);
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 dx = __fadd2_rn(__fadd2_rn(txh[p], nsx), __fadd2_rn(txl[p], nlx));
            const float2 dy = __fadd2_rn(__fadd2_rn(tyh[p], nsy), __fadd2_rn(tyl[p], nly));
            const float2 dz = __fadd2_rn(__fadd2_rn(tzh[p], nsz), __fadd2_rn(tzl[p], nlz));
            const float2 u = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
            terms(ac[p], dx, dy, dz, __fadd2_rn(u, __fadd2_rn(pr[p].nc, ncj)), u, sr, sp);
          }
        }
      }
    }
    ++tile;
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        comp_add(hs[p][c].x, ls[p][c].x, ac[p][c].x);
        comp_add(hs[p][c].y, ls[p][c].y, ac[p][c].y);
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

// ====================================================================== beta-plane stream functions
// The beta plane's SetStreamFunctionsOnMesh, src/BetaPlane.f90:399-442, in FP32 for two
// targets at a time (the direct form of beta_stream_rel_sweep_kernel, csrc/beta_rel.cuh):
//   G = log(cosh(2 pi dy) - cos(2 pi dx)) / (4 pi),  psi += G zeta_j A_j  (j != i).
// cosh 2a - cos 2b = 2 (sinh^2 a + sin^2 b) = 2 4^(k-1) (sh'^2 + sn'^2) with a = pi |dy| =
// k ln 2 + r, b = pi dx and the 2^(k-1)-scaled sh', sn' of BetaF32, so
//   4 pi G = (2k - 1) ln 2 + ln(sh'^2 + sn'^2),
// no cancellation for close pairs and no overflow for far ones; the (2k - 1) ln 2 rides on the
// exponent of ln_q2_shift.  S = zeta A / (4 pi); the self pair (sh' = sn' = 0) is a zero term.
// Terms of both signs cancel to psi, so the caller flushes the FP32 partials often.
struct BetaStreamF32 {
  struct __align__(16) Rec {
    float4 a;  // x_hi, y_hi, x_lo, y_lo
    float4 b;  // S_rel, S_abs, 0, 0
  };
  using Tgt = BetaTgt;
  __device__ static __forceinline__ void interact2(const Tgt& t0, const Tgt& t1, const Rec& r, float (&a0)[2],
                                                   float (&a1)[2], const float2* tab) {
    float2 tt, dy;
    beta_deltas2(t0, t1, r.a, tt, dy);
    const float2 sn = sinpi2(tt, __fmul2_rn(tt, tt));
    const float2 a = __fmul2_rn(make_float2(3.1415927f, 3.1415927f), bits_abs(dy));
    float2 shr, chr, kb;
    sinh_cosh_reduced2(a, shr, chr, kb);
    const int k0 = static_cast<int>(__float_as_uint(kb.x) - 0x4b400000u);
    const int k1 = static_cast<int>(__float_as_uint(kb.y) - 0x4b400000u);
    const unsigned c0 = static_cast<unsigned>(k0 < 126 ? k0 : 126), c1 = static_cast<unsigned>(k1 < 126 ? k1 : 126);
    const float2 pk = make_float2(__uint_as_float(0x3f800000u - (c0 << 23)), __uint_as_float(0x3f800000u - (c1 << 23)));
    const float2 sc = __fadd2_rn(pk, pk);
    const float2 q = __fmul2_rn(pk, pk);
    const float2 shp = __ffma2_rn(__fadd2_rn(make_float2(1.0f, 1.0f), make_float2(-q.x, -q.y)), chr,
                                  __fmul2_rn(__fadd2_rn(make_float2(1.0f, 1.0f), q), shr));
    const float2 snp = __fmul2_rn(sn, sc);
    const float2 x = __ffma2_rn(shp, shp, __fmul2_rn(snp, snp));
    const float2 lg = ln_q2_shift(make_float2(x.x > 0.f ? x.x : 1.0f, x.y > 0.f ? x.y : 1.0f),
                                  shift_bias(1 - 2 * k0, 1 - 2 * k1), tab);
    const float2 g = make_float2(x.x > 0.f ? lg.x : 0.f, x.y > 0.f ? lg.y : 0.f);
    const float2 pr = __ffma2_rn(make_float2(r.b.x, r.b.x), g, make_float2(a0[0], a1[0]));
    const float2 pa = __ffma2_rn(make_float2(r.b.y, r.b.y), g, make_float2(a0[1], a1[1]));
    a0[0] = pr.x;
    a1[0] = pr.y;
    a0[1] = pa.x;
    a1[1] = pa.y;
  }
};

}  // namespace lpm
