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
// a fixed-order FP64 total minus the target's own term.  Per target pair and source (far
// form): d (3 FADD2), |d|^2 (3), q (1-2), the self-pair select and the clamp to >= 2^-126
// (scalar), ln q (ln_q2: 4 integer operations per lane, 15 packed, 2 MUFU), and the two
// accumulations (2 FFMA2).  The FP32 partials are flushed into compensated (hi, lo) pairs
// every 32 sources, because the terms cancel to a much smaller psi.
#pragma once

#include "bve_rel.cuh"
#include "ops.cuh"

namespace lpm {

struct StreamRel {
  struct __align__(16) Rec {
    float4 a;  // -sx_hi, -sx_hi, -sy_hi, -sy_hi
    float4 b;  // -sz_hi, -sz_hi, -c_j, -c_j
    float4 c;  // S_rel, S_rel, S_abs, S_abs
    float4 d;  // -sx_lo, -sx_lo, -sy_lo, -sy_lo
    float4 e;  // -sz_lo, -sz_lo, 0, 0
  };
  static constexpr int kFlush = 32;
};

// ln_q of two lanes at once: the integer exponent split per lane, the rest packed.  The
// argument is a positive normal float (the sweep clamps it).
__device__ __forceinline__ float2 ln_q2(float2 q) {
  const int b0 = __float_as_int(q.x), b1 = __float_as_int(q.y);
  const int k0 = (b0 - 0x3f3504f3) >> 23, k1 = (b1 - 0x3f3504f3) >> 23;
  const float2 m = make_float2(__int_as_float(b0 - (k0 << 23)), __int_as_float(b1 - (k1 << 23)));
  const float2 kf = __fadd2_rn(make_float2(__int_as_float(k0 + 0x4b400000), __int_as_float(k1 + 0x4b400000)),
                               make_float2(-12582912.0f, -12582912.0f));
  const float2 f = __fadd2_rn(m, make_float2(-1.0f, -1.0f));
  const float2 den = __fadd2_rn(f, make_float2(2.0f, 2.0f));
  const float2 r = make_float2(rcp_approx(den.x), rcp_approx(den.y));
  const float2 t0 = __fmul2_rn(f, r);
  const float2 res = __ffma2_rn(make_float2(-t0.x, -t0.y), f, __ffma2_rn(make_float2(-2.0f, -2.0f), t0, f));
  const float2 t = __ffma2_rn(r, res, t0);
  const float2 tt = __fadd2_rn(t, t);
  const float2 s = __fmul2_rn(t, t);
  float2 p = __ffma2_rn(make_float2(0.11111111f, 0.11111111f), s, make_float2(0.14285715f, 0.14285715f));
  p = __ffma2_rn(p, s, make_float2(0.2f, 0.2f));
  p = __ffma2_rn(p, s, make_float2(0.33333334f, 0.33333334f));
  const float2 lnm = __ffma2_rn(__fmul2_rn(tt, s), p, tt);
  return __ffma2_rn(kf, make_float2(0.69314718f, 0.69314718f), lnm);
}

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
  __shared__ __align__(128) Rec stage[2][TILE];
  __shared__ __align__(8) uint64_t bars[2];

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

  pipe_init(bars);
  uint32_t g = 0;
  int64_t tile = tile0;
  staged_sweep<Rec, TILE>(src, tile0, ntl, stage[0], stage[1], bars, g, a.status, [&](const Rec* tl) {
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
      if (o.hi.w == 0.f || !warp_near<NP>(tx, ty, tz, o.hi.w)) {  // R = 0: compact, never near
        // compact or far group: d = t_hi - s_hi
#pragma unroll 1
        for (int j0 = 0; j0 < G; j0 += FL) {
#pragma unroll 2
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
              const float2 lg = ln_q2(stream_arg(u, q));
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
              const float2 lg = ln_q2(stream_arg(u, q));
              ar[p] = __ffma2_rn(sr, lg, ar[p]);
              aa[p] = __ffma2_rn(sa, lg, aa[p]);
            }
          }
          stream_flush<NP>(ar, aa, hr, lr, ha, la);
        }
      }
    }
    ++tile;
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
                                                               BveRel::Origin* org, double* self_w) {
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
  const GroupFrame f = sphere_group_frame<TILE>(valid, px, py, pz, cj);
  StreamRel::Rec r;
  if (valid) {
    float hi[3], lo[3];
    group_offsets(f, px, py, pz, hi, lo);
    const float nc = __double2float_rn(-cj);
    const double wr = qr[j] * area[j], wa = qa[j] * area[j];
    const float sr = __double2float_rn(wr * -kInv4Pi), sa = __double2float_rn(wa * -kInv4Pi);
    r.a = make_float4(-hi[0], -hi[0], -hi[1], -hi[1]);
    r.b = make_float4(-hi[2], -hi[2], nc, nc);
    r.c = make_float4(sr, sr, sa, sa);
    r.d = make_float4(-lo[0], -lo[0], -lo[1], -lo[1]);
    r.e = make_float4(-lo[2], -lo[2], 0.f, 0.f);
    if (j >= ib && j < ib + nt) {
      self_w[j - ib] = wr;
      self_w[nt + j - ib] = wa;
    }
  } else {
    // inert: zero strength at the centroid (q = |t - o|^2 - c_i > 0 unless the target sits
    // on o, where d = 0 gives a zero term)
    r.a = r.b = r.c = r.d = r.e = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  out[k] = r;
  if (threadIdx.x % BveRel::kGroup == 0) org[t * (TILE / BveRel::kGroup) + threadIdx.x / BveRel::kGroup] = group_origin(f);
}

}  // namespace lpm
