// sums.cu -- direct-sum kernels (prep, sweep, finish), their launchers and the host-buffer
// C-ABI entry points lpm_bve_velocity, lpm_plane_velocity, lpm_pse_*_laplacian and the
// stream functions.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "bve_rel.cuh"
#include "beta_rel.cuh"
#include "bve_x2.cuh"
#include "engine.cuh"
#include "ops.cuh"
#include "plane_rel.cuh"
#include "pse_rel.cuh"
#include "sort.cuh"
#include "stream_rel.cuh"
#include "sums.cuh"

namespace lpm {

namespace {

constexpr double kPi = 3.1415926535897932384626433832795027975;

// FP32C sweep shapes (threads per CTA, targets per thread, tile, min CTAs per SM)
constexpr int kBveTile = 256;
// Shapes of the sphere-BVE FP32C sweep the autotuner chooses from: threads per CTA,
// targets per thread (in pairs), CTAs per SM.  All fit without register spills.
struct BveShape {
  int threads, tpt, minb;
};
constexpr BveShape kBveShapes[] = {{128, 4, 4}, {256, 4, 2}, {128, 6, 2}, {128, 8, 2}};
constexpr int kBveShapeCount = sizeof(kBveShapes) / sizeof(kBveShapes[0]);
constexpr int kPlaneThreads = 128, kPlaneTpt = 4, kPlaneTile = 256, kPlaneMinB = 4;
// PSE sweeps (warp-decoupled pipeline): 256-source tiles in two stages; the divergence, whose
// sweep holds more per-target state (128 registers), runs faster on 128-source tiles in four
constexpr int kPseThreads = 128, kPseTpt = 4, kPseTile = 256, kPseMinB = 4, kPseStages = 2;
constexpr int kPseDivTile = 128, kPseDivStages = 4;
constexpr int kStreamThreads = 128, kStreamTpt = 4, kStreamTile = 256, kStreamMinB = 4;
constexpr int kBetaThreads = 128, kBetaTpt = 4, kBetaTile = 256, kBetaMinB = 4;
constexpr int kSweMinB = 3;        // planar SWE velocity sweep: 128 x 4 targets, 3 CTAs per SM
constexpr int kSweSphereMinB = 2;  // sphere SWE velocity sweep: 2 CTAs per SM (no spills; 10 % over 3)
// FP64 sequential sweep shape
// 64-source tiles: the PSE sums' tile cutoff skips 14-25 % more work than with 128 and the
// sweeps without a cutoff run at the same rate
constexpr int k64Threads = 128, k64Tile = 64;
constexpr int kSplit64 = 4;  // lanes per target of the split FP64 sweep (small target sets; 8 was slower)

// ------------------------------------------------------------------ FP64 sequential sweep
// One thread per target, sources in ascending particle order, one accumulator: the same
// summation order as the Fortran j loop, hence bit-identical sums.
//
// The PSE kernels all carry exp(-r^2), r = distance / eps: at r >= 7 each kernel (its
// polynomial times e^-49) is below 1e-14 of its peak, far below the FP64 sums' 1e-12
// agreement with the reference (whose exp is not CUDA's anyway; the all-pairs oracle tests
// hold that bound with the cutoff).  For those a warp skips a whole source tile when every
// one of its targets is farther than the tile's radius plus `reach` from the tile's centre,
// in the space the distance is measured in:
//   - unit directions for the great-circle kernels (reach 7 eps / radius; the angle is never
//     shorter than the chord of the unit directions);
//   - raw positions for the chord and planar ones (reach 7 eps).
// The pairs it keeps are summed in the reference's order.  The FP32C sweeps cut at the same
// r^2 = 49 (PseRel::kCutR2).
struct __align__(32) TileBall {
  double x, y, z, r;  // centre and radius in the test space
};

struct Fp64Cut {
  const TileBall* bounds = nullptr;  // per source tile
  const double *x = nullptr, *y = nullptr, *z = nullptr;  // target positions (z may be null)
  double reach = 0.0;
  int unit = 0;  // 1: the test space is unit directions
  // the targets in curve order (nt global indices), or nullptr for index order: a warp then
  // holds 32 targets close together and skips more tiles; each target's own sum is unchanged
  const int32_t* tperm = nullptr;
};

// The point of particle i in the test space.  A point at the origin has no direction (and
// atan2(0, 0) puts it at distance 0 from everything): it becomes NaN, which the tests below
// read as "in reach", so nothing is skipped for it.
__device__ __forceinline__ double3 cut_point(const double* x, const double* y, const double* z, int64_t i,
                                             int unit) {
  double3 q = make_double3(x[i], y[i], z ? z[i] : 0.0);
  if (unit) {
    const double nq = sqrt(q.x * q.x + q.y * q.y + q.z * q.z);
    const double inv = nq > 0.0 ? 1.0 / nq : __longlong_as_double(0x7ff8000000000000LL);
    q = make_double3(q.x * inv, q.y * inv, q.z * inv);
  }
  return q;
}

template <class Op, class Rec, class P>
__global__ void __launch_bounds__(k64Threads) seq_fp64_kernel(P p, const Rec* __restrict__ src,
                                                              int64_t ns, int64_t ib, int64_t nt,
                                                              int* status, Fp64Cut cut = Fp64Cut{}) {
  __shared__ __align__(128) Rec stage[2][k64Tile];
  __shared__ __align__(8) uint64_t bars[2];
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const bool valid = k < nt;
  const int64_t i = cut.tperm ? static_cast<int64_t>(cut.tperm[valid ? k : nt - 1]) : ib + (valid ? k : nt - 1);
  const int64_t il = i - ib;  // the target's place in the outputs
  const typename Op::Tgt t = Op::load(p, i);
  typename Op::Acc acc{};
  const int64_t n_tiles = ceil_div(ns, k64Tile);
  const double3 tp = cut.bounds ? cut_point(cut.x, cut.y, cut.z, i, cut.unit) : make_double3(0.0, 0.0, 0.0);
  int64_t tile = 0;
  pipe_init(bars);
  uint32_t g = 0;
  staged_sweep<Rec, k64Tile>(src, 0, n_tiles, stage[0], stage[1], bars, g, status,
                             [&](const Rec* tl) {
                               bool run = true;
                               if (cut.bounds) {
                                 const TileBall b = cut.bounds[tile];
                                 const double dx = tp.x - b.x, dy = tp.y - b.y, dz = tp.z - b.z;
                                 const double lim = b.r + cut.reach;
                                 run = __any_sync(0xffffffffu, !(dx * dx + dy * dy + dz * dz > lim * lim));
                               }
                               if (run) {
                                 const int64_t j0 = tile * k64Tile;
                                 const int cnt = static_cast<int>(ns - j0 < k64Tile ? ns - j0 : k64Tile);
                                 for (int j = 0; j < cnt; ++j) {
                                   const Rec& r = tl[j];
                                   if (Op::kSkipSelf && r.idx == i) continue;
                                   Op::interact(p, t, r, acc);
                                 }
                               }
                               ++tile;
                             });
  if (valid) Op::store(p, i, il, acc);
}

// The FP64 sweep for a small target set, S lanes per target.  Lane k of a target's group
// evaluates sources j = j0 + k of each run of S, on an accumulator of zero, so it holds the
// term itself (0 + X = X).  The S terms of a run are then added in ascending j, with the same
// rounding as the sequential sweep, each accumulator component by one lane of the group:
// lane k keeps components k, k + S, ...  (one FP64 add per lane and term instead of one per
// component: on GB300's 2 FP64 lanes per clock per SM the adds of all components in every
// lane cost a quarter of the pipe at S = 4 and three components).  The group's first lane
// collects the components at the end.  This is for operators whose interact adds exactly one
// term to each accumulator component (a = a + X, or a = a - X, which is a + (-X)), so the
// sums stay bit-identical up to the sign of an exact zero.  S times as many warps share the
// FP64 work.
template <class Op, class Rec, class P, int S, int THREADS>
__global__ void __launch_bounds__(THREADS) seq_fp64_split_kernel(P p, const Rec* __restrict__ src,
                                                                 int64_t ns, int64_t ib, int64_t nt,
                                                                 int* status) {
  static_assert(32 % S == 0, "a target's lanes stay in one warp");
  using Acc = typename Op::Acc;
  static_assert(sizeof(Acc) % sizeof(double) == 0, "accumulators are doubles");
  constexpr int NA = static_cast<int>(sizeof(Acc) / sizeof(double));
  constexpr int NSLOT = (NA + S - 1) / S;  // components per lane
  __shared__ __align__(128) Rec stage[2][k64Tile];
  __shared__ __align__(8) uint64_t bars[2];
  const int k = static_cast<int>(threadIdx.x) % S;
  const int lane0 = static_cast<int>(threadIdx.x & 31u) - k;  // the group's first lane in the warp
  const int64_t il = static_cast<int64_t>(blockIdx.x) * (THREADS / S) + threadIdx.x / S;
  const bool valid = il < nt;
  const int64_t i = ib + (valid ? il : nt - 1);
  const typename Op::Tgt t = Op::load(p, i);
  double slot[NSLOT];  // slot m: component k + m S of the target's sum
#pragma unroll
  for (int m = 0; m < NSLOT; ++m) slot[m] = 0.0;
  const int64_t n_tiles = ceil_div(ns, k64Tile);
  int64_t tile = 0;
  pipe_init(bars);
  uint32_t g = 0;
  staged_sweep<Rec, k64Tile>(src, 0, n_tiles, stage[0], stage[1], bars, g, status, [&](const Rec* tl) {
    const int64_t j0 = tile * k64Tile;
    const int cnt = static_cast<int>(ns - j0 < k64Tile ? ns - j0 : k64Tile);
    for (int jb = 0; jb < cnt; jb += S) {
      const int j = jb + k;
      Acc d{};
      const bool has = j < cnt && !(Op::kSkipSelf && tl[j < cnt ? j : 0].idx == i);
      if (has) Op::interact(p, t, tl[j], d);
      const double* dv = reinterpret_cast<const double*>(&d);
#pragma unroll
      for (int q = 0; q < S; ++q) {
        const bool hq = __shfl_sync(0xffffffffu, has, lane0 + q);
        double x[NA];
#pragma unroll
        for (int c = 0; c < NA; ++c) x[c] = __shfl_sync(0xffffffffu, dv[c], lane0 + q);
#pragma unroll
        for (int m = 0; m < NSLOT; ++m) {
          const int c = k + m * S;
          double xc = x[0];
#pragma unroll
          for (int cc = 1; cc < NA; ++cc) xc = c == cc ? x[cc] : xc;
          if (hq && c < NA) slot[m] = __dadd_rn(slot[m], xc);
        }
      }
    }
    ++tile;
  });
  Acc acc{};
  double* av = reinterpret_cast<double*>(&acc);
#pragma unroll
  for (int c = 0; c < NA; ++c) av[c] = __shfl_sync(0xffffffffu, slot[c / S], lane0 + c % S);
  if (valid && k == 0) Op::store(p, i, il, acc);
}

// The split sweep at a CTA size of 128, 64 or 32 threads.
template <class Op, class Rec, class P>
void launch_split64(int threads, unsigned grid, cudaStream_t stream, const P& p, const Rec* src, int64_t ns,
                    int64_t ib, int64_t nt, int* status) {
  if (threads == 32) {
    seq_fp64_split_kernel<Op, Rec, P, kSplit64, 32><<<grid, 32, 0, stream>>>(p, src, ns, ib, nt, status);
  } else if (threads == 64) {
    seq_fp64_split_kernel<Op, Rec, P, kSplit64, 64><<<grid, 64, 0, stream>>>(p, src, ns, ib, nt, status);
  } else {
    seq_fp64_split_kernel<Op, Rec, P, kSplit64, k64Threads><<<grid, k64Threads, 0, stream>>>(p, src, ns, ib, nt,
                                                                                             status);
  }
}

// The bounding ball (centre, radius) of each FP64 source tile (k64Tile consecutive active
// sources) in the cutoff's test space; one CTA of k64Tile threads per tile.  The radius is
// widened by 1e-9 of itself and of the centre's size, which covers the rounding of the test.
__global__ void __launch_bounds__(k64Tile) tile_bounds64_kernel(const double* x, const double* y, const double* z,
                                                                const int32_t* idx, int64_t ns, int unit,
                                                                TileBall* bounds) {
  __shared__ double red[4][k64Tile];
  const int tid = threadIdx.x;
  const int64_t k = static_cast<int64_t>(blockIdx.x) * k64Tile + tid;
  const bool valid = k < ns;
  const double3 q = valid ? cut_point(x, y, z, idx[k], unit) : make_double3(0.0, 0.0, 0.0);
  // a source without a direction (NaN point) leaves the centre alone and makes the radius
  // infinite: the tile is in reach of every target
  const bool dirless = valid && !(q.x == q.x && q.y == q.y && q.z == q.z);
  red[0][tid] = dirless ? 0.0 : q.x;
  red[1][tid] = dirless ? 0.0 : q.y;
  red[2][tid] = dirless ? 0.0 : q.z;
  red[3][tid] = valid && !dirless ? 1.0 : 0.0;
  __syncthreads();
  for (int w = k64Tile / 2; w > 0; w >>= 1) {
    if (tid < w) {
#pragma unroll
      for (int c = 0; c < 4; ++c) red[c][tid] += red[c][tid + w];
    }
    __syncthreads();
  }
  const double cnt = red[3][0] > 0.0 ? red[3][0] : 1.0;
  const double cx = red[0][0] / cnt, cy = red[1][0] / cnt, cz = red[2][0] / cnt;
  __syncthreads();
  red[0][tid] = dirless ? __longlong_as_double(0x7ff0000000000000LL)
                : valid ? sqrt((q.x - cx) * (q.x - cx) + (q.y - cy) * (q.y - cy) + (q.z - cz) * (q.z - cz))
                        : 0.0;
  __syncthreads();
  for (int w = k64Tile / 2; w > 0; w >>= 1) {
    if (tid < w) red[0][tid] = fmax(red[0][tid], red[0][tid + w]);
    __syncthreads();
  }
  if (tid == 0) {
    const double sz = fabs(cx) + fabs(cy) + fabs(cz);
    bounds[blockIdx.x] = TileBall{cx, cy, cz, red[0][0] * (1.0 + 1e-9) + 1e-9 * sz};
  }
}

// ------------------------------------------------------------------ prep kernels
// Gather the active particles (src_idx) into source records; records ns..npad-1 are inert.

__global__ void prep_rec64_kernel(const double* x, const double* y, const double* z,
                                  const double* s1, const double* area, const int32_t* idx,
                                  int64_t ns, int pse, Rec64* out) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= ns) return;
  const int64_t j = idx[k];
  Rec64 r;
  r.x = x[j];
  r.y = y[j];
  r.z = z ? z[j] : 0.0;
  if (pse) {
    r.q = s1[j];  // f_j
    r.r = area[j];
  } else {
    r.q = __dmul_rn(s1[j], area[j]);  // zeta_j * A_j, the first product of the Fortran term
    r.r = 0.0;
  }
  r.idx = j;
  out[k] = r;
}

__global__ void prep_vec64_kernel(const double* x, const double* y, const double* z, const double* vx,
                                  const double* vy, const double* vz, const double* area, const int32_t* idx,
                                  int64_t ns, RecVec64* out) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= ns) return;
  const int64_t j = idx[k];
  out[k] = RecVec64{x[j], y[j], z ? z[j] : 0.0, vx[j], vy[j], vz ? vz[j] : 0.0, area[j], static_cast<long long>(j)};
}

__global__ void prep_plane64_kernel(const double* x, const double* y, const double* omega,
                                    const double* area, const int32_t* idx, int64_t ns,
                                    RecPlane64* out) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= ns) return;
  const int64_t j = idx[k];
  RecPlane64 r;
  r.x = x[j];
  r.y = y[j];
  r.q = __dmul_rn(omega[j], area[j]);
  r.idx = j;
  out[k] = r;
}

__global__ void prep_stream64_kernel(const double* x, const double* y, const double* z,
                                     const double* qr, const double* qa, const double* area,
                                     const int32_t* idx, int64_t ns, RecStream64* out) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= ns) return;
  const int64_t j = idx[k];
  RecStream64 r;
  r.x = x[j];
  r.y = y[j];
  r.z = z ? z[j] : 0.0;
  r.qr = qr[j];
  r.qa = qa ? qa[j] : 0.0;
  r.area = area[j];
  r.idx = j;
  r.pad = 0;
  out[k] = r;
}

// Totals sum_j zeta_j A_j over the active sources (relative and absolute), FP64 in a fixed
// order: one block, strided per thread, then a tree.
__global__ void __launch_bounds__(1024) stream_totals_kernel(const double* qr, const double* qa, const double* area,
                                                             const int32_t* idx, int64_t ns, double* tot) {
  __shared__ double sr[1024], sa[1024];
  double a = 0.0, b = 0.0;
  for (int64_t k = threadIdx.x; k < ns; k += 1024) {
    const int64_t j = idx[k];
    a += qr[j] * area[j];
    b += qa[j] * area[j];
  }
  sr[threadIdx.x] = a;
  sa[threadIdx.x] = b;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sr[threadIdx.x] += sr[threadIdx.x + w];
      sa[threadIdx.x] += sa[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    tot[0] = sr[0];
    tot[1] = sa[0];
  }
}

// ------------------------------------------------------------------ finish kernels
// Fixed-order FP64 reduction over the split-K chunks, then the per-target epilogue.

__global__ void finish_bve_kernel(const double* partial, int64_t nsplit, int64_t nt, int64_t ib,
                                  const double* x, const double* y, const double* z, double inv_a,
                                  double* u, double* v, double* w) {
  const int64_t il = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (il >= nt) return;
  double d0 = 0.0, d1 = 0.0, d2 = 0.0;
  for (int64_t c = 0; c < nsplit; ++c) {
    d0 += partial[(c * 3 + 0) * nt + il];
    d1 += partial[(c * 3 + 1) * nt + il];
    d2 += partial[(c * 3 + 2) * nt + il];
  }
  const int64_t i = ib + il;
  const double px = x[i] * inv_a, py = y[i] * inv_a, pz = z[i] * inv_a;
  u[il] = d1 * pz - d2 * py;
  v[il] = d2 * px - d0 * pz;
  w[il] = d0 * py - d1 * px;
}

__global__ void finish_plane_kernel(const double* partial, int64_t nsplit, int64_t nt, double* u,
                                    double* v) {
  const int64_t il = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (il >= nt) return;
  double su = 0.0, sv = 0.0;
  for (int64_t c = 0; c < nsplit; ++c) {
    su += partial[(c * 2 + 0) * nt + il];
    sv += partial[(c * 2 + 1) * nt + il];
  }
  u[il] = -su;
  v[il] = sv;
}

// u, v and the double dot product ux ux + 2 uy vx + vy vy of the SWE velocity sweep's six
// partials [chunk][6][nt] (SWEPlaneSolver.f90:530)
__global__ void swe_finish_kernel(const double* partial, int64_t nsplit, int64_t nt, double* u, double* v,
                                  double* ddot) {
  const int64_t il = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (il >= nt) return;
  double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int64_t k = 0; k < nsplit; ++k)
    for (int c = 0; c < 6; ++c) s[c] += partial[(k * 6 + c) * nt + il];
  u[il] = s[0];
  v[il] = s[1];
  ddot[il] = (s[2] * s[2] + (2.0 * s[3]) * s[4]) + s[5] * s[5];
}

// The sphere SWE velocity from the seven partials [chunk][7][nt] (Dr, Dp, W):
// u = Dr x p_i + Dp - p_i W with p_i = x_i / a, in FP64.
__global__ void swe_sphere_finish_kernel(const double* partial, int64_t nsplit, int64_t nt, int64_t ib,
                                         const double* x, const double* y, const double* z, double inv_a, double* u,
                                         double* v, double* w) {
  const int64_t il = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (il >= nt) return;
  double s[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int64_t k = 0; k < nsplit; ++k)
    for (int c = 0; c < 7; ++c) s[c] += partial[(k * 7 + c) * nt + il];
  const int64_t i = ib + il;
  const double px = x[i] * inv_a, py = y[i] * inv_a, pz = z[i] * inv_a;
  u[il] = (s[1] * pz - s[2] * py) + (s[3] - px * s[6]);
  v[il] = (s[2] * px - s[0] * pz) + (s[4] - py * s[6]);
  w[il] = (s[0] * py - s[1] * px) + (s[5] - pz * s[6]);
}

__global__ void finish_scalar_kernel(const double* partial, int64_t nsplit, int64_t nt,
                                     double scale, double* out) {
  const int64_t il = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (il >= nt) return;
  double s = 0.0;
  for (int64_t c = 0; c < nsplit; ++c) s += partial[c * nt + il];
  out[il] = s * scale;
}

// Stream functions: fixed-order chunk sum per component, plus (sphere) the ln(a^2) term
// k_const * (total - own term).
__global__ void finish_stream_kernel(const double* partial, int64_t nsplit, int64_t nt, int nc, double k_const,
                                     const double* tot, const double* self_w, double* out0, double* out1) {
  const int64_t il = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (il >= nt) return;
  for (int c = 0; c < nc; ++c) {
    double s = 0.0;
    for (int64_t k = 0; k < nsplit; ++k) s += partial[(k * nc + c) * nt + il];
    if (tot) s += k_const * (tot[c] - self_w[c * nt + il]);
    (c == 0 ? out0 : out1)[il] = s;
  }
}

// The FP64 kinds whose kernel decays as exp(-r^2) (the PSE operators), whose sweep skips
// source tiles beyond r = 10; *unit tells whether the distance is a great-circle one.
bool fp64_cutoff(int kind, int* unit) {
  switch (kind) {
    case kSumPseK8Geo:
    case kSumPseGrad:
    case kSumPseDiv:
    case kSumPseSphereDdot:
    case kSumPseInterpSphere:
      *unit = 1;
      return true;
    case kSumPseGaussChord:
    case kSumPseK8Chord:
    case kSumPsePlaneGrad:
    case kSumPsePlaneSecond:
    case kSumPsePlaneDdot:
    case kSumPseInterpPlane:
      *unit = 0;
      return true;
    default:
      return false;
  }
}

int tile_of(int kind, int mode) {
  if (mode == LPM_MODE_FP64) return k64Tile;
  switch (kind) {
    case kSumBve:
    case kSumBveMesh:
      return kBveTile;
    case kSumPlane:
    case kSumSwePlane:
      return kPlaneTile;
    case kSumPseGrad:
      return kPseTile;
    case kSumPseDiv:
      return kPseDivTile;
    case kSumSphereStream:
    case kSumPlaneStream:
    case kSumSweSphere:
      return kStreamTile;
    case kSumBetaPlane:
    case kSumBetaStream:
      return kBetaTile;
    default:
      return kPseTile;
  }
}

// Sources per group origin of a group-relative FP32C layout: 128 for the sphere BVE sweep and
// the sweeps that share its layout, 64 for the PSE sweeps (their cutoff's granularity) and
// the planar and beta-plane ones.
int origin_group(int kind) {
  static_assert(PseRel::kGroup == PlanePseRel::kGroup, "the Gaussian-chord kind serves the sphere and the plane");
  switch (kind) {
    case kSumBve:
    case kSumBveMesh:
    case kSumSphereStream:
    case kSumSweSphere:
      return BveRel::kGroup;
    case kSumPseK8Geo:
    case kSumPseGaussChord:
    case kSumPseGrad:
    case kSumPseDiv:
      return PseRel::kGroup;
    case kSumPseK8Chord:
      return PlanePseRel::kGroup;
    case kSumBetaPlane:
      return BetaRel::kGroup;
    case kSumBetaStream:
      return BetaStreamRel::kGroup;
    default:
      return PlaneRel::kGroup;
  }
}

size_t rec_bytes(int kind, int mode) {
  if (mode == LPM_MODE_FP64) {
    if (kind == kSumPlane) return sizeof(RecPlane64);
    if (kind == kSumPseDiv || kind == kSumPsePlaneSecond || kind == kSumPsePlaneDdot || kind == kSumPseSphereDdot ||
        kind == kSumSwePlane || kind == kSumSweSphere)
      return sizeof(RecVec64);
    if (kind == kSumSphereStream || kind == kSumPlaneStream || kind == kSumBetaPlane || kind == kSumBetaStream)
      return sizeof(RecStream64);
    return sizeof(Rec64);
  }
  switch (kind) {
    case kSumBve:
    case kSumBveMesh:
      return sizeof(BveRel::Rec);
    case kSumPlane:
      return sizeof(PlaneRel::Rec);
    case kSumSphereStream:
    case kSumSweSphere:
      return sizeof(StreamRel::Rec);
    case kSumPlaneStream:
      return sizeof(PlaneRel::Rec);
    case kSumBetaPlane:
      return sizeof(BetaRel::Rec);
    case kSumBetaStream:
      return sizeof(BetaStreamRel::Rec);
    case kSumSwePlane:
      return sizeof(PlaneRel::Rec);
    case kSumPseK8Geo:
    case kSumPseGaussChord:
    case kSumPseGrad:
    case kSumPseDiv:
      return sizeof(PseRel::Rec);  // also covers the planar record of the Gaussian-chord kind
    default:
      return sizeof(PlanePseRel::Rec);
  }
}

int comps_of(int kind) {
  switch (kind) {
    case kSumBve:
    case kSumBveMesh:
      return 3;
    case kSumPlane:
    case kSumSphereStream:
    case kSumBetaPlane:
    case kSumBetaStream:
      return 2;
    case kSumPseGrad:
      return 3;
    case kSumSwePlane:
      return 6;
    case kSumSweSphere:
      return 7;
    default:
      return 1;
  }
}

int targets_per_cta(int kind, int shape) {
  switch (kind) {
    case kSumBve:
    case kSumBveMesh:
      return kBveShapes[shape].threads * kBveShapes[shape].tpt;
    case kSumPlane:
      return kPlaneThreads * kPlaneTpt;
    case kSumSphereStream:
    case kSumPlaneStream:
    case kSumSweSphere:
      return kStreamThreads * kStreamTpt;
    case kSumBetaPlane:
    case kSumBetaStream:
      return kBetaThreads * kBetaTpt;
    default:
      return kPseThreads * kPseTpt;
  }
}

}  // namespace

// CTA size of an FP64 sweep over `lanes` threads (one per target, or kSplit64 per target):
// every CTA does the same work and all of them are resident at once, so an SM's time is its
// CTA count times the CTA size, and the sweep takes the longest SM's.  Of 128, 64 and 32
// threads, the size that minimises ceil(CTAs / SMs) x size (the larger on a tie): e.g. at
// 7,682 targets x 4 lanes, 961 CTAs of 32 threads put at most 7 on an SM (224 thread-slots)
// where 241 CTAs of 128 put 2 (256).
static int fp64_block_threads(int64_t lanes, int64_t sms) {
  int best = k64Threads;
  int64_t best_cost = ceil_div(ceil_div(lanes, k64Threads), sms) * k64Threads;
  for (int t : {64, 32}) {
    const int64_t cost = ceil_div(ceil_div(lanes, t), sms) * t;
    if (cost < best_cost) {
      best_cost = cost;
      best = t;
    }
  }
  return best;
}

int64_t choose_split(int64_t blocks, int64_t tiles, int64_t slots, int64_t max_split) {
  if (blocks < 1) blocks = 1;
  if (slots < 1) slots = 1;
  int64_t lim = tiles < max_split ? tiles : max_split;
  if (lim > 4096) lim = 4096;
  int64_t best = 1;
  double best_cost = 1e300;
  for (int64_t s = 1; s <= lim; ++s) {
    const int64_t tpc = ceil_div(tiles, s);
    if (s > 1 && ceil_div(tiles, tpc) < s) continue;  // same chunks as a smaller split
    const double cost = static_cast<double>(ceil_div(blocks * s, slots)) * static_cast<double>(tpc + 1);
    if (cost < best_cost) {
      best_cost = cost;
      best = s;
    }
  }
  return best;
}

bool sum_uses_sorted_sources(int kind, int mode) {
  return mode == LPM_MODE_FP32C && (kind == kSumBve || kind == kSumBveMesh || kind == kSumPlane ||
                                    kind == kSumSphereStream || kind == kSumPseK8Geo || kind == kSumPseGaussChord ||
                                    kind == kSumPseK8Chord || kind == kSumPseGrad || kind == kSumPseDiv ||
                                    kind == kSumPlaneStream || kind == kSumSwePlane || kind == kSumSweSphere ||
                                    kind == kSumBetaPlane || kind == kSumBetaStream);
}

namespace {
// The FP32C PSE sums sweep only the tiles within reach of each CTA's targets, in balanced
// shares (engine.cuh); their prep kernels write a ball per tile.
bool pse_culls_tiles(int kind) {
  return kind == kSumPseK8Geo || kind == kSumPseGaussChord || kind == kSumPseK8Chord || kind == kSumPseGrad ||
         kind == kSumPseDiv;
}

// Shares per target block of a culled sweep: about six waves of CTAs in all, at most 32 per
// block.  A block's in-reach work is split evenly, but tiles differ in cost (near and partly
// reached groups), so finer CTAs balance the SMs better until the per-CTA scan of the tile
// balls (every CTA of a block scans them all) starts to count.  Measured on GB300 (K8 and
// Gaussian at cubed nests 6-8, planar K8 at quad nests 7-8, 1 to 32 shares): within 3 % of
// the best count at every size, where a fixed 3 was up to 2x slower (cubed nest 6).
int64_t cull_shares(int64_t blocks, int64_t slots) {
  if (blocks < 1) blocks = 1;
  const int64_t m = ceil_div(6 * (slots > 0 ? slots : 1), blocks);
  return m < 1 ? 1 : (m > 32 ? 32 : m);
}

// The FP32C PSE kinds also sort their targets (nt of them) with the same scratch.
bool pse_sorts_targets(int kind) {
  return kind == kSumPseK8Geo || kind == kSumPseGaussChord || kind == kSumPseK8Chord || kind == kSumPseGrad ||
         kind == kSumPseDiv;
}
}  // namespace

size_t sort_scratch_bytes(int kind, int64_t ns, int64_t nt) {
  int unit = 0;
  const bool targets = pse_sorts_targets(kind) || fp64_cutoff(kind, &unit);  // FP64 cut sums sort targets only
  const int64_t m = targets && nt > ns ? nt : ns;
  // planar kinds sort in 2-D; the Gaussian-chord Laplacian serves the plane and the sphere
  if (kind == kSumPlane || kind == kSumPseK8Chord || kind == kSumPlaneStream || kind == kSumSwePlane ||
      kind == kSumBetaPlane || kind == kSumBetaStream || kind == kSumPsePlaneGrad || kind == kSumPsePlaneSecond ||
      kind == kSumPsePlaneDdot || kind == kSumPseInterpPlane)
    return std::max(curve_sort2d_bytes(m), pse_sorts_targets(kind) ? select_in_order_bytes(m) : size_t{0});
  if (kind == kSumPseGaussChord) return std::max({curve_sort_bytes(m), curve_sort2d_bytes(m), select_in_order_bytes(m)});
  return std::max(curve_sort_bytes(m), pse_sorts_targets(kind) ? select_in_order_bytes(m) : size_t{0});
}

int bve_shape_count() { return kBveShapeCount; }

SumPlan plan_sum(int kind, int mode, int64_t ns, int64_t nt, int sm_count, int shape) {
  if (shape < 0 || shape >= kBveShapeCount) shape = 0;
  SumPlan pl;
  pl.shape = shape;
  const int tile = tile_of(kind, mode);
  pl.n_tiles = ceil_div(ns > 0 ? ns : 1, tile);
  pl.src_bytes = static_cast<size_t>(pl.n_tiles) * tile * rec_bytes(kind, mode);
  if (sum_uses_sorted_sources(kind, mode)) {
    // the group origins follow the records
    static_assert(sizeof(BveRel::Origin) == sizeof(PlaneRel::Origin) &&
                      sizeof(BveRel::Origin) == sizeof(BetaRel::Origin) &&
                      sizeof(BveRel::Origin) == sizeof(BetaStreamRel::Origin),
                  "one origin layout size");
    pl.src_bytes = align_up(pl.src_bytes, 256) +
                   static_cast<size_t>(pl.n_tiles) * (tile / origin_group(kind)) * sizeof(BveRel::Origin);
  }
  if (mode == LPM_MODE_FP32C && pse_culls_tiles(kind)) {
    // the tiles' balls follow the group origins
    pl.src_bytes = align_up(pl.src_bytes, 256) + static_cast<size_t>(pl.n_tiles) * sizeof(float4);
  }
  if (mode == LPM_MODE_FP32C && pse_sorts_targets(kind)) {
    pl.tperm_offset = align_up(pl.src_bytes, 256);
    pl.src_bytes = pl.tperm_offset + 2 * align_up(static_cast<size_t>(nt) * sizeof(int32_t), 256);
  }
  if (mode == LPM_MODE_FP32C && kind == kSumSphereStream) {
    // the sources' own zeta A (2 x nt) and the two totals follow the group origins
    pl.src_bytes = align_up(pl.src_bytes, 256) + align_up(2 * static_cast<size_t>(nt) * sizeof(double), 256) +
                   2 * sizeof(double);
  }
  if (mode == LPM_MODE_FP64) {
    int unit = 0;
    if (fp64_cutoff(kind, &unit)) {
      // the tiles' bounding balls follow the records, then the targets' curve order (two
      // lists of nt int32, as for the FP32C PSE sums)
      pl.src_bytes = align_up(pl.src_bytes, 256) + static_cast<size_t>(pl.n_tiles) * sizeof(TileBall);
      pl.tperm_offset = align_up(pl.src_bytes, 256);
      pl.src_bytes = pl.tperm_offset + 2 * align_up(static_cast<size_t>(nt) * sizeof(int32_t), 256);
    }
    // one target per thread and no split (the sum is sequential per target): a target set
    // too small for one 128-thread CTA per SM takes CTAs of one warp (and, for the BVE and
    // planar velocity, the split sweep) so that more SMs share the FP64 work.  At one CTA
    // per SM and above the sequential sweep keeps the FP64 pipe busy (85 % at icos nest 5).
    const int64_t sms = sm_count > 0 ? sm_count : 152;
    pl.fp64_small = ceil_div(nt, k64Threads) < sms;
    pl.fp64_threads = fp64_block_threads(nt, sms);
    pl.fp64_split_threads = fp64_block_threads(nt * kSplit64, sms);
    pl.nsplit = 1;
    pl.tiles_per_chunk = pl.n_tiles;
    pl.partial_bytes = 0;
    return pl;
  }
  // Split the source range so that the last wave of CTAs is nearly full.
  const int64_t tblocks = ceil_div(nt, targets_per_cta(kind, shape));
  const int minb = (kind == kSumBve || kind == kSumBveMesh)          ? kBveShapes[shape].minb
                   : kind == kSumSwePlane                            ? kSweMinB
                   : kind == kSumSweSphere                           ? kSweSphereMinB
                                                                     : 4;
  const int64_t slots = static_cast<int64_t>(sm_count > 0 ? sm_count : 152) * minb;
  if (mode == LPM_MODE_FP32C && pse_culls_tiles(kind)) {
    // every CTA scans the whole source range for its in-reach tiles and takes one of nsplit
    // equal shares of them
    pl.tiles_per_chunk = pl.n_tiles;
    pl.nsplit = cull_shares(tblocks, slots);
  } else {
    const int64_t nsplit = choose_split(tblocks, pl.n_tiles, slots, 65535);
    pl.tiles_per_chunk = ceil_div(pl.n_tiles, nsplit);
    pl.nsplit = ceil_div(pl.n_tiles, pl.tiles_per_chunk);
  }
  pl.partial_bytes = static_cast<size_t>(pl.nsplit) * comps_of(kind) * nt * sizeof(double);
  if (kind == kSumSwePlane || kind == kSumSweSphere) {
    // the surface-height Laplacian: the K8 PSE sweep (planar or geodesic), after the velocity sweep
    const SumPlan pp = plan_sum(kind == kSumSwePlane ? kSumPseK8Chord : kSumPseK8Geo, mode, ns, nt, sm_count, 0);
    pl.aux_n_tiles = pp.n_tiles;
    pl.aux_tiles_per_chunk = pp.tiles_per_chunk;
    pl.aux_nsplit = pp.nsplit;
    pl.aux_src_offset = align_up(pl.src_bytes, 256);
    pl.src_bytes = pl.aux_src_offset + pp.src_bytes;
    pl.partial_bytes = std::max(pl.partial_bytes, pp.partial_bytes);
  }
  return pl;
}

namespace {
// The sphere PSE sums on the group-relative layout (pse_rel.cuh): sort, prep and sweep.
template <int OP, int ANG>
void pse_rel_launch(const SumJob& job, const SumPlan& plan, const int32_t* src_list, const PseRelArgs& a) {
  constexpr int TILE = OP == kPseOpDiv ? kPseDivTile : kPseTile;
  constexpr int S = OP == kPseOpDiv ? kPseDivStages : kPseStages;
  pse_rel_prep_kernel<OP, ANG, TILE><<<static_cast<unsigned>(plan.n_tiles), TILE, 0, job.stream>>>(
      job.x, job.y, job.z, job.s1, job.s2, job.s3, job.area, src_list, job.ns, a.inv_a,
      const_cast<PseRel::Rec*>(a.src), const_cast<BveRel::Origin*>(a.org), const_cast<float4*>(a.tball));
  const dim3 grid(static_cast<unsigned>(ceil_div(job.nt, kPseThreads * kPseTpt)), static_cast<unsigned>(plan.nsplit));
  pse_rel_sweep_kernel<OP, ANG, kPseThreads, kPseTpt, TILE, kPseMinB, S><<<grid, kPseThreads, 0, job.stream>>>(a);
}

// The list ib, ib + 1, ..., ib + n - 1.
__global__ void iota_kernel(int64_t n, int64_t ib, int32_t* out) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) out[k] = static_cast<int32_t>(ib + k);
}

// The targets of a PSE sweep in curve order, when the plan has room for them and the job
// brings sort scratch (nullptr otherwise: the sweep takes targets in index order).  The sort
// scratch is reused after the sources' sort (stream order).
template <class SortFn>
int sorted_targets(const SumJob& job, const SumPlan& plan, SortFn&& sort, const int32_t** tperm) {
  *tperm = nullptr;
  if (!job.sort_scratch || plan.tperm_offset == 0 || job.nt < 2) return LPM_OK;
  int32_t* in = reinterpret_cast<int32_t*>(static_cast<char*>(job.src_buf) + plan.tperm_offset);
  int32_t* out = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(in) +
                                            align_up(static_cast<size_t>(job.nt) * sizeof(int32_t), 256));
  iota_kernel<<<static_cast<unsigned>(ceil_div(job.nt, 256)), 256, 0, job.stream>>>(job.nt, job.ib, in);
  LPM_TRY(sort(in, out));
  *tperm = out;
  return LPM_OK;
}

// Whether a PSE job's targets are every particle, so that its sources (the active ones) can take
// the targets' curve order instead of a sort of their own.
bool targets_cover_sources(const SumJob& job, const SumPlan& plan) {
  return job.sort_scratch && plan.tperm_offset != 0 && job.ib == 0 && job.nt == job.n && job.nt >= 2;
}

int launch_pse_rel(const SumJob& job, const SumPlan& plan, int64_t npad) {
  const double inv_a = 1.0 / job.radius;
  const int32_t* src_list = job.src_idx;
  const int32_t* tperm = nullptr;
  auto sort3 = [&](const int32_t* in, int32_t* out) {
    return curve_sort(job.stream, job.nt, in, job.x, job.y, job.z, inv_a, job.sort_scratch, job.sort_bytes, out);
  };
  if (targets_cover_sources(job, plan)) {
    // one sort: every particle in curve order, the sources picked out of it in that order
    // (the same order as a sort of their own, whose keys are the same function of position)
    LPM_TRY(sorted_targets(job, plan, sort3, &tperm));
    LPM_TRY(select_in_order(job.stream, job.n, tperm, job.ns, job.src_idx, job.sort_scratch, job.sort_bytes,
                            job.sorted));
    src_list = job.sorted;
  } else {
    if (job.sort_scratch) {
      LPM_TRY(curve_sort(job.stream, job.ns, job.src_idx, job.x, job.y, job.z, inv_a, job.sort_scratch,
                         job.sort_bytes, job.sorted));
      src_list = job.sorted;
    }
    LPM_TRY(sorted_targets(job, plan, sort3, &tperm));
  }
  PseRelArgs a;
  a.tperm = tperm;
  a.x = job.x;
  a.y = job.y;
  a.z = job.z;
  a.f = job.s1;
  a.vy = job.s2;
  a.vz = job.s3;
  a.inv_a = inv_a;
  const double ks = job.radius / job.eps;
  a.ks2 = static_cast<float>(ks * ks);
  a.c_cut = static_cast<float>(std::sqrt(static_cast<double>(PseRel::kCutR2)) * job.eps / job.radius);
  a.half_a2 = static_cast<float>(0.5 * job.radius * job.radius);
  a.src = static_cast<PseRel::Rec*>(job.src_buf);
  a.org = reinterpret_cast<BveRel::Origin*>(static_cast<char*>(job.src_buf) +
                                            align_up(static_cast<size_t>(npad) * sizeof(PseRel::Rec), 256));
  // the Laplacians' tile balls follow the origins (plan_sum)
  const int tile = job.kind == kSumPseDiv ? kPseDivTile : kPseTile;
  a.tball = reinterpret_cast<const float4*>(
      reinterpret_cast<const char*>(a.org) +
      align_up(static_cast<size_t>(plan.n_tiles) * (tile / PseRel::kGroup) * sizeof(BveRel::Origin), 256));
  a.n_tiles = plan.n_tiles;
  a.tiles_per_chunk = plan.tiles_per_chunk;
  a.ib = job.ib;
  a.nt = job.nt;
  a.partial = job.partial;
  a.status = job.status;
  a.wait = job.wait;
  const bool series = job.eps <= 0.06 * job.radius;  // the asin^2 series angle (pse_rel.cuh)
  switch (job.kind) {
    case kSumPseK8Geo:
      if (series) pse_rel_launch<kPseOpLapK8, kPseAngleSeries>(job, plan, src_list, a);
      else pse_rel_launch<kPseOpLapK8, kPseAngleAsin>(job, plan, src_list, a);
      break;
    case kSumPseGaussChord:
      pse_rel_launch<kPseOpLapGauss, kPseAngleChord>(job, plan, src_list, a);
      break;
    case kSumPseGrad:
      if (series) pse_rel_launch<kPseOpGrad, kPseAngleSeries>(job, plan, src_list, a);
      else pse_rel_launch<kPseOpGrad, kPseAngleAsin>(job, plan, src_list, a);
      break;
    default:
      if (series) pse_rel_launch<kPseOpDiv, kPseAngleSeries>(job, plan, src_list, a);
      else pse_rel_launch<kPseOpDiv, kPseAngleAsin>(job, plan, src_list, a);
      break;
  }
  return LPM_OK;
}
}  // namespace

namespace {
int launch_plane_pse_rel(const SumJob& job, const SumPlan& plan, int64_t npad) {
  const int32_t* src_list = job.src_idx;
  const int32_t* tperm = nullptr;
  auto sort2 = [&](const int32_t* in, int32_t* out) {
    return curve_sort2d(job.stream, job.nt, in, job.x, job.y, job.sort_scratch, job.sort_bytes, out);
  };
  if (targets_cover_sources(job, plan)) {
    // one sort: every particle along the curve over their bounding box, the sources picked
    // out of it in that order
    LPM_TRY(sorted_targets(job, plan, sort2, &tperm));
    LPM_TRY(select_in_order(job.stream, job.n, tperm, job.ns, job.src_idx, job.sort_scratch, job.sort_bytes,
                            job.sorted));
    src_list = job.sorted;
  } else {
    if (job.sort_scratch) {
      LPM_TRY(curve_sort2d(job.stream, job.ns, job.src_idx, job.x, job.y, job.sort_scratch, job.sort_bytes,
                           job.sorted));
      src_list = job.sorted;
    }
    LPM_TRY(sorted_targets(job, plan, sort2, &tperm));
  }
  PlanePseRelArgs a;
  a.tperm = tperm;
  a.x = job.x;
  a.y = job.y;
  a.f = job.s1;
  a.ks2 = static_cast<float>(1.0 / (job.eps * job.eps));
  a.c_cut = static_cast<float>(std::sqrt(static_cast<double>(PseRel::kCutR2)) * job.eps);
  a.src = static_cast<PlanePseRel::Rec*>(job.src_buf);
  a.org = reinterpret_cast<PlaneRel::Origin*>(static_cast<char*>(job.src_buf) +
                                              align_up(static_cast<size_t>(npad) * sizeof(PlanePseRel::Rec), 256));
  // the tile balls follow the origins (plan_sum)
  a.tball = reinterpret_cast<const float4*>(
      reinterpret_cast<const char*>(a.org) +
      align_up(static_cast<size_t>(plan.n_tiles) * (kPseTile / PlanePseRel::kGroup) * sizeof(PlaneRel::Origin), 256));
  a.n_tiles = plan.n_tiles;
  a.tiles_per_chunk = plan.tiles_per_chunk;
  a.ib = job.ib;
  a.nt = job.nt;
  a.partial = job.partial;
  a.status = job.status;
  plane_pse_rel_prep_kernel<kPseTile><<<static_cast<unsigned>(plan.n_tiles), kPseTile, 0, job.stream>>>(
      job.x, job.y, job.s1, job.area, src_list, job.ns, const_cast<PlanePseRel::Rec*>(a.src),
      const_cast<PlaneRel::Origin*>(a.org), const_cast<float4*>(a.tball));
  const dim3 grid(static_cast<unsigned>(ceil_div(job.nt, kPseThreads * kPseTpt)), static_cast<unsigned>(plan.nsplit));
  if (job.kind == kSumPseK8Chord) {
    plane_pse_rel_sweep_kernel<true, kPseThreads, kPseTpt, kPseTile, kPseMinB, kPseStages>
        <<<grid, kPseThreads, 0, job.stream>>>(a);
  } else {
    plane_pse_rel_sweep_kernel<false, kPseThreads, kPseTpt, kPseTile, kPseMinB, kPseStages>
        <<<grid, kPseThreads, 0, job.stream>>>(a);
  }
  return LPM_OK;
}
}  // namespace

int launch_sum(const SumJob& job, const SumPlan& plan) {
  const int pb = 256;
  const unsigned prep_grid_ns = static_cast<unsigned>(ceil_div(job.ns > 0 ? job.ns : 1, pb));
  const unsigned fin_grid = static_cast<unsigned>(ceil_div(job.nt, pb));
  const int tile = tile_of(job.kind, job.mode);
  const int64_t npad = plan.n_tiles * tile;
  const unsigned prep_grid_pad = static_cast<unsigned>(ceil_div(npad, pb));

  if (job.mode == LPM_MODE_FP64) {
    const int t64 = plan.fp64_threads;
    const unsigned g = static_cast<unsigned>(ceil_div(job.nt, t64));
    const int ts = plan.fp64_split_threads;
    const unsigned gs = static_cast<unsigned>(ceil_div(job.nt, ts / kSplit64));  // the split sweep's grid
    Fp64Cut cut;
    if (fp64_cutoff(job.kind, &cut.unit)) {
      TileBall* bounds = reinterpret_cast<TileBall*>(
          static_cast<char*>(job.src_buf) +
          align_up(static_cast<size_t>(plan.n_tiles) * k64Tile * rec_bytes(job.kind, job.mode), 256));
      tile_bounds64_kernel<<<static_cast<unsigned>(plan.n_tiles), k64Tile, 0, job.stream>>>(
          job.x, job.y, job.z, job.src_idx, job.ns, cut.unit, bounds);
      cut.bounds = bounds;
      cut.x = job.x;
      cut.y = job.y;
      cut.z = job.z;
      cut.reach = std::sqrt(static_cast<double>(PseRel::kCutR2)) * job.eps / (cut.unit ? job.radius : 1.0);
      // targets in curve order when the job brings sort scratch (the host-buffer calls)
      const bool sphere = cut.unit || (job.kind == kSumPseGaussChord && job.z);
      LPM_TRY(sorted_targets(job, plan, [&](const int32_t* in, int32_t* out) {
        return sphere ? curve_sort(job.stream, job.nt, in, job.x, job.y, job.z, 1.0 / job.radius, job.sort_scratch,
                                   job.sort_bytes, out)
                      : curve_sort2d(job.stream, job.nt, in, job.x, job.y, job.sort_scratch, job.sort_bytes, out);
      }, &cut.tperm));
    }
    switch (job.kind) {
      case kSumBve:
      case kSumBveMesh: {
        prep_rec64_kernel<<<prep_grid_ns, pb, 0, job.stream>>>(job.x, job.y, job.z, job.s1, job.area,
                                                               job.src_idx, job.ns, 0,
                                                               static_cast<Rec64*>(job.src_buf));
        BveF64Params p{job.x, job.y, job.z, job.radius * job.radius, (4.0 * kPi) * job.radius,
                       job.out0, job.out1, job.out2};
        const Rec64* src = static_cast<const Rec64*>(job.src_buf);
        if (plan.fp64_small) {
          // a small target set: kSplit64 lanes per target (the terms in parallel, the sum in order)
          if (job.kind == kSumBve) {
            launch_split64<BveF64<0>, Rec64>(ts, gs, job.stream, p, src, job.ns, job.ib, job.nt, job.status);
          } else {
            launch_split64<BveF64<1>, Rec64>(ts, gs, job.stream, p, src, job.ns, job.ib, job.nt, job.status);
          }
        } else if (job.kind == kSumBve) {
          seq_fp64_kernel<BveF64<0>, Rec64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib, job.nt, job.status);
        } else {
          seq_fp64_kernel<BveF64<1>, Rec64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib, job.nt, job.status);
        }
        break;
      }
      case kSumPlane: {
        prep_plane64_kernel<<<prep_grid_ns, pb, 0, job.stream>>>(job.x, job.y, job.s1, job.area, job.src_idx,
                                                                 job.ns, static_cast<RecPlane64*>(job.src_buf));
        PlaneF64Params p{job.x, job.y, 2.0 * kPi, job.delta * job.delta, job.out0, job.out1};
        const RecPlane64* src = static_cast<const RecPlane64*>(job.src_buf);
        if (plan.fp64_small) {
          launch_split64<PlaneF64, RecPlane64>(ts, gs, job.stream, p, src, job.ns, job.ib, job.nt, job.status);
        } else {
          seq_fp64_kernel<PlaneF64, RecPlane64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib, job.nt,
                                                                           job.status);
        }
        break;
      }
      case kSumPseK8Geo:
      case kSumPseGaussChord:
      case kSumPseK8Chord: {
        prep_rec64_kernel<<<prep_grid_ns, pb, 0, job.stream>>>(job.x, job.y, job.z, job.s1, job.area,
                                                               job.src_idx, job.ns, 1,
                                                               static_cast<Rec64*>(job.src_buf));
        const double eps2 = job.eps * job.eps;
        PseF64Params p{job.x, job.y, job.z, job.s1, job.eps, eps2, 1.0 / eps2, job.radius, job.out0};
        const Rec64* src = static_cast<const Rec64*>(job.src_buf);
        if (job.kind == kSumPseK8Geo) {
          seq_fp64_kernel<PseF64<kPseK8Geodesic>, Rec64><<<g, t64, 0, job.stream>>>(
              p, src, job.ns, job.ib, job.nt, job.status, cut);
        } else if (job.kind == kSumPseGaussChord) {
          seq_fp64_kernel<PseF64<kPseGaussChord>, Rec64><<<g, t64, 0, job.stream>>>(
              p, src, job.ns, job.ib, job.nt, job.status, cut);
        } else {
          seq_fp64_kernel<PseF64<kPseK8Chord>, Rec64><<<g, t64, 0, job.stream>>>(
              p, src, job.ns, job.ib, job.nt, job.status, cut);
        }
        break;
      }
      case kSumPseGrad:
      case kSumPseDiv: {
        const double eps2 = job.eps * job.eps;
        PseVecF64Params p{job.x, job.y, job.z, job.s1, job.s1, job.s2, job.s3, job.eps, eps2,
                          job.eps * eps2, job.radius, 0.0, job.out0, job.out1, job.out2};
        if (job.kind == kSumPseGrad) {
          p.scale = 1.0 / eps2;  // MultiplyFieldByScalar(scalarGrad, 1/eps**2)
          prep_rec64_kernel<<<prep_grid_ns, pb, 0, job.stream>>>(job.x, job.y, job.z, job.s1, job.area,
                                                                 job.src_idx, job.ns, 1,
                                                                 static_cast<Rec64*>(job.src_buf));
          seq_fp64_kernel<PseGradF64, Rec64><<<g, t64, 0, job.stream>>>(
              p, static_cast<const Rec64*>(job.src_buf), job.ns, job.ib, job.nt, job.status, cut);
        } else {
          p.scale = 1.0 / job.eps;  // MultiplyFieldByScalar(divergence, 1/eps)
          prep_vec64_kernel<<<prep_grid_ns, pb, 0, job.stream>>>(job.x, job.y, job.z, job.s1, job.s2, job.s3,
                                                                 job.area, job.src_idx, job.ns,
                                                                 static_cast<RecVec64*>(job.src_buf));
          seq_fp64_kernel<PseDivF64, RecVec64><<<g, t64, 0, job.stream>>>(
              p, static_cast<const RecVec64*>(job.src_buf), job.ns, job.ib, job.nt, job.status, cut);
        }
        break;
      }
      case kSumSphereStream:
      case kSumPlaneStream: {
        prep_stream64_kernel<<<prep_grid_ns, pb, 0, job.stream>>>(job.x, job.y, job.z, job.s1, job.s2,
                                                                  job.area, job.src_idx, job.ns,
                                                                  static_cast<RecStream64*>(job.src_buf));
        StreamF64Params p{job.x, job.y, job.z, job.radius * job.radius, 4.0 * kPi, 2.0 * kPi, job.out0, job.out1};
        const RecStream64* src = static_cast<const RecStream64*>(job.src_buf);
        if (job.kind == kSumSphereStream) {
          seq_fp64_kernel<SphereStreamF64, RecStream64><<<g, t64, 0, job.stream>>>(
              p, src, job.ns, job.ib, job.nt, job.status);
        } else {
          seq_fp64_kernel<PlaneStreamF64, RecStream64><<<g, t64, 0, job.stream>>>(
              p, src, job.ns, job.ib, job.nt, job.status);
        }
        break;
      }
      case kSumPsePlaneGrad:
      case kSumPseInterpPlane:
      case kSumPseInterpSphere: {
        prep_rec64_kernel<<<prep_grid_ns, pb, 0, job.stream>>>(job.x, job.y, job.z, job.s1, job.area,
                                                               job.src_idx, job.ns, 1,
                                                               static_cast<Rec64*>(job.src_buf));
        const double eps2 = job.eps * job.eps;
        PseExtF64Params p{job.x, job.y, job.z, job.s1, job.s2, job.s3, job.eps, eps2, job.eps * eps2,
                          job.radius, job.radius2, 0.0, 1.0 / job.eps, job.out0, job.out1, job.out2, job.out3};
        const Rec64* src = static_cast<const Rec64*>(job.src_buf);
        if (job.kind == kSumPsePlaneGrad) {
          seq_fp64_kernel<PsePlaneGradF64, Rec64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib, job.nt,
                                                                                    job.status, cut);
        } else if (job.kind == kSumPseInterpPlane) {
          seq_fp64_kernel<PseInterpF64<false>, Rec64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib,
                                                                                        job.nt, job.status, cut);
        } else {
          seq_fp64_kernel<PseInterpF64<true>, Rec64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib,
                                                                                       job.nt, job.status, cut);
        }
        break;
      }
      case kSumPsePlaneSecond:
      case kSumPsePlaneDdot:
      case kSumPseSphereDdot:
      case kSumSwePlane:
      case kSumSweSphere: {
        prep_vec64_kernel<<<prep_grid_ns, pb, 0, job.stream>>>(job.x, job.y, job.z, job.s1, job.s2, job.s3,
                                                               job.area, job.src_idx, job.ns,
                                                               static_cast<RecVec64*>(job.src_buf));
        const double eps2 = job.eps * job.eps;
        PseExtF64Params p{job.x, job.y, job.z, job.s1, job.s2, job.s3, job.eps, eps2, job.eps * eps2,
                          job.radius, job.radius2, 0.0, 1.0 / job.eps, job.out0, job.out1, job.out2, job.out3};
        const RecVec64* src = static_cast<const RecVec64*>(job.src_buf);
        switch (job.kind) {
          case kSumPsePlaneSecond:
            seq_fp64_kernel<PsePlaneSecondF64, RecVec64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib,
                                                                                          job.nt, job.status, cut);
            break;
          case kSumPsePlaneDdot:
            seq_fp64_kernel<PsePlaneDdotF64, RecVec64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib,
                                                                                        job.nt, job.status, cut);
            break;
          case kSumPseSphereDdot:
            seq_fp64_kernel<PseSphereDdotF64, RecVec64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib,
                                                                                         job.nt, job.status, cut);
            break;
          case kSumSwePlane:
            p.k0 = 2.0 * kPi;  // 2.0_kreal * PI
            seq_fp64_kernel<SwePlaneF64, RecVec64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib,
                                                                                    job.nt, job.status);
            break;
          default:
            p.k0 = ((4.0 * kPi) * job.radius) * job.radius;  // 4.0_kreal * PI * radius * radius
            seq_fp64_kernel<SweSphereF64, RecVec64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib,
                                                                                     job.nt, job.status);
            break;
        }
        break;
      }
      case kSumBetaPlane:
      case kSumBetaStream: {
        prep_stream64_kernel<<<prep_grid_ns, pb, 0, job.stream>>>(job.x, job.y, nullptr, job.s1, job.s2,
                                                                  job.area, job.src_idx, job.ns,
                                                                  static_cast<RecStream64*>(job.src_buf));
        BetaF64Params p{job.x, job.y, 2.0 * kPi, 4.0 * kPi, job.out0, job.out1};
        const RecStream64* src = static_cast<const RecStream64*>(job.src_buf);
        if (job.kind == kSumBetaPlane) {
          seq_fp64_kernel<BetaVelF64, RecStream64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib, job.nt,
                                                                                    job.status);
        } else {
          seq_fp64_kernel<BetaStreamF64, RecStream64><<<g, t64, 0, job.stream>>>(p, src, job.ns, job.ib,
                                                                                       job.nt, job.status);
        }
        break;
      }
      default:
        return set_error(LPM_ERR_ARG, "unknown sum kind %d", job.kind);
    }
    LPM_CUDA_TRY(cudaGetLastError());
    return LPM_OK;
  }
  if (sum_is_fp64_only(job.kind)) return set_error(LPM_ERR_ARG, "this operator has only the FP64 mode");

  // ---------------- FP32C
  switch (job.kind) {
    case kSumBve:
    case kSumBveMesh: {
      const double inv_a = 1.0 / job.radius;
      const int32_t* src_list = job.src_idx;
      if (job.sort_scratch) {
        LPM_TRY(curve_sort(job.stream, job.ns, job.src_idx, job.x, job.y, job.z, inv_a, job.sort_scratch,
                            job.sort_bytes, job.sorted));
        src_list = job.sorted;
      }
      BveRel::Rec* recs = static_cast<BveRel::Rec*>(job.src_buf);
      BveRel::Origin* org = reinterpret_cast<BveRel::Origin*>(
          static_cast<char*>(job.src_buf) + align_up(static_cast<size_t>(npad) * sizeof(BveRel::Rec), 256));
      bve_rel_prep_kernel<kBveTile><<<static_cast<unsigned>(plan.n_tiles), kBveTile, 0, job.stream>>>(
          job.x, job.y, job.z, job.s1, job.area, src_list, job.ns, inv_a, -1.0 / (2.0 * kPi * job.radius), recs,
          org);
      SweepArgs<BveF32> a;
      a.p = BveF32::Params{job.x, job.y, job.z, inv_a};
      a.src = reinterpret_cast<const BveF32::Rec*>(job.src_buf);
      a.n_tiles = plan.n_tiles;
      a.tiles_per_chunk = plan.tiles_per_chunk;
      a.ib = job.ib;
      a.nt = job.nt;
      a.partial = job.partial;
      a.status = job.status;
      a.wait = job.wait;
      const BveShape sh = kBveShapes[plan.shape];
      const dim3 grid(static_cast<unsigned>(ceil_div(job.nt, sh.threads * sh.tpt)), static_cast<unsigned>(plan.nsplit));
      switch (plan.shape) {
        case 0:
          bve_rel_sweep_kernel<128, 4, kBveTile, 4><<<grid, 128, 0, job.stream>>>(a, org);
          break;
        case 1:
          bve_rel_sweep_kernel<256, 4, kBveTile, 2><<<grid, 256, 0, job.stream>>>(a, org);
          break;
        case 2:
          bve_rel_sweep_kernel<128, 6, kBveTile, 2><<<grid, 128, 0, job.stream>>>(a, org);
          break;
        default:
          bve_rel_sweep_kernel<128, 8, kBveTile, 2><<<grid, 128, 0, job.stream>>>(a, org);
          break;
      }
      finish_bve_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, plan.nsplit, job.nt, job.ib, job.x,
                                                         job.y, job.z, inv_a, job.out0, job.out1, job.out2);
      break;
    }
    case kSumPlane: {
      const int32_t* src_list = job.src_idx;
      if (job.sort_scratch) {
        LPM_TRY(curve_sort2d(job.stream, job.ns, job.src_idx, job.x, job.y, job.sort_scratch, job.sort_bytes,
                             job.sorted));
        src_list = job.sorted;
      }
      PlaneRel::Rec* recs = static_cast<PlaneRel::Rec*>(job.src_buf);
      PlaneRel::Origin* org = reinterpret_cast<PlaneRel::Origin*>(
          static_cast<char*>(job.src_buf) + align_up(static_cast<size_t>(npad) * sizeof(PlaneRel::Rec), 256));
      plane_rel_prep_kernel<kPlaneTile><<<static_cast<unsigned>(plan.n_tiles), kPlaneTile, 0, job.stream>>>(
          job.x, job.y, job.s1, job.area, src_list, job.ns, 1.0 / (2.0 * kPi), recs, org);
      PlaneRelArgs a;
      a.x = job.x;
      a.y = job.y;
      a.d2 = static_cast<float>(job.delta * job.delta) + 7.888609052210118e-31f;  // + 2^-100
      a.src = recs;
      a.org = org;
      a.n_tiles = plan.n_tiles;
      a.tiles_per_chunk = plan.tiles_per_chunk;
      a.ib = job.ib;
      a.nt = job.nt;
      a.partial = job.partial;
      a.status = job.status;
      const dim3 grid(static_cast<unsigned>(ceil_div(job.nt, kPlaneThreads * kPlaneTpt)),
                      static_cast<unsigned>(plan.nsplit));
      plane_rel_sweep_kernel<kPlaneThreads, kPlaneTpt, kPlaneTile, kPlaneMinB><<<grid, kPlaneThreads, 0, job.stream>>>(a);
      finish_plane_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, plan.nsplit, job.nt, job.out0,
                                                           job.out1);
      break;
    }
    case kSumPseK8Geo:
    case kSumPseGaussChord:
    case kSumPseK8Chord: {
      const double e4 = (job.eps * job.eps) * (job.eps * job.eps);
      const double cscale = (job.kind == kSumPseGaussChord ? 4.0 : 1.0) / kPi / e4;
      if (job.z && (job.kind == kSumPseK8Geo || job.kind == kSumPseGaussChord)) {
        // sphere: group-relative sweep with the r^2 >= 49 group cutoff (pse_rel.cuh)
        LPM_TRY(launch_pse_rel(job, plan, npad));
      } else {
        // plane: the 2-D group-relative sweep with the same cutoff (plane_rel.cuh)
        LPM_TRY(launch_plane_pse_rel(job, plan, npad));
      }
      finish_scalar_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, plan.nsplit, job.nt, cscale, job.out0);
      break;
    }
    case kSumPseGrad:
    case kSumPseDiv: {
      LPM_TRY(launch_pse_rel(job, plan, npad));
      const double scale = job.radius / (kPi * (job.eps * job.eps) * (job.eps * job.eps));
      if (job.kind == kSumPseGrad) {
        pse_grad_finish_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, plan.nsplit, job.nt, job.ib, job.x, job.y,
                                                                job.z, scale, job.out0, job.out1, job.out2);
      } else {
        finish_scalar_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, plan.nsplit, job.nt, scale, job.out0);
      }
      break;
    }
    case kSumSphereStream: {
      const double inv_a = 1.0 / job.radius;
      const int32_t* src_list = job.src_idx;
      if (job.sort_scratch) {
        LPM_TRY(curve_sort(job.stream, job.ns, job.src_idx, job.x, job.y, job.z, inv_a, job.sort_scratch,
                           job.sort_bytes, job.sorted));
        src_list = job.sorted;
      }
      // layout of src_buf: records, group origins, the sources' own zeta A (2 x nt), totals
      char* base = static_cast<char*>(job.src_buf);
      StreamRel::Rec* recs = reinterpret_cast<StreamRel::Rec*>(base);
      const size_t org_off = align_up(static_cast<size_t>(npad) * sizeof(StreamRel::Rec), 256);
      BveRel::Origin* org = reinterpret_cast<BveRel::Origin*>(base + org_off);
      const size_t self_off = align_up(
          org_off + static_cast<size_t>(plan.n_tiles) * (kStreamTile / BveRel::kGroup) * sizeof(BveRel::Origin), 256);
      double* self_w = reinterpret_cast<double*>(base + self_off);
      double* tot =
          reinterpret_cast<double*>(base + self_off + align_up(2 * static_cast<size_t>(job.nt) * sizeof(double), 256));
      LPM_CUDA_TRY(cudaMemsetAsync(self_w, 0, 2 * static_cast<size_t>(job.nt) * sizeof(double), job.stream));
      stream_rel_prep_kernel<kStreamTile><<<static_cast<unsigned>(plan.n_tiles), kStreamTile, 0, job.stream>>>(
          job.x, job.y, job.z, job.s1, job.s2, job.area, src_list, job.ns, inv_a, job.ib, job.nt, recs, org, self_w);
      stream_totals_kernel<<<1, 1024, 0, job.stream>>>(job.s1, job.s2, job.area, job.src_idx, job.ns, tot);
      SweepArgs<BveF32> a;
      a.p = BveF32::Params{job.x, job.y, job.z, inv_a};
      a.src = nullptr;
      a.n_tiles = plan.n_tiles;
      a.tiles_per_chunk = plan.tiles_per_chunk;
      a.ib = job.ib;
      a.nt = job.nt;
      a.partial = job.partial;
      a.status = job.status;
      const dim3 grid(static_cast<unsigned>(ceil_div(job.nt, kStreamThreads * kStreamTpt)),
                      static_cast<unsigned>(plan.nsplit));
      stream_rel_sweep_kernel<kStreamThreads, kStreamTpt, kStreamTile, kStreamMinB>
          <<<grid, kStreamThreads, 0, job.stream>>>(a, recs, org);
      // a^2 - x_i.x_j = (a^2 / 2) q_ij: the constant term is -ln(a^2 / 2) / (4 pi) per zeta A
      const double k_const = -std::log(0.5 * job.radius * job.radius) * kInv4Pi;
      finish_stream_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, plan.nsplit, job.nt, 2, k_const, tot, self_w,
                                                            job.out0, job.out1);
      break;
    }
    case kSumPlaneStream: {
      const int32_t* src_list = job.src_idx;
      if (job.sort_scratch) {
        LPM_TRY(curve_sort2d(job.stream, job.ns, job.src_idx, job.x, job.y, job.sort_scratch, job.sort_bytes,
                             job.sorted));
        src_list = job.sorted;
      }
      PlaneRel::Rec* recs = static_cast<PlaneRel::Rec*>(job.src_buf);
      PlaneRel::Origin* org = reinterpret_cast<PlaneRel::Origin*>(
          static_cast<char*>(job.src_buf) + align_up(static_cast<size_t>(npad) * sizeof(PlaneRel::Rec), 256));
      plane_rel_prep_kernel<kStreamTile><<<static_cast<unsigned>(plan.n_tiles), kStreamTile, 0, job.stream>>>(
          job.x, job.y, job.s1, job.area, src_list, job.ns, kInv4Pi, recs, org);
      PlaneRelArgs a;
      a.x = job.x;
      a.y = job.y;
      a.d2 = 0.f;
      a.src = recs;
      a.org = org;
      a.n_tiles = plan.n_tiles;
      a.tiles_per_chunk = plan.tiles_per_chunk;
      a.ib = job.ib;
      a.nt = job.nt;
      a.partial = job.partial;
      a.status = job.status;
      const dim3 grid(static_cast<unsigned>(ceil_div(job.nt, kStreamThreads * kStreamTpt)),
                      static_cast<unsigned>(plan.nsplit));
      plane_stream_rel_sweep_kernel<kStreamThreads, kStreamTpt, kStreamTile, kStreamMinB>
          <<<grid, kStreamThreads, 0, job.stream>>>(a);
      finish_stream_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, plan.nsplit, job.nt, 1, 0.0, nullptr, nullptr,
                                                            job.out0, nullptr);
      break;
    }
    case kSumBetaPlane: {
      const int32_t* src_list = job.src_idx;
      if (job.sort_scratch) {
        LPM_TRY(curve_sort2d(job.stream, job.ns, job.src_idx, job.x, job.y, job.sort_scratch, job.sort_bytes,
                             job.sorted));
        src_list = job.sorted;
      }
      BetaRel::Rec* recs = static_cast<BetaRel::Rec*>(job.src_buf);
      BetaRel::Origin* org = reinterpret_cast<BetaRel::Origin*>(
          static_cast<char*>(job.src_buf) + align_up(static_cast<size_t>(npad) * sizeof(BetaRel::Rec), 256));
      beta_rel_prep_kernel<kBetaTile><<<static_cast<unsigned>(plan.n_tiles), kBetaTile, 0, job.stream>>>(
          job.x, job.y, job.s1, job.area, src_list, job.ns, recs, org);
      BetaRelArgs a;
      a.x = job.x;
      a.y = job.y;
      a.src = recs;
      a.org = org;
      a.n_tiles = plan.n_tiles;
      a.tiles_per_chunk = plan.tiles_per_chunk;
      a.ib = job.ib;
      a.nt = job.nt;
      a.partial = job.partial;
      a.status = job.status;
      const dim3 grid(static_cast<unsigned>(ceil_div(job.nt, kBetaThreads * kBetaTpt)),
                      static_cast<unsigned>(plan.nsplit));
      beta_rel_sweep_kernel<kBetaThreads, kBetaTpt, kBetaTile, kBetaMinB><<<grid, kBetaThreads, 0, job.stream>>>(a);
      finish_stream_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, plan.nsplit, job.nt, 2, 0.0, nullptr, nullptr,
                                                            job.out0, job.out1);
      break;
    }
    case kSumSweSphere: {
      const double inv_a = 1.0 / job.radius;
      const int32_t* src_list = job.src_idx;
      if (job.sort_scratch) {
        LPM_TRY(curve_sort(job.stream, job.ns, job.src_idx, job.x, job.y, job.z, inv_a, job.sort_scratch,
                            job.sort_bytes, job.sorted));
        src_list = job.sorted;
      }
      // velocity: S_r = -zeta A / (2 pi a^2), S_p = div A / (2 pi a^2) on the two-strength layout
      StreamRel::Rec* recs = static_cast<StreamRel::Rec*>(job.src_buf);
      BveRel::Origin* org = reinterpret_cast<BveRel::Origin*>(
          static_cast<char*>(job.src_buf) + align_up(static_cast<size_t>(npad) * sizeof(StreamRel::Rec), 256));
      const double k2 = 1.0 / (2.0 * kPi * job.radius * job.radius);
      stream_rel_prep_kernel<kStreamTile><<<static_cast<unsigned>(plan.n_tiles), kStreamTile, 0, job.stream>>>(
          job.x, job.y, job.z, job.s1, job.s2, job.area, src_list, job.ns, inv_a, job.ib, job.nt, recs, org, nullptr,
          -k2, k2);
      SweepArgs<BveF32> a;
      a.p = BveF32::Params{job.x, job.y, job.z, inv_a};
      a.n_tiles = plan.n_tiles;
      a.tiles_per_chunk = plan.tiles_per_chunk;
      a.ib = job.ib;
      a.nt = job.nt;
      a.partial = job.partial;
      a.status = job.status;
      const dim3 grid(static_cast<unsigned>(ceil_div(job.nt, kStreamThreads * kStreamTpt)),
                      static_cast<unsigned>(plan.nsplit));
      sphere_swe_rel_sweep_kernel<kStreamThreads, kStreamTpt, kStreamTile, kSweSphereMinB>
          <<<grid, kStreamThreads, 0, job.stream>>>(a, recs, org);
      swe_sphere_finish_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, plan.nsplit, job.nt, job.ib, job.x, job.y,
                                                                job.z, inv_a, job.out0, job.out1, job.out2);
      // surface-height Laplacian: K8(SphereDistance / eps) / eps**2 with SphereDistance scaled by
      // radius2, i.e. the geodesic PSE sweep at eps' = eps a / radius2 on the sphere of radius a
      SumJob jp = job;
      jp.kind = kSumPseK8Geo;
      jp.s1 = job.s3;
      jp.src_idx = src_list;
      jp.sort_scratch = nullptr;
      jp.eps = job.eps * job.radius / job.radius2;
      jp.src_buf = static_cast<char*>(job.src_buf) + plan.aux_src_offset;
      SumPlan pp;
      pp.n_tiles = plan.aux_n_tiles;
      pp.tiles_per_chunk = plan.aux_tiles_per_chunk;
      pp.nsplit = plan.aux_nsplit;
      LPM_TRY(launch_pse_rel(jp, pp, plan.aux_n_tiles * kPseTile));
      finish_scalar_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, pp.nsplit, job.nt,
                                                            1.0 / (kPi * job.eps * job.eps), job.out3);
      break;
    }
    case kSumBetaStream: {
      const int32_t* src_list = job.src_idx;
      if (job.sort_scratch) {
        LPM_TRY(curve_sort2d(job.stream, job.ns, job.src_idx, job.x, job.y, job.sort_scratch, job.sort_bytes,
                             job.sorted));
        src_list = job.sorted;
      }
      BetaStreamRel::Rec* recs = static_cast<BetaStreamRel::Rec*>(job.src_buf);
      BetaStreamRel::Origin* org = reinterpret_cast<BetaStreamRel::Origin*>(
          static_cast<char*>(job.src_buf) + align_up(static_cast<size_t>(npad) * sizeof(BetaStreamRel::Rec), 256));
      beta_stream_rel_prep_kernel<kBetaTile><<<static_cast<unsigned>(plan.n_tiles), kBetaTile, 0, job.stream>>>(
          job.x, job.y, job.s1, job.s2, job.area, src_list, job.ns, recs, org);
      BetaStreamRelArgs a;
      a.x = job.x;
      a.y = job.y;
      a.src = recs;
      a.org = org;
      a.n_tiles = plan.n_tiles;
      a.tiles_per_chunk = plan.tiles_per_chunk;
      a.ib = job.ib;
      a.nt = job.nt;
      a.partial = job.partial;
      a.status = job.status;
      const dim3 grid(static_cast<unsigned>(ceil_div(job.nt, kBetaThreads * kBetaTpt)),
                      static_cast<unsigned>(plan.nsplit));
      beta_stream_rel_sweep_kernel<kBetaThreads, kBetaTpt, kBetaTile, kBetaMinB>
          <<<grid, kBetaThreads, 0, job.stream>>>(a);
      finish_stream_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, plan.nsplit, job.nt, 2, 0.0, nullptr, nullptr,
                                                            job.out0, job.out1);
      break;
    }
    case kSumSwePlane: {
      const int32_t* src_list = job.src_idx;
      if (job.sort_scratch) {
        LPM_TRY(curve_sort2d(job.stream, job.ns, job.src_idx, job.x, job.y, job.sort_scratch, job.sort_bytes,
                             job.sorted));
        src_list = job.sorted;
      }
      // velocity and velocity gradient (W = vort A / (2 pi), D = div A / (2 pi))
      PlaneRel::Rec* recs = static_cast<PlaneRel::Rec*>(job.src_buf);
      PlaneRel::Origin* org = reinterpret_cast<PlaneRel::Origin*>(
          static_cast<char*>(job.src_buf) + align_up(static_cast<size_t>(npad) * sizeof(PlaneRel::Rec), 256));
      plane_rel_prep_kernel<kPlaneTile><<<static_cast<unsigned>(plan.n_tiles), kPlaneTile, 0, job.stream>>>(
          job.x, job.y, job.s1, job.area, src_list, job.ns, 1.0 / (2.0 * kPi), recs, org, job.s2);
      PlaneRelArgs a;
      a.x = job.x;
      a.y = job.y;
      a.d2 = 0.f;
      a.src = recs;
      a.org = org;
      a.n_tiles = plan.n_tiles;
      a.tiles_per_chunk = plan.tiles_per_chunk;
      a.ib = job.ib;
      a.nt = job.nt;
      a.partial = job.partial;
      a.status = job.status;
      const dim3 grid(static_cast<unsigned>(ceil_div(job.nt, kPseThreads * kPseTpt)),
                      static_cast<unsigned>(plan.nsplit));
      plane_swe_rel_sweep_kernel<kPseThreads, kPseTpt, kPlaneTile, kSweMinB><<<grid, kPseThreads, 0, job.stream>>>(a);
      swe_finish_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, plan.nsplit, job.nt, job.out0, job.out1,
                                                         job.out2);
      // surface-height Laplacian: the planar K8 PSE sweep on sh = s3, same source order
      SumJob jp = job;
      jp.kind = kSumPseK8Chord;
      jp.s1 = job.s3;
      jp.src_idx = src_list;
      jp.sort_scratch = nullptr;
      jp.src_buf = static_cast<char*>(job.src_buf) + plan.aux_src_offset;
      SumPlan pp;
      pp.n_tiles = plan.aux_n_tiles;
      pp.tiles_per_chunk = plan.aux_tiles_per_chunk;
      pp.nsplit = plan.aux_nsplit;
      LPM_TRY(launch_plane_pse_rel(jp, pp, plan.aux_n_tiles * kPseTile));
      const double e4 = (job.eps * job.eps) * (job.eps * job.eps);
      finish_scalar_kernel<<<fin_grid, pb, 0, job.stream>>>(job.partial, pp.nsplit, job.nt, 1.0 / kPi / e4,
                                                            job.out3);
      break;
    }
    default:
      return set_error(LPM_ERR_ARG, "sum kind %d has no FP32C form", job.kind);
  }
  LPM_CUDA_TRY(cudaGetLastError());
  return LPM_OK;
}

// ------------------------------------------------------------------ autotuner

namespace {
constexpr int64_t kTuneTargets = 256 * 1024;  // timing subset of the targets
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, int> g_tune_cache;  // (kind, log2 ns, log2 nt, SMs) -> shape

int log2_bucket(int64_t v) {
  int b = 0;
  while ((int64_t{1} << (b + 1)) <= v) ++b;
  return b;
}
}  // namespace

SumPlan plan_sum_max(int kind, int mode, int64_t ns, int64_t nt, int sm_count) {
  SumPlan best = plan_sum(kind, mode, ns, nt, sm_count, 0);
  if (mode != LPM_MODE_FP32C || (kind != kSumBve && kind != kSumBveMesh)) return best;
  const int64_t sub = nt < kTuneTargets ? nt : kTuneTargets;
  for (int sh = 0; sh < kBveShapeCount; ++sh) {
    for (const int64_t t : {nt, sub}) {
      const SumPlan p = plan_sum(kind, mode, ns, t, sm_count, sh);
      if (p.partial_bytes > best.partial_bytes) best.partial_bytes = p.partial_bytes;
      if (p.src_bytes > best.src_bytes) best.src_bytes = p.src_bytes;
    }
  }
  return best;
}

int autotune_bve_shape(const SumJob& job, int sm_count, int* shape) {
  *shape = 0;
  if (job.mode != LPM_MODE_FP32C || (job.kind != kSumBve && job.kind != kSumBveMesh) || job.ns == 0) return LPM_OK;
  const auto key = std::make_tuple(job.kind == kSumBveMesh ? static_cast<int>(kSumBve) : job.kind,
                                   log2_bucket(job.ns), log2_bucket(job.nt), sm_count);
  std::lock_guard<std::mutex> lock(g_tune_mu);
  const auto it = g_tune_cache.find(key);
  if (it != g_tune_cache.end()) {
    *shape = it->second;
    return LPM_OK;
  }
  SumJob j = job;
  if (j.nt > kTuneTargets) j.nt = kTuneTargets;
  cudaEvent_t e0, e1;
  LPM_CUDA_TRY(cudaEventCreate(&e0));
  LPM_CUDA_TRY(cudaEventCreate(&e1));
  float best_ms = 3.4e38f;
  int best = 0;
  int rc = LPM_OK;
  for (int sh = 0; sh < kBveShapeCount && rc == LPM_OK; ++sh) {
    const SumPlan p = plan_sum(j.kind, j.mode, j.ns, j.nt, sm_count, sh);
    rc = launch_sum(j, p);  // warm-up (and sort) run
    if (rc != LPM_OK) break;
    cudaEventRecord(e0, j.stream);
    rc = launch_sum(j, p);
    cudaEventRecord(e1, j.stream);
    if (rc != LPM_OK) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = set_error(LPM_ERR_CUDA, "autotune: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) {
      best_ms = ms;
      best = sh;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != LPM_OK) return rc;
  g_tune_cache[key] = best;
  *shape = best;
  return LPM_OK;
}

// ------------------------------------------------------------------ host-buffer entry points

namespace {

struct HostArgs {
  int kind;
  int64_t n;
  const double *x, *y, *z, *s1, *s2, *area;
  const int32_t* active;
  double radius, delta, eps;
  int64_t i_begin, i_end;  // 1-based inclusive
  double *out0, *out1, *out2;
  int mode;
  const double* s3 = nullptr;  // vz (PSE divergence), w (sphere double dot), surface height (SWE)
  double* out3 = nullptr;      // lapSurf (SWE)
  double radius2 = 1.0;        // SphereRadius of SphereDistance (sphere SWE)
};

int check_common(const HostArgs& a, int nout) {
  LPM_TRY(check_count(a.n));
  if (!a.x || !a.y || !a.s1 || !a.area || !a.active)
    return set_error(LPM_ERR_ARG, "null input array");
  if (!a.out0 || (nout > 1 && !a.out1) || (nout > 2 && !a.out2) || (nout > 3 && !a.out3))
    return set_error(LPM_ERR_ARG, "null output array");
  if (a.i_begin < 1 || a.i_end > a.n || a.i_begin > a.i_end)
    return set_error(LPM_ERR_ARG, "target range [%lld, %lld] is not inside [1, %lld]", (long long)a.i_begin,
                     (long long)a.i_end, (long long)a.n);
  const int prec = a.mode & LPM_MODE_MASK;
  if (prec != LPM_MODE_FP64 && prec != LPM_MODE_FP32C)
    return set_error(LPM_ERR_ARG, "unknown precision mode %d", prec);
  if ((a.mode & ~(LPM_MODE_MASK | LPM_FLAG_CHECK_FINITE)) != 0)
    return set_error(LPM_ERR_ARG, "unknown mode flags 0x%x", a.mode);
  if (prec == LPM_MODE_FP32C && sum_is_fp64_only(a.kind))
    return set_error(LPM_ERR_ARG, "this operator has only the FP64 mode (LPM_MODE_FP64)");
  return LPM_OK;
}

int run_host(const HostArgs& a, int nout) {
  Context* ctx = nullptr;
  LPM_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lock(ctx->mu);
  clear_error();
  const int prec = a.mode & LPM_MODE_MASK;
  const int64_t n = a.n;
  const int64_t ib = a.i_begin - 1;
  const int64_t nt = a.i_end - a.i_begin + 1;

  // the active list, in a host buffer the context keeps between calls (no page faults on a
  // fresh allocation per call), filled without a branch per particle
  std::vector<int32_t>& idx = ctx->h_idx;
  if (idx.size() < static_cast<size_t>(n)) idx.resize(static_cast<size_t>(n));
  int64_t ns = 0;
  for (int64_t j = 0; j < n; ++j) {
    idx[static_cast<size_t>(ns)] = static_cast<int32_t>(j);
    ns += a.active[j] != 0 ? 1 : 0;
  }

  const bool has_z = a.z != nullptr;
  const bool has_s2 = a.s2 != nullptr;
  const bool has_s3 = a.s3 != nullptr;
  const int narr = 4 + (has_z ? 1 : 0) + (has_s2 ? 1 : 0) + (has_s3 ? 1 : 0);  // x, y, s1, area (+z, s2, s3)
  void* p_in = nullptr;
  LPM_TRY(workspace(ctx, kWsTargets, static_cast<size_t>(narr) * n * sizeof(double), &p_in));
  double* d = static_cast<double*>(p_in);
  double* dx = d;
  double* dy = d + n;
  double* ds1 = d + 2 * n;
  double* darea = d + 3 * n;
  double* dz = has_z ? d + 4 * n : nullptr;
  double* ds2 = has_s2 ? d + (4 + (has_z ? 1 : 0)) * n : nullptr;
  double* ds3 = has_s3 ? d + (4 + (has_z ? 1 : 0) + (has_s2 ? 1 : 0)) * n : nullptr;
  const size_t nb = static_cast<size_t>(n) * sizeof(double);
  cudaStream_t s = ctx->stream;
  LPM_CUDA_TRY(cudaMemcpyAsync(dx, a.x, nb, cudaMemcpyHostToDevice, s));
  LPM_CUDA_TRY(cudaMemcpyAsync(dy, a.y, nb, cudaMemcpyHostToDevice, s));
  LPM_CUDA_TRY(cudaMemcpyAsync(ds1, a.s1, nb, cudaMemcpyHostToDevice, s));
  LPM_CUDA_TRY(cudaMemcpyAsync(darea, a.area, nb, cudaMemcpyHostToDevice, s));
  if (has_z) LPM_CUDA_TRY(cudaMemcpyAsync(dz, a.z, nb, cudaMemcpyHostToDevice, s));
  if (has_s2) LPM_CUDA_TRY(cudaMemcpyAsync(ds2, a.s2, nb, cudaMemcpyHostToDevice, s));
  if (has_s3) LPM_CUDA_TRY(cudaMemcpyAsync(ds3, a.s3, nb, cudaMemcpyHostToDevice, s));

  void* p_out = nullptr;
  LPM_TRY(workspace(ctx, kWsOutput, static_cast<size_t>(nout) * nt * sizeof(double), &p_out));
  double* dout = static_cast<double*>(p_out);

  if (ns == 0) {
    LPM_CUDA_TRY(cudaMemsetAsync(dout, 0, static_cast<size_t>(nout) * nt * sizeof(double), s));
  } else {
    void* p_idx = nullptr;
    LPM_TRY(workspace(ctx, kWsActive, static_cast<size_t>(ns) * sizeof(int32_t), &p_idx));
    LPM_CUDA_TRY(cudaMemcpyAsync(p_idx, idx.data(), static_cast<size_t>(ns) * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, s));
    SumPlan plan = plan_sum_max(a.kind, prec, ns, nt, ctx->sm_count);
    SumJob job;
    job.kind = a.kind;
    job.mode = prec;
    job.n = n;
    job.x = dx;
    job.y = dy;
    job.z = dz;
    job.s1 = ds1;
    job.s2 = ds2;
    job.s3 = ds3;
    job.area = darea;
    job.src_idx = static_cast<const int32_t*>(p_idx);
    job.ns = ns;
    job.radius = a.radius;
    job.delta = a.delta;
    job.eps = a.eps;
    job.radius2 = a.radius2;
    job.ib = ib;
    job.nt = nt;
    job.out0 = dout;
    job.out1 = nout > 1 ? dout + nt : nullptr;
    job.out2 = nout > 2 ? dout + 2 * nt : nullptr;
    job.out3 = nout > 3 ? dout + 3 * nt : nullptr;
    LPM_TRY(workspace(ctx, kWsSources, plan.src_bytes, &job.src_buf));
    int unit = 0;
    if (sum_uses_sorted_sources(a.kind, prec) || (prec == LPM_MODE_FP64 && fp64_cutoff(a.kind, &unit))) {
      void* ps = nullptr;
      const size_t sb = sort_scratch_bytes(a.kind, ns, nt);
      const size_t sorted_off = align_up(sb, 256);
      LPM_TRY(workspace(ctx, kWsScan, sorted_off + static_cast<size_t>(ns) * sizeof(int32_t), &ps));
      job.sort_scratch = ps;
      job.sort_bytes = sb;
      job.sorted = reinterpret_cast<int32_t*>(static_cast<char*>(ps) + sorted_off);
    }
    if (plan.partial_bytes) {
      void* pp = nullptr;
      LPM_TRY(workspace(ctx, kWsPartial, plan.partial_bytes, &pp));
      job.partial = static_cast<double*>(pp);
    }
    job.status = ctx->d_status;
    job.stream = s;
    int shape = 0;
    LPM_TRY(autotune_bve_shape(job, ctx->sm_count, &shape));
    plan = plan_sum(a.kind, prec, ns, nt, ctx->sm_count, shape);
    if (prec == LPM_MODE_FP32C && (a.kind == kSumBve || a.kind == kSumBveMesh || a.kind == kSumPseK8Geo ||
                                   (a.kind == kSumPseGaussChord && job.z) || a.kind == kSumPseGrad ||
                                   a.kind == kSumPseDiv))
      job.wait = take_injected_wait();
    LPM_TRY(launch_sum(job, plan));
  }
  // the caller's outputs are written only when every bounded wait of the sum succeeded
  LPM_TRY(sync_and_check(ctx, "direct sum"));
  double* outs[4] = {a.out0, a.out1, a.out2, a.out3};
  for (int c = 0; c < nout; ++c) {
    LPM_CUDA_TRY(cudaMemcpyAsync(outs[c] + ib, dout + c * nt, static_cast<size_t>(nt) * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
  }
  LPM_CUDA_TRY(cudaStreamSynchronize(s));
  if (a.mode & LPM_FLAG_CHECK_FINITE) {
    for (int c = 0; c < nout; ++c) {
      for (int64_t i = ib; i < ib + nt; ++i) {
        if (!std::isfinite(outs[c][i])) {
          return set_error(LPM_ERR_NONFINITE, "non-finite output %d at particle %lld", c, (long long)(i + 1));
        }
      }
    }
  }
  return LPM_OK;
}

}  // namespace
}  // namespace lpm

using lpm::HostArgs;

extern "C" int lpm_bve_velocity(int64_t n, const double* x, const double* y, const double* z,
                                const double* zeta, const double* area, const int32_t* active,
                                double radius, int64_t i_begin, int64_t i_end, double* u, double* v,
                                double* w, int mode) {
  HostArgs a{lpm::kSumBve, n, x, y, z, zeta, nullptr, area, active, radius, 0.0, 0.0, i_begin, i_end, u, v, w, mode};
  LPM_TRY(lpm::check_common(a, 3));
  if (!z) return lpm::set_error(LPM_ERR_ARG, "null z array");
  if (!(radius > 0.0)) return lpm::set_error(LPM_ERR_ARG, "radius must be positive");
  return lpm::run_host(a, 3);
}

extern "C" int lpm_bve_set_velocity_from_vorticity(int64_t n, const double* x, const double* y,
                                                   const double* z, const double* zeta, const double* area,
                                                   const int32_t* active, double radius, int64_t i_begin,
                                                   int64_t i_end, double* u, double* v, double* w, int mode) {
  HostArgs a{lpm::kSumBveMesh, n, x, y, z, zeta, nullptr, area, active, radius, 0.0, 0.0, i_begin, i_end, u, v, w, mode};
  LPM_TRY(lpm::check_common(a, 3));
  if (!z) return lpm::set_error(LPM_ERR_ARG, "null z array");
  if (!(radius > 0.0)) return lpm::set_error(LPM_ERR_ARG, "radius must be positive");
  return lpm::run_host(a, 3);
}

extern "C" int lpm_plane_velocity(int64_t n, const double* x, const double* y, const double* omega,
                                  const double* area, const int32_t* active, double delta, int64_t i_begin,
                                  int64_t i_end, double* u, double* v, int mode) {
  HostArgs a{lpm::kSumPlane, n, x, y, nullptr, omega, nullptr, area, active, 1.0, delta, 0.0, i_begin, i_end, u, v, nullptr, mode};
  LPM_TRY(lpm::check_common(a, 2));
  if (!(delta >= 0.0)) return lpm::set_error(LPM_ERR_ARG, "delta must be >= 0");
  return lpm::run_host(a, 2);
}

extern "C" int lpm_pse_sphere_laplacian(int64_t n, const double* x, const double* y, const double* z,
                                        const double* f, const double* area, const int32_t* active, double eps,
                                        double radius, int kernel, int64_t i_begin, int64_t i_end, double* lap,
                                        int mode) {
  int kind;
  if (kernel == LPM_PSE_K8_GEODESIC) kind = lpm::kSumPseK8Geo;
  else if (kernel == LPM_PSE_GAUSS_CHORD) kind = lpm::kSumPseGaussChord;
  else return lpm::set_error(LPM_ERR_ARG, "unknown sphere PSE kernel %d", kernel);
  HostArgs a{kind, n, x, y, z, f, nullptr, area, active, radius, 0.0, eps, i_begin, i_end, lap, nullptr, nullptr, mode};
  LPM_TRY(lpm::check_common(a, 1));
  if (!z) return lpm::set_error(LPM_ERR_ARG, "null z array");
  if (!(eps > 0.0) || !(radius > 0.0)) return lpm::set_error(LPM_ERR_ARG, "eps and radius must be positive");
  return lpm::run_host(a, 1);
}

extern "C" int lpm_pse_plane_laplacian(int64_t n, const double* x, const double* y, const double* f,
                                       const double* area, const int32_t* active, double eps, int kernel,
                                       int64_t i_begin, int64_t i_end, double* lap, int mode) {
  int kind;
  if (kernel == LPM_PSE_K8_CHORD) kind = lpm::kSumPseK8Chord;
  else if (kernel == LPM_PSE_GAUSS_CHORD) kind = lpm::kSumPseGaussChord;
  else return lpm::set_error(LPM_ERR_ARG, "unknown plane PSE kernel %d", kernel);
  HostArgs a{kind, n, x, y, nullptr, f, nullptr, area, active, 1.0, 0.0, eps, i_begin, i_end, lap, nullptr, nullptr, mode};
  LPM_TRY(lpm::check_common(a, 1));
  if (!(eps > 0.0)) return lpm::set_error(LPM_ERR_ARG, "eps must be positive");
  return lpm::run_host(a, 1);
}

extern "C" int lpm_bve_stream_functions(int64_t n, const double* x, const double* y, const double* z,
                                        const double* relvort, const double* absvort, const double* area,
                                        const int32_t* active, double radius, int64_t i_begin, int64_t i_end,
                                        double* psi_rel, double* psi_abs, int mode) {
  HostArgs a{lpm::kSumSphereStream, n, x, y, z, relvort, absvort, area, active, radius, 0.0, 0.0,
             i_begin, i_end, psi_rel, psi_abs, nullptr, mode};
  LPM_TRY(lpm::check_common(a, 2));
  if (!z || !absvort) return lpm::set_error(LPM_ERR_ARG, "null z or absvort array");
  if (!(radius > 0.0)) return lpm::set_error(LPM_ERR_ARG, "radius must be positive");
  return lpm::run_host(a, 2);
}

extern "C" int lpm_plane_stream_function(int64_t n, const double* x, const double* y, const double* omega,
                                         const double* area, const int32_t* active, int64_t i_begin,
                                         int64_t i_end, double* psi, int mode) {
  HostArgs a{lpm::kSumPlaneStream, n, x, y, nullptr, omega, nullptr, area, active, 1.0, 0.0, 0.0,
             i_begin, i_end, psi, nullptr, nullptr, mode};
  LPM_TRY(lpm::check_common(a, 1));
  return lpm::run_host(a, 1);
}

extern "C" int lpm_pse_sphere_gradient(int64_t n, const double* x, const double* y, const double* z, const double* f,
                                       const double* area, const int32_t* active, double eps, double radius,
                                       int64_t i_begin, int64_t i_end, double* gx, double* gy, double* gz, int mode) {
  HostArgs a{lpm::kSumPseGrad, n, x, y, z, f, nullptr, area, active, radius, 0.0, eps, i_begin, i_end, gx, gy, gz, mode};
  LPM_TRY(lpm::check_common(a, 3));
  if (!z) return lpm::set_error(LPM_ERR_ARG, "null z array");
  if (!(eps > 0.0) || !(radius > 0.0)) return lpm::set_error(LPM_ERR_ARG, "eps and radius must be positive");
  return lpm::run_host(a, 3);
}

extern "C" int lpm_pse_sphere_divergence(int64_t n, const double* x, const double* y, const double* z,
                                         const double* vx, const double* vy, const double* vz, const double* area,
                                         const int32_t* active, double eps, double radius, int64_t i_begin,
                                         int64_t i_end, double* div, int mode) {
  HostArgs a{lpm::kSumPseDiv, n, x, y, z, vx, vy, area, active, radius, 0.0, eps, i_begin, i_end, div, nullptr,
             nullptr, mode, vz};
  LPM_TRY(lpm::check_common(a, 1));
  if (!z || !vy || !vz) return lpm::set_error(LPM_ERR_ARG, "null z or vector component array");
  if (!(eps > 0.0) || !(radius > 0.0)) return lpm::set_error(LPM_ERR_ARG, "eps and radius must be positive");
  return lpm::run_host(a, 1);
}

extern "C" int lpm_pse_plane_gradient(int64_t n, const double* x, const double* y, const double* f, const double* area,
                                      const int32_t* active, double eps, int64_t i_begin, int64_t i_end, double* gx,
                                      double* gy, int mode) {
  HostArgs a{lpm::kSumPsePlaneGrad, n, x, y, nullptr, f, nullptr, area, active, 1.0, 0.0, eps, i_begin, i_end, gx, gy,
             nullptr, mode};
  LPM_TRY(lpm::check_common(a, 2));
  if (!(eps > 0.0)) return lpm::set_error(LPM_ERR_ARG, "eps must be positive");
  return lpm::run_host(a, 2);
}

extern "C" int lpm_pse_plane_second_partials(int64_t n, const double* x, const double* y, const double* gx,
                                             const double* gy, const double* area, const int32_t* active, double eps,
                                             int64_t i_begin, int64_t i_end, double* dxx, double* dxy, double* dyy,
                                             int mode) {
  HostArgs a{lpm::kSumPsePlaneSecond, n, x, y, nullptr, gx, gy, area, active, 1.0, 0.0, eps, i_begin, i_end, dxx,
             dxy, dyy, mode};
  LPM_TRY(lpm::check_common(a, 3));
  if (!gy) return lpm::set_error(LPM_ERR_ARG, "null gradient component array");
  if (!(eps > 0.0)) return lpm::set_error(LPM_ERR_ARG, "eps must be positive");
  return lpm::run_host(a, 3);
}

extern "C" int lpm_pse_plane_double_dot(int64_t n, const double* x, const double* y, const double* u, const double* v,
                                        const double* area, const int32_t* active, double eps, int64_t i_begin,
                                        int64_t i_end, double* ddot, int mode) {
  HostArgs a{lpm::kSumPsePlaneDdot, n, x, y, nullptr, u, v, area, active, 1.0, 0.0, eps, i_begin, i_end, ddot, nullptr,
             nullptr, mode};
  LPM_TRY(lpm::check_common(a, 1));
  if (!v) return lpm::set_error(LPM_ERR_ARG, "null velocity component array");
  if (!(eps > 0.0)) return lpm::set_error(LPM_ERR_ARG, "eps must be positive");
  return lpm::run_host(a, 1);
}

extern "C" int lpm_pse_sphere_double_dot(int64_t n, const double* x, const double* y, const double* z, const double* u,
                                         const double* v, const double* w, const double* area, const int32_t* active,
                                         double eps, double radius, int64_t i_begin, int64_t i_end, double* ddot,
                                         int mode) {
  HostArgs a{lpm::kSumPseSphereDdot, n, x, y, z, u, v, area, active, radius, 0.0, eps, i_begin, i_end, ddot, nullptr,
             nullptr, mode, w};
  LPM_TRY(lpm::check_common(a, 1));
  if (!z || !v || !w) return lpm::set_error(LPM_ERR_ARG, "null z or velocity component array");
  if (!(eps > 0.0) || !(radius > 0.0)) return lpm::set_error(LPM_ERR_ARG, "eps and radius must be positive");
  return lpm::run_host(a, 1);
}

extern "C" int lpm_pse_interpolate_scalar(int64_t n, const double* x, const double* y, const double* z, const double* f,
                                          const double* area, const int32_t* active, double eps, double radius,
                                          int geometry, int64_t m, const double* qx, const double* qy,
                                          const double* qz, double* out, int mode) {
  if (m <= 0 || !qx || !qy || !out) return lpm::set_error(LPM_ERR_ARG, "need m > 0 query points and an output array");
  if (geometry != LPM_GEOMETRY_PLANE && geometry != LPM_GEOMETRY_SPHERE)
    return lpm::set_error(LPM_ERR_ARG, "unknown geometry %d", geometry);
  if (geometry == LPM_GEOMETRY_SPHERE && (!z || !qz))
    return lpm::set_error(LPM_ERR_ARG, "the sphere needs z and qz");
  if (!(eps > 0.0) || !(radius > 0.0)) return lpm::set_error(LPM_ERR_ARG, "eps and radius must be positive");
  LPM_TRY(lpm::check_count(n));
  if (m > lpm::kMaxParticles - n) return lpm::set_error(LPM_ERR_ARG, "n + m is above 2^31 - 1 particles");
  if (!x || !y || !f || !area || !active) return lpm::set_error(LPM_ERR_ARG, "null input array");
  // The query points become passive particles n .. n+m-1 (area 0, inactive), the targets.
  const int64_t nn = n + m;
  std::vector<double> cx(nn), cy(nn), cz(nn), cf(nn, 0.0), ca(nn, 0.0), co(nn, 0.0);
  std::vector<int32_t> act(nn, 0);
  for (int64_t i = 0; i < n; ++i) {
    cx[i] = x[i];
    cy[i] = y[i];
    cz[i] = z ? z[i] : 0.0;
    cf[i] = f[i];
    ca[i] = area[i];
    act[i] = active[i] ? 1 : 0;
  }
  for (int64_t k = 0; k < m; ++k) {
    cx[n + k] = qx[k];
    cy[n + k] = qy[k];
    cz[n + k] = qz ? qz[k] : 0.0;
  }
  const int kind = geometry == LPM_GEOMETRY_SPHERE ? lpm::kSumPseInterpSphere : lpm::kSumPseInterpPlane;
  HostArgs a{kind, nn, cx.data(), cy.data(), cz.data(), cf.data(), nullptr, ca.data(), act.data(), radius, 0.0, eps,
             n + 1, nn, co.data(), nullptr, nullptr, mode};
  LPM_TRY(lpm::check_common(a, 1));
  LPM_TRY(lpm::run_host(a, 1));
  for (int64_t k = 0; k < m; ++k) out[k] = co[n + k];
  return LPM_OK;
}

extern "C" int lpm_swe_plane_rhs_integrals(int64_t n, const double* x, const double* y, const double* vort,
                                           const double* div, const double* surf_height, const double* area,
                                           const int32_t* active, double eps, int64_t i_begin, int64_t i_end,
                                           double* u, double* v, double* double_dot, double* lap_surf, int mode) {
  HostArgs a{lpm::kSumSwePlane, n, x, y, nullptr, vort, div, area, active, 1.0, 0.0, eps, i_begin, i_end, u, v,
             double_dot, mode, surf_height, lap_surf};
  LPM_TRY(lpm::check_common(a, 4));
  if (!div || !surf_height) return lpm::set_error(LPM_ERR_ARG, "null divergence or surface height array");
  if (!(eps > 0.0)) return lpm::set_error(LPM_ERR_ARG, "eps must be positive");
  return lpm::run_host(a, 4);
}

extern "C" int lpm_swe_sphere_rhs_integrals(int64_t n, const double* x, const double* y, const double* z,
                                            const double* relvort, const double* div, const double* surf_height,
                                            const double* area, const int32_t* active, double radius,
                                            double sphere_radius, double eps, int64_t i_begin, int64_t i_end,
                                            double* u, double* v, double* w, double* double_dot, double* lap_surf,
                                            int mode) {
  HostArgs a{lpm::kSumSweSphere, n, x, y, z, relvort, div, area, active, radius, 0.0, eps, i_begin, i_end, u, v, w,
             mode, surf_height, lap_surf, sphere_radius};
  LPM_TRY(lpm::check_common(a, 4));
  if (!z || !div || !surf_height || !double_dot)
    return lpm::set_error(LPM_ERR_ARG, "null z, divergence, surface height or doubleDot array");
  if (!(eps > 0.0) || !(radius > 0.0) || !(sphere_radius > 0.0))
    return lpm::set_error(LPM_ERR_ARG, "eps and the radii must be positive");
  LPM_TRY(lpm::run_host(a, 4));
  for (int64_t i = i_begin - 1; i < i_end; ++i) double_dot[i] = 0.0;  // never set by the reference
  return LPM_OK;
}

extern "C" int lpm_beta_plane_velocity(int64_t n, const double* x, const double* y, const double* zeta,
                                       const double* area, const int32_t* active, int64_t i_begin, int64_t i_end,
                                       double* u, double* v, int mode) {
  HostArgs a{lpm::kSumBetaPlane, n, x, y, nullptr, zeta, nullptr, area, active, 1.0, 0.0, 0.0, i_begin, i_end, u, v,
             nullptr, mode};
  LPM_TRY(lpm::check_common(a, 2));
  return lpm::run_host(a, 2);
}

extern "C" int lpm_beta_plane_stream_functions(int64_t n, const double* x, const double* y, const double* relvort,
                                               const double* absvort, const double* area, const int32_t* active,
                                               int64_t i_begin, int64_t i_end, double* psi_rel, double* psi_abs,
                                               int mode) {
  HostArgs a{lpm::kSumBetaStream, n, x, y, nullptr, relvort, absvort, area, active, 1.0, 0.0, 0.0, i_begin, i_end,
             psi_rel, psi_abs, nullptr, mode};
  LPM_TRY(lpm::check_common(a, 2));
  if (!absvort) return lpm::set_error(LPM_ERR_ARG, "null absolute vorticity array");
  return lpm::run_host(a, 2);
}
