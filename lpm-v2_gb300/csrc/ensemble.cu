// ensemble.cu -- many independent sphere-BVE instances of uneven size, advanced together.
//
// Layout in HBM: the instances' particle arrays are concatenated (instance k owns
// particles off[k] .. off[k+1]-1); each instance's active sources are compacted into its
// own tile-padded range of one packed source-record array.
//
// Sources: at the start of every velocity evaluation the active sources of all instances are
// put in Hilbert-curve order within their instance (one device sort on (instance, curve index)
// keys), and each instance's sources fill its own tile-padded range of group-relative
// records -- the layout and arithmetic of the single-instance sweep (bve_rel.cuh).
//
// Work decomposition: each velocity evaluation of all instances is a flattened list of
// work items (instance, block of targets, range of source tiles).  Source ranges are cut
// so that items cost about the same, and the items are sorted by decreasing cost.  One
// persistent launch (a few CTAs per SM) pulls items from an atomic queue; each item writes
// its own FP64 partial slot, and a finish kernel reduces the slots of a target block in a
// fixed order, so the result does not depend on which CTA ran which item.  One RK4 step of
// all instances (4 stage kernels, 4 x (sort, prep, sweep, finish)) is one CUDA graph.
//
// Autotuner: the persistent kernel comes in the CTA shapes the single-instance tuner picks
// from (128 threads x 4 targets at 4 CTAs per SM: 512 targets per item; 128 x 8 at 2 per SM:
// 1024), and the source ranges are cut for about 4, 8 or 16 items per resident CTA (fewer,
// longer items cost less per item; more, shorter ones leave a shorter tail).  At creation
// the work queue of each of the six choices is built and one velocity evaluation of all
// instances is timed; the fastest is kept for the ensemble's life.
//
// FP64 mode (parity) runs the bit-exact sequential sweep per instance instead.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "bve_rel.cuh"
#include "lpm_common.cuh"
#include "solver.cuh"
#include "sort.cuh"
#include "sums.cuh"

namespace lpm {
namespace {

constexpr int kTile = 256;
// CTA shapes of the persistent sweep: threads, targets per thread, CTAs per SM
struct EnsShape {
  int threads, tpt, minb;
};
constexpr EnsShape kEnsShapes[] = {{128, 4, 4}, {128, 8, 2}};
constexpr double kPi = 3.1415926535897932384626433832795027975;
constexpr int kStage = 256;

struct Item {
  int inst;
  int nt;         // targets in this item (<= the shape's targets per item)
  long long t0;   // first target (global particle index)
  long long tile0;  // first source tile (global tile index)
  int ntiles;
  int pad;
  long long slot;  // partial slot (item id in block order)
};

// Queue choices of the autotuner: (sweep shape, items per resident CTA slot).
struct QueueChoice {
  int shape, per_slot;
};
constexpr QueueChoice kQueueChoices[] = {{0, 4}, {0, 8}, {0, 16}, {1, 4}, {1, 8}, {1, 16}};
constexpr int kQueueChoiceCount = sizeof(kQueueChoices) / sizeof(kQueueChoices[0]);

// The flattened work queue of one sweep shape, on the host.
struct Queue {
  std::vector<Item> items;
  std::vector<int> order;  // items by decreasing cost
  std::vector<int32_t> boff, bfirst, bcnt;
  int grid = 0;
};

struct EnsArgs {
  const Item* items;
  const int* queue;
  int n_items;
  int* head;
  const BveRel::Rec* src;
  const BveRel::Origin* org;
  const double *x, *y, *z;
  const double* inv_a;  // per instance
  double* partial;      // [slot][3][targets per item]
  int* status;
};

template <int THREADS, int TPT, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) ensemble_sweep_kernel(EnsArgs a) {
  constexpr int NP = TPT / 2;
  constexpr int TB = THREADS * TPT;  // targets per item
  constexpr int GPT = kTile / BveRel::kGroup;
  using Rec = BveRel::Rec;
  __shared__ __align__(128) Rec stage[2][kTile];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ int s_item;
  pipe_init(bars);
  uint32_t g = 0;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.head, 1);
    __syncthreads();
    const int q = s_item;
    __syncthreads();
    if (q >= a.n_items) break;
    const Item it = a.items[a.queue[q]];
    const BveF32::Params prm{a.x, a.y, a.z, a.inv_a[it.inst]};
    BveX2::Pair pr[NP];
    float2 hx[NP], hy[NP], hz[NP], lx[NP], ly[NP], lz[NP];
    bve_load_pairs<NP>(prm, it.t0, it.nt, THREADS, pr);
#pragma unroll
    for (int p = 0; p < NP; ++p) hx[p] = hy[p] = hz[p] = lx[p] = ly[p] = lz[p] = make_float2(0.f, 0.f);
    int64_t tile = it.tile0;
    const bool ok = staged_sweep<Rec, kTile>(a.src, it.tile0, it.ntiles, stage[0], stage[1], bars, g, a.status,
                                             [&](const Rec* tl) {
      float2 ax[NP], ay[NP], az[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) ax[p] = ay[p] = az[p] = make_float2(0.f, 0.f);
      bve_rel_tile<NP, kTile, (NP >= 4 ? 4 : 2)>(tl, a.org + tile * GPT, pr, ax, ay, az);  // no spills at 128 x 4
      ++tile;
      bve_merge_pairs<NP>(ax, ay, az, hx, hy, hz, lx, ly, lz);
    });
    if (!ok) break;
    double* slot = a.partial + it.slot * 3 * TB;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int l = (2 * p + h) * THREADS + threadIdx.x;
        if (l < it.nt) {
          slot[0 * TB + l] = static_cast<double>(h ? hx[p].y : hx[p].x) + static_cast<double>(h ? lx[p].y : lx[p].x);
          slot[1 * TB + l] = static_cast<double>(h ? hy[p].y : hy[p].x) + static_cast<double>(h ? ly[p].y : ly[p].x);
          slot[2 * TB + l] = static_cast<double>(h ? hz[p].y : hz[p].x) + static_cast<double>(h ? lz[p].y : lz[p].x);
        }
      }
    }
  }
}

// Group-relative records of all instances: one CTA per (global) tile.  Tile t belongs to
// instance tile_inst[t]; its sources are that instance's Hilbert-sorted sources
// sorted[src_start[k] + (t - tile_off[k]) * kTile + lane], valid below ns_k.
__global__ void __launch_bounds__(kTile) ensemble_prep_kernel(const int32_t* tile_inst, const int64_t* tile_off,
                                                              const int64_t* src_start, const int64_t* ns_k,
                                                              const int32_t* sorted, const double* x, const double* y,
                                                              const double* z, const double* zeta, const double* area,
                                                              const double* radius, BveRel::Rec* out,
                                                              BveRel::Origin* org) {
  const int64_t t = blockIdx.x;
  const int k = tile_inst[t];
  const int64_t local = (t - tile_off[k]) * kTile + threadIdx.x;
  const bool valid = local < ns_k[k];
  const int32_t j = valid ? sorted[src_start[k] + local] : 0;
  const double a = radius[k];
  bve_rel_prep_tile<kTile>(x, y, z, zeta, area, valid, j, 1.0 / a, -1.0 / (2.0 * kPi * a), out + t * kTile + threadIdx.x,
                           org + t * (kTile / BveRel::kGroup));
}

// Per target: fixed-order FP64 sum of its block's item slots (tb targets per block), then
// u = D x p.
__global__ void ensemble_finish_kernel(int64_t n, int tb, const int32_t* pinst, const int64_t* off,
                                       const int32_t* blk_off, const int32_t* blk_first, const int32_t* blk_cnt,
                                       const double* partial, const double* x, const double* y, const double* z,
                                       const double* inv_a, double* u, double* v, double* w) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = pinst[i];
  const int64_t local = i - off[k];
  const int b = blk_off[k] + static_cast<int>(local / tb);
  const int l = static_cast<int>(local % tb);
  double d0 = 0.0, d1 = 0.0, d2 = 0.0;
  for (int c = 0; c < blk_cnt[b]; ++c) {
    const double* slot = partial + static_cast<int64_t>(blk_first[b] + c) * 3 * tb;
    d0 += slot[l];
    d1 += slot[tb + l];
    d2 += slot[2 * tb + l];
  }
  const double ia = inv_a[k];
  const double px = x[i] * ia, py = y[i] * ia, pz = z[i] * ia;
  u[i] = d1 * pz - d2 * py;
  v[i] = d2 * px - d0 * pz;
  w[i] = d0 * py - d1 * px;
}

__device__ __forceinline__ void project_to(double a, double& x, double& y, double& z) {
  const double s = a / sqrt(x * x + y * y + z * z);
  x *= s;
  y *= s;
  z *= s;
}

// RK4 stages of timestepPrivate (SphereBVESolver.f90:238-329) with per-instance radius and
// rotation rate; the arithmetic and its order are those of the single-instance solver.
__global__ void ensemble_stage_kernel(int64_t n, int which, int renorm, double dt, const int32_t* pinst,
                                      const double* radius, const double* omega, double* x, double* y, double* z,
                                      double* q, const double* us, const double* vs, const double* ws, double* ax,
                                      double* ay, double* az, double* aq, double* xin, double* yin, double* zin,
                                      double* qin) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = pinst[i];
  const double a = radius[k];
  const double two_dt_omega = __dmul_rn(__dmul_rn(dt, 2.0), omega[k]);
  const double kq = -__ddiv_rn(__dmul_rn(two_dt_omega, ws[i]), a);
  const double kx = __dmul_rn(dt, us[i]);
  const double ky = __dmul_rn(dt, vs[i]);
  const double kz = __dmul_rn(dt, ws[i]);
  double px, py, pz;
  if (which == 0) {  // stage 1: k1 from the stored velocity
    ax[i] = __dadd_rn(x[i], __ddiv_rn(kx, 6.0));
    ay[i] = __dadd_rn(y[i], __ddiv_rn(ky, 6.0));
    az[i] = __dadd_rn(z[i], __ddiv_rn(kz, 6.0));
    aq[i] = __dadd_rn(q[i], __ddiv_rn(kq, 6.0));
  } else if (which < 3) {
    ax[i] = __dadd_rn(ax[i], __ddiv_rn(kx, 3.0));
    ay[i] = __dadd_rn(ay[i], __ddiv_rn(ky, 3.0));
    az[i] = __dadd_rn(az[i], __ddiv_rn(kz, 3.0));
    aq[i] = __dadd_rn(aq[i], __ddiv_rn(kq, 3.0));
  }
  if (which < 2) {
    px = __dadd_rn(x[i], __dmul_rn(0.5, kx));
    py = __dadd_rn(y[i], __dmul_rn(0.5, ky));
    pz = __dadd_rn(z[i], __dmul_rn(0.5, kz));
    qin[i] = __dadd_rn(q[i], __dmul_rn(0.5, kq));
  } else if (which == 2) {
    px = __dadd_rn(x[i], kx);
    py = __dadd_rn(y[i], ky);
    pz = __dadd_rn(z[i], kz);
    qin[i] = __dadd_rn(q[i], kq);
  } else {
    px = __dadd_rn(ax[i], __ddiv_rn(kx, 6.0));
    py = __dadd_rn(ay[i], __ddiv_rn(ky, 6.0));
    pz = __dadd_rn(az[i], __ddiv_rn(kz, 6.0));
    if (renorm) project_to(a, px, py, pz);
    x[i] = px;
    y[i] = py;
    z[i] = pz;
    q[i] = __dadd_rn(aq[i], __ddiv_rn(kq, 6.0));
    return;
  }
  if (renorm) project_to(a, px, py, pz);
  xin[i] = px;
  yin[i] = py;
  zin[i] = pz;
}

}  // namespace
}  // namespace lpm

using namespace lpm;

struct lpm_ensemble {
  Context* ctx = nullptr;
  cudaStream_t stream = nullptr;
  DeviceArena arena;
  int K = 0;
  int64_t n = 0;
  int mode = LPM_MODE_FP32C;
  std::vector<int64_t> off;  // host copy
  std::vector<int64_t> ns_k;
  double *x, *y, *z, *q, *u, *v, *w, *area;
  double *ax, *ay, *az, *aq, *xin, *yin, *zin, *qin, *us, *vs, *ws;
  int32_t* pinst = nullptr;
  int64_t* d_off = nullptr;
  double *radius = nullptr, *omega = nullptr, *inv_a = nullptr;
  // FP32C work queue
  int64_t n_tiles = 0;
  int64_t ns_total = 0;
  int32_t* act_idx = nullptr;   // active sources in instance order
  int32_t* act_grp = nullptr;   // their instance
  int32_t* sorted = nullptr;    // Hilbert-curve order within each instance
  void* sort_scratch = nullptr;
  size_t sort_bytes = 0;
  int32_t* tile_inst = nullptr;
  int64_t *d_tile_off = nullptr, *d_src_start = nullptr, *d_ns_k = nullptr;
  BveRel::Rec* rec = nullptr;
  BveRel::Origin* org = nullptr;
  Item* items = nullptr;
  int* queue = nullptr;
  int n_items = 0;
  int shape = 0;                     // kEnsShapes index of the persistent sweep
  int choice = 0;                    // kQueueChoices index in use
  std::vector<Queue> queues;         // host copies of every choice's work queue
  std::vector<float> tuned_ms;       // the chosen shape's time for one evaluation
  int* head = nullptr;
  int32_t *blk_off = nullptr, *blk_first = nullptr, *blk_cnt = nullptr;
  double* partial = nullptr;
  int grid = 0;
  // FP64 per-instance scratch
  std::vector<SumScratch> scratch64;
  std::vector<int32_t*> idx64;
  int* status = nullptr;
  int* h_status = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double graph_dt = 0.0;
  int graph_renorm = -1;
  cudaEvent_t ev[8] = {};
  double kernel_ms = 0.0;
  int64_t launches = 0;
  int64_t step_kernels = 0;  // kernel nodes of the captured step graph

  int velocity(const double* px, const double* py, const double* pz, const double* pq, double* o0, double* o1,
               double* o2, int kind = kSumBve) {
    if (mode == LPM_MODE_FP64) {
      for (int k = 0; k < K; ++k) {
        const int64_t nk = off[k + 1] - off[k];
        if (ns_k[k] == 0) {
          LPM_CUDA_TRY(cudaMemsetAsync(o0 + off[k], 0, nk * sizeof(double), stream));
          LPM_CUDA_TRY(cudaMemsetAsync(o1 + off[k], 0, nk * sizeof(double), stream));
          LPM_CUDA_TRY(cudaMemsetAsync(o2 + off[k], 0, nk * sizeof(double), stream));
          continue;
        }
        SumJob j;
        j.kind = kind;
        j.mode = LPM_MODE_FP64;
        j.n = nk;
        j.x = px + off[k];
        j.y = py + off[k];
        j.z = pz + off[k];
        j.s1 = pq + off[k];
        j.area = area + off[k];
        j.src_idx = idx64[k];
        j.ns = ns_k[k];
        j.radius = h_radius[k];
        j.ib = 0;
        j.nt = nk;
        j.out0 = o0 + off[k];
        j.out1 = o1 + off[k];
        j.out2 = o2 + off[k];
        j.src_buf = scratch64[k].src_buf;
        j.status = status;
        j.stream = stream;
        LPM_TRY(launch_sum(j, scratch64[k].plan));
      }
      return LPM_OK;
    }
    if (n_tiles > 0) {
      LPM_TRY(grouped_curve_sort(stream, ns_total, K, act_idx, act_grp, px, py, pz, inv_a, sort_scratch, sort_bytes,
                                  sorted));
      ensemble_prep_kernel<<<static_cast<unsigned>(n_tiles), kTile, 0, stream>>>(
          tile_inst, d_tile_off, d_src_start, d_ns_k, sorted, px, py, pz, pq, area, radius, rec, org);
    }
    LPM_CUDA_TRY(cudaMemsetAsync(head, 0, sizeof(int), stream));
    EnsArgs a{items, queue, n_items, head, rec, org, px, py, pz, inv_a, partial, status};
    if (shape == 0) {
      ensemble_sweep_kernel<128, 4, 4><<<grid, 128, 0, stream>>>(a);
    } else {
      ensemble_sweep_kernel<128, 8, 2><<<grid, 128, 0, stream>>>(a);
    }
    const int tb = kEnsShapes[shape].threads * kEnsShapes[shape].tpt;
    ensemble_finish_kernel<<<static_cast<unsigned>(ceil_div(n, 256)), 256, 0, stream>>>(
        n, tb, pinst, d_off, blk_off, blk_first, blk_cnt, partial, px, py, pz, inv_a, o0, o1, o2);
    LPM_CUDA_TRY(cudaGetLastError());
    return LPM_OK;
  }

  std::vector<double> h_radius, h_omega;

  int enqueue_step(double dt, int renorm) {
    const unsigned g = static_cast<unsigned>(ceil_div(n, kStage));
    ensemble_stage_kernel<<<g, kStage, 0, stream>>>(n, 0, renorm, dt, pinst, radius, omega, x, y, z, q, u, v, w, ax,
                                                    ay, az, aq, xin, yin, zin, qin);
    LPM_CUDA_TRY(cudaGetLastError());
    for (int s = 0; s < 3; ++s) {
      LPM_CUDA_TRY(cudaEventRecordWithFlags(ev[2 * s], stream, cudaEventRecordExternal));
      LPM_TRY(velocity(xin, yin, zin, qin, us, vs, ws));
      LPM_CUDA_TRY(cudaEventRecordWithFlags(ev[2 * s + 1], stream, cudaEventRecordExternal));
      ensemble_stage_kernel<<<g, kStage, 0, stream>>>(n, s + 1, renorm, dt, pinst, radius, omega, x, y, z, q, us, vs,
                                                      ws, ax, ay, az, aq, xin, yin, zin, qin);
      LPM_CUDA_TRY(cudaGetLastError());
    }
    LPM_CUDA_TRY(cudaEventRecordWithFlags(ev[6], stream, cudaEventRecordExternal));
    LPM_TRY(velocity(x, y, z, q, u, v, w));
    LPM_CUDA_TRY(cudaEventRecordWithFlags(ev[7], stream, cudaEventRecordExternal));
    return LPM_OK;
  }

  int capture(double dt, int renorm) {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    LPM_CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_step(dt, renorm);
    cudaGraph_t gr = nullptr;
    const cudaError_t e = cudaStreamEndCapture(stream, &gr);
    if (rc != LPM_OK) {
      if (gr) cudaGraphDestroy(gr);
      return rc;
    }
    if (e != cudaSuccess) return set_error(LPM_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(e));
    graph = gr;
    LPM_CUDA_TRY(cudaGraphInstantiate(&exec, graph, 0));
    step_kernels = graph_kernel_nodes(graph);
    graph_dt = dt;
    graph_renorm = renorm;
    return LPM_OK;
  }

  int check_status(const char* what) {
    LPM_CUDA_TRY(cudaMemcpyAsync(h_status, status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    const cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return set_error(LPM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    if (*h_status != kDevOk) {
      const int st = *h_status;
      LPM_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), stream));
      LPM_CUDA_TRY(cudaStreamSynchronize(stream));
      return set_error(st == kDevTimeout ? LPM_ERR_TIMEOUT : LPM_ERR_CUDA, "%s: device status %d", what, st);
    }
    return LPM_OK;
  }

  void destroy() {
    if (stream) cudaStreamSynchronize(stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (h_status) cudaFreeHost(h_status);
    arena.release();
    if (stream) cudaStreamDestroy(stream);
  }

  template <class T>
  int dev_array(T** p, size_t count) {
    void* q = nullptr;
    LPM_TRY(arena.alloc(count * sizeof(T), &q));
    *p = static_cast<T*>(q);
    return LPM_OK;
  }

  template <class T>
  int upload_vec(T** p, const std::vector<T>& h) {
    LPM_TRY(dev_array(p, h.size()));
    if (!h.empty()) LPM_CUDA_TRY(cudaMemcpyAsync(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, stream));
    return LPM_OK;
  }

  Queue make_queue(int sh, int per_slot, const std::vector<int64_t>& tile_off) const {
    const int tb = kEnsShapes[sh].threads * kEnsShapes[sh].tpt;
    Queue Q;
    // item size: aim at ~per_slot items per resident CTA slot
    double units = 0.0;
    for (int k = 0; k < K; ++k)
      units += static_cast<double>(ceil_div(off[k + 1] - off[k], tb)) * static_cast<double>(tile_off[k + 1] - tile_off[k]);
    const int slots = ctx->sm_count * kEnsShapes[sh].minb;
    const int64_t chunk_tiles =
        std::max<int64_t>(1, static_cast<int64_t>(std::ceil(units / (static_cast<double>(per_slot) * slots))));
    Q.boff.assign(K + 1, 0);
    for (int k = 0; k < K; ++k) {
      const int64_t nk = off[k + 1] - off[k];
      const int64_t tiles = tile_off[k + 1] - tile_off[k];
      const int64_t nblk = ceil_div(nk, tb);
      Q.boff[k + 1] = Q.boff[k] + static_cast<int32_t>(nblk);
      const int64_t nch = tiles > 0 ? ceil_div(tiles, chunk_tiles) : 0;
      const int64_t per = nch > 0 ? ceil_div(tiles, nch) : 0;
      for (int64_t b = 0; b < nblk; ++b) {
        Q.bfirst.push_back(static_cast<int32_t>(Q.items.size()));
        int cnt = 0;
        for (int64_t t = 0; t < tiles; t += per) {
          Item m;
          m.inst = k;
          m.t0 = off[k] + b * tb;
          m.nt = static_cast<int>(std::min<int64_t>(tb, nk - b * tb));
          m.tile0 = tile_off[k] + t;
          m.ntiles = static_cast<int>(std::min<int64_t>(per, tiles - t));
          m.pad = 0;
          m.slot = static_cast<long long>(Q.items.size());
          Q.items.push_back(m);
          ++cnt;
        }
        Q.bcnt.push_back(cnt);
      }
    }
    Q.order.resize(Q.items.size());
    std::iota(Q.order.begin(), Q.order.end(), 0);
    std::stable_sort(Q.order.begin(), Q.order.end(), [&](int p, int q) {
      return static_cast<int64_t>(Q.items[p].nt) * Q.items[p].ntiles >
             static_cast<int64_t>(Q.items[q].nt) * Q.items[q].ntiles;
    });
    Q.grid = std::max(1, std::min(static_cast<int>(Q.items.size()), slots));
    return Q;
  }

  template <class T>
  int upload_into(T* dst, const std::vector<T>& h) {
    if (!h.empty()) LPM_CUDA_TRY(cudaMemcpyAsync(dst, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, stream));
    return LPM_OK;
  }

  // Makes queue choice `ch` current: its queue into the (shared, largest-size) device buffers.
  int use_queue(int ch) {
    const Queue& Q = queues[ch];
    LPM_TRY(upload_into(items, Q.items));
    LPM_TRY(upload_into(queue, Q.order));
    LPM_TRY(upload_into(blk_off, Q.boff));
    LPM_TRY(upload_into(blk_first, Q.bfirst));
    LPM_TRY(upload_into(blk_cnt, Q.bcnt));
    n_items = static_cast<int>(Q.items.size());
    grid = Q.grid;
    shape = kQueueChoices[ch].shape;
    choice = ch;
    return LPM_OK;
  }

  // Builds the source layout and the work queues of every sweep shape (FP32C).
  int build_queue(const int32_t* active) {
    std::vector<int32_t> aidx, agrp, tinst;
    std::vector<int64_t> tile_off(K + 1, 0), src_start(K + 1, 0);
    for (int k = 0; k < K; ++k) {
      for (int64_t j = off[k]; j < off[k + 1]; ++j) {
        if (active[j]) {
          aidx.push_back(static_cast<int32_t>(j));
          agrp.push_back(k);
        }
      }
      src_start[k + 1] = static_cast<int64_t>(aidx.size());
      const int64_t tiles = ceil_div(src_start[k + 1] - src_start[k], kTile);
      tile_off[k + 1] = tile_off[k] + tiles;
      for (int64_t t = 0; t < tiles; ++t) tinst.push_back(k);
    }
    ns_total = static_cast<int64_t>(aidx.size());
    n_tiles = tile_off[K];
    size_t n_it = 1, n_blk = 1, n_part = 1;
    queues.clear();
    for (int ch = 0; ch < kQueueChoiceCount; ++ch) {
      const int sh = kQueueChoices[ch].shape;
      queues.push_back(make_queue(sh, kQueueChoices[ch].per_slot, tile_off));
      const Queue& Q = queues.back();
      const size_t tb = static_cast<size_t>(kEnsShapes[sh].threads) * kEnsShapes[sh].tpt;
      n_it = std::max(n_it, Q.items.size());
      n_blk = std::max(n_blk, Q.bcnt.size());
      n_part = std::max(n_part, Q.items.size() * 3 * tb);
    }
    LPM_TRY(upload_vec(&act_idx, aidx));
    LPM_TRY(upload_vec(&act_grp, agrp));
    LPM_TRY(upload_vec(&tile_inst, tinst));
    LPM_TRY(upload_vec(&d_tile_off, tile_off));
    LPM_TRY(upload_vec(&d_src_start, src_start));
    LPM_TRY(upload_vec(&d_ns_k, ns_k));
    LPM_TRY(dev_array(&sorted, std::max<int64_t>(ns_total, 1)));
    sort_bytes = grouped_curve_sort_bytes(std::max<int64_t>(ns_total, 1), K);
    LPM_TRY(arena.alloc(sort_bytes, &sort_scratch));
    LPM_TRY(dev_array(&rec, std::max<int64_t>(n_tiles * kTile, 1)));
    LPM_TRY(dev_array(&org, std::max<int64_t>(n_tiles * (kTile / BveRel::kGroup), 1)));
    LPM_TRY(dev_array(&items, n_it));
    LPM_TRY(dev_array(&queue, n_it));
    LPM_TRY(dev_array(&blk_off, static_cast<size_t>(K) + 1));
    LPM_TRY(dev_array(&blk_first, n_blk));
    LPM_TRY(dev_array(&blk_cnt, n_blk));
    LPM_TRY(dev_array(&head, 1));
    LPM_TRY(dev_array(&partial, n_part));
    return use_queue(0);
  }

  // Times one velocity evaluation of all instances with each queue choice (after an untimed
  // one) and keeps the fastest.  The results land in the stage-velocity scratch arrays.
  int tune_shape() {
    if (n_tiles == 0) return LPM_OK;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    LPM_CUDA_TRY(cudaEventCreate(&e0));
    LPM_CUDA_TRY(cudaEventCreate(&e1));
    int best = 0, rc = LPM_OK;
    float best_ms = 3.4e38f;
    for (int sh = 0; sh < kQueueChoiceCount && rc == LPM_OK; ++sh) {
      rc = use_queue(sh);
      if (rc == LPM_OK) rc = velocity(x, y, z, q, us, vs, ws);
      if (rc == LPM_OK && cudaEventRecord(e0, stream) != cudaSuccess) rc = set_error(LPM_ERR_CUDA, "event record");
      if (rc == LPM_OK) rc = velocity(x, y, z, q, us, vs, ws);
      if (rc == LPM_OK && cudaEventRecord(e1, stream) != cudaSuccess) rc = set_error(LPM_ERR_CUDA, "event record");
      if (rc == LPM_OK) rc = check_status("ensemble autotune");
      float ms = 0.f;
      if (rc == LPM_OK && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = set_error(LPM_ERR_CUDA, "event time");
      if (rc == LPM_OK && ms < best_ms) {
        best_ms = ms;
        best = sh;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != LPM_OK) return rc;
    tuned_ms.assign(1, best_ms);
    return use_queue(best);
  }
};

namespace {

int ens_create(lpm_ensemble* E, int K, const int64_t* offsets, const double* x, const double* y, const double* z,
               const double* q, const double* area, const int32_t* active, const double* radius,
               const double* omega, int mode) {
  LPM_TRY(get_context(&E->ctx));
  E->K = K;
  E->mode = mode;
  E->off.assign(offsets, offsets + K + 1);
  E->n = E->off[K];
  E->h_radius.assign(radius, radius + K);
  E->h_omega.assign(omega, omega + K);
  LPM_CUDA_TRY(cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking));
  const int64_t n = E->n;
  double** arrs[] = {&E->x, &E->y, &E->z, &E->q, &E->u, &E->v, &E->w, &E->area, &E->ax, &E->ay, &E->az,
                     &E->aq, &E->xin, &E->yin, &E->zin, &E->qin, &E->us, &E->vs, &E->ws};
  for (double** a : arrs) LPM_TRY(E->dev_array(a, n));
  std::vector<int32_t> pinst(n);
  E->ns_k.assign(K, 0);
  for (int k = 0; k < K; ++k) {
    for (int64_t j = E->off[k]; j < E->off[k + 1]; ++j) {
      pinst[j] = k;
      E->ns_k[k] += active[j] ? 1 : 0;
    }
  }
  std::vector<double> inv(K);
  for (int k = 0; k < K; ++k) inv[k] = 1.0 / radius[k];
  LPM_TRY(E->upload_vec(&E->pinst, pinst));
  LPM_TRY(E->upload_vec(&E->d_off, E->off));
  LPM_TRY(E->upload_vec(&E->radius, E->h_radius));
  LPM_TRY(E->upload_vec(&E->omega, E->h_omega));
  LPM_TRY(E->upload_vec(&E->inv_a, inv));
  LPM_TRY(E->dev_array(&E->status, 1));
  LPM_CUDA_TRY(cudaMemsetAsync(E->status, 0, sizeof(int), E->stream));
  LPM_CUDA_TRY(cudaMallocHost(&E->h_status, sizeof(int)));
  const size_t nb = n * sizeof(double);
  LPM_CUDA_TRY(cudaMemcpyAsync(E->x, x, nb, cudaMemcpyHostToDevice, E->stream));
  LPM_CUDA_TRY(cudaMemcpyAsync(E->y, y, nb, cudaMemcpyHostToDevice, E->stream));
  LPM_CUDA_TRY(cudaMemcpyAsync(E->z, z, nb, cudaMemcpyHostToDevice, E->stream));
  LPM_CUDA_TRY(cudaMemcpyAsync(E->q, q, nb, cudaMemcpyHostToDevice, E->stream));
  LPM_CUDA_TRY(cudaMemcpyAsync(E->area, area, nb, cudaMemcpyHostToDevice, E->stream));
  for (auto& e : E->ev) LPM_CUDA_TRY(cudaEventCreate(&e));
  if (mode == LPM_MODE_FP64) {
    E->scratch64.resize(K);
    E->idx64.assign(K, nullptr);
    for (int k = 0; k < K; ++k) {
      const int64_t nk = E->off[k + 1] - E->off[k];
      const std::vector<int32_t> idx = active_list(nk, active + E->off[k]);
      LPM_TRY(E->upload_vec(&E->idx64[k], idx));
      LPM_TRY(E->scratch64[k].init(E->arena, kSumBve, LPM_MODE_FP64, E->ns_k[k], nk, E->ctx->sm_count));
    }
  } else {
    LPM_TRY(E->build_queue(active));
    LPM_TRY(E->tune_shape());
  }
  // initial velocity: setVelocityFromVorticity (SphereBVE.f90:489-531)
  LPM_TRY(E->velocity(E->x, E->y, E->z, E->q, E->u, E->v, E->w, kSumBveMesh));
  return E->check_status("lpm_ensemble_create");
}

}  // namespace

extern "C" int lpm_ensemble_create(lpm_ensemble** out, int n_instances, const int64_t* offsets, const double* x,
                                   const double* y, const double* z, const double* relvort, const double* area,
                                   const int32_t* active, const double* radius, const double* rotation_rate,
                                   int mode) {
  if (!out) return set_error(LPM_ERR_ARG, "null ensemble handle pointer");
  *out = nullptr;
  if (n_instances <= 0 || !offsets) return set_error(LPM_ERR_ARG, "need at least one instance and offsets");
  if (!x || !y || !z || !relvort || !area || !active || !radius || !rotation_rate)
    return set_error(LPM_ERR_ARG, "null input array");
  if (mode != LPM_MODE_FP64 && mode != LPM_MODE_FP32C) return set_error(LPM_ERR_ARG, "unknown mode %d", mode);
  if (offsets[0] != 0) return set_error(LPM_ERR_ARG, "offsets[0] must be 0");
  for (int k = 0; k < n_instances; ++k) {
    if (offsets[k + 1] <= offsets[k]) return set_error(LPM_ERR_ARG, "instance %d is empty", k);
    if (!(radius[k] > 0.0)) return set_error(LPM_ERR_ARG, "instance %d radius must be positive", k);
  }
  if (offsets[n_instances] > INT32_MAX) return set_error(LPM_ERR_ARG, "too many particles");
  lpm_ensemble* E = new lpm_ensemble();
  const int rc = ens_create(E, n_instances, offsets, x, y, z, relvort, area, active, radius, rotation_rate, mode);
  if (rc != LPM_OK) {
    E->destroy();
    delete E;
    return rc;
  }
  *out = E;
  return LPM_OK;
}

extern "C" int lpm_ensemble_timestep(lpm_ensemble* E, double dt, int n_steps, int renormalize) {
  if (!E) return set_error(LPM_ERR_ARG, "null ensemble");
  if (n_steps < 0 || !std::isfinite(dt)) return set_error(LPM_ERR_ARG, "bad dt or n_steps");
  const int renorm = renormalize ? 1 : 0;
  if (!E->exec || E->graph_dt != dt || E->graph_renorm != renorm) LPM_TRY(E->capture(dt, renorm));
  for (int s = 0; s < n_steps; ++s) {
    LPM_CUDA_TRY(cudaGraphLaunch(E->exec, E->stream));
    LPM_TRY(E->check_status("lpm_ensemble_timestep"));
    for (int k = 0; k < 4; ++k) {
      float ms = 0.f;
      LPM_CUDA_TRY(cudaEventElapsedTime(&ms, E->ev[2 * k], E->ev[2 * k + 1]));
      E->kernel_ms += ms;
    }
    E->launches += E->step_kernels;
  }
  return LPM_OK;
}

extern "C" int lpm_ensemble_velocity(lpm_ensemble* E) {
  if (!E) return set_error(LPM_ERR_ARG, "null ensemble");
  LPM_TRY(E->velocity(E->x, E->y, E->z, E->q, E->u, E->v, E->w));
  return E->check_status("lpm_ensemble_velocity");
}

extern "C" int lpm_ensemble_get_state(lpm_ensemble* E, double* x, double* y, double* z, double* relvort, double* u,
                                      double* v, double* w) {
  if (!E) return set_error(LPM_ERR_ARG, "null ensemble");
  const size_t nb = E->n * sizeof(double);
  double* hs[] = {x, y, z, relvort, u, v, w};
  const double* ds[] = {E->x, E->y, E->z, E->q, E->u, E->v, E->w};
  for (int c = 0; c < 7; ++c)
    if (hs[c]) LPM_CUDA_TRY(cudaMemcpyAsync(hs[c], ds[c], nb, cudaMemcpyDeviceToHost, E->stream));
  return E->check_status("lpm_ensemble_get_state");
}

extern "C" int lpm_ensemble_kernel_timing(lpm_ensemble* E, double* total_ms, int64_t* launches) {
  if (!E) return set_error(LPM_ERR_ARG, "null ensemble");
  if (total_ms) *total_ms = E->kernel_ms;
  if (launches) *launches = E->launches;
  return LPM_OK;
}

extern "C" int lpm_ensemble_sweep_shape(lpm_ensemble* E, int* threads, int* targets_per_thread, int* ctas_per_sm,
                                        int* items_per_slot) {
  if (!E) return set_error(LPM_ERR_ARG, "null ensemble");
  const bool fp32c = E->mode == LPM_MODE_FP32C;
  const EnsShape& sh = kEnsShapes[E->shape];
  if (threads) *threads = fp32c ? sh.threads : 0;
  if (targets_per_thread) *targets_per_thread = fp32c ? sh.tpt : 0;
  if (ctas_per_sm) *ctas_per_sm = fp32c ? sh.minb : 0;
  if (items_per_slot) *items_per_slot = fp32c ? kQueueChoices[E->choice].per_slot : 0;
  return LPM_OK;
}

extern "C" int lpm_ensemble_select_sweep(lpm_ensemble* E, int threads, int targets_per_thread, int items_per_slot) {
  if (!E) return set_error(LPM_ERR_ARG, "null ensemble");
  if (E->mode != LPM_MODE_FP32C) return set_error(LPM_ERR_STATE, "the FP64 ensemble has no sweep shape to select");
  for (int ch = 0; ch < kQueueChoiceCount; ++ch) {
    const EnsShape& sh = kEnsShapes[kQueueChoices[ch].shape];
    if (sh.threads == threads && sh.tpt == targets_per_thread && kQueueChoices[ch].per_slot == items_per_slot) {
      LPM_CUDA_TRY(cudaStreamSynchronize(E->stream));
      LPM_TRY(E->use_queue(ch));
      // the captured step graph holds the previous shape's kernel and grid: capture again
      if (E->exec) cudaGraphExecDestroy(E->exec);
      if (E->graph) cudaGraphDestroy(E->graph);
      E->exec = nullptr;
      E->graph = nullptr;
      return E->check_status("lpm_ensemble_select_sweep");
    }
  }
  return set_error(LPM_ERR_ARG, "no sweep shape %d threads x %d targets with %d items per CTA slot", threads,
                   targets_per_thread, items_per_slot);
}

extern "C" int lpm_ensemble_destroy(lpm_ensemble* E) {
  if (!E) return LPM_OK;
  E->destroy();
  delete E;
  return LPM_OK;
}
