// solver.cu -- device-resident RK4 solvers (BVESolver and PlaneSolver) with CUDA graphs.
//
// The state lives in HBM for the solver's lifetime.  One RK4 step is captured once into a
// CUDA graph (four stage kernels, four direct sums, event-record nodes around each sum) and
// replayed per step, so a step costs one graph launch.  The stage arithmetic restates
// timestepPrivate (src/SphereBVESolver.f90:219-353, src/PlaneIncompressibleSolver.f90:
// 171-259) in FP64 with explicit round-to-nearest intrinsics: the RK4 combination
// x + k1/6 + k2/3 + k3/3 + k4/6 is accumulated stage by stage in the same left-to-right
// order, so with LPM_MODE_FP64 sums the whole trajectory is bit-identical to the Fortran
// loop built without FMA contraction.
#include <cmath>
#include <vector>

#include "lpm_common.cuh"
#include "solver.cuh"
#include "sort.cuh"
#include "sums.cuh"

namespace lpm {

namespace {

constexpr int kStageThreads = 256;

// Stage 1 (SphereBVESolver.f90:238-244 and :249-255): k1 = dt u_prev,
// q1 = -(dt 2 Omega w)/a; acc = x + k1/6; xin = x + k1/2.
// Projection onto the sphere of radius a, used when the solver renormalises (an extension:
// the reference never does).  The RK4 stage inputs x + c k leave the sphere by O(dt^2 |u|^2);
// on fine meshes that offset exceeds the nearest-neighbour a^2 - x.x_j and the Biot-Savart
// denominator changes sign, so the renormalising solver evaluates every stage on the sphere.
__device__ __forceinline__ void project(double a, double& x, double& y, double& z) {
  const double s = a / sqrt(x * x + y * y + z * z);
  x *= s;
  y *= s;
  z *= s;
}

__global__ void bve_stage1_kernel(int64_t n, int renorm, double dt, double two_dt_omega, double radius,
                                  const double* __restrict__ x, const double* __restrict__ y,
                                  const double* __restrict__ z, const double* __restrict__ q,
                                  const double* __restrict__ u, const double* __restrict__ v,
                                  const double* __restrict__ w, double* acc_x, double* acc_y,
                                  double* acc_z, double* acc_q, double* xin, double* yin,
                                  double* zin, double* qin) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double kx = __dmul_rn(dt, u[i]);
  const double ky = __dmul_rn(dt, v[i]);
  const double kz = __dmul_rn(dt, w[i]);
  const double kq = -__ddiv_rn(__dmul_rn(two_dt_omega, w[i]), radius);
  acc_x[i] = __dadd_rn(x[i], __ddiv_rn(kx, 6.0));
  acc_y[i] = __dadd_rn(y[i], __ddiv_rn(ky, 6.0));
  acc_z[i] = __dadd_rn(z[i], __ddiv_rn(kz, 6.0));
  acc_q[i] = __dadd_rn(q[i], __ddiv_rn(kq, 6.0));
  double px = __dadd_rn(x[i], __dmul_rn(0.5, kx));
  double py = __dadd_rn(y[i], __dmul_rn(0.5, ky));
  double pz = __dadd_rn(z[i], __dmul_rn(0.5, kz));
  if (renorm) project(radius, px, py, pz);
  xin[i] = px;
  yin[i] = py;
  zin[i] = pz;
  qin[i] = __dadd_rn(q[i], __dmul_rn(0.5, kq));
}

// Stages 2-4 (:256-313): from the velocity (us, vs, ws) of the previous sum,
// q_s = -(dt 2 Omega ws)/a, k_s = dt us; acc += k_s * wt (wt = 1/3 as a division by 3, or
// 1/6 for the last stage, which also writes the new state); xin = x + c k_s.
// mode 0: stage 2 (acc += k/3, xin = x + k/2); 1: stage 3 (acc += k/3, xin = x + k);
// 2: stage 4 (x = acc + k/6).
__global__ void bve_stage_kernel(int64_t n, int which, int renorm, double dt, double two_dt_omega,
                                 double radius, double* __restrict__ x, double* __restrict__ y,
                                 double* __restrict__ z, double* __restrict__ q,
                                 const double* __restrict__ us, const double* __restrict__ vs,
                                 const double* __restrict__ ws, double* acc_x, double* acc_y,
                                 double* acc_z, double* acc_q, double* xin, double* yin,
                                 double* zin, double* qin) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double kq = -__ddiv_rn(__dmul_rn(two_dt_omega, ws[i]), radius);
  const double kx = __dmul_rn(dt, us[i]);
  const double ky = __dmul_rn(dt, vs[i]);
  const double kz = __dmul_rn(dt, ws[i]);
  if (which < 2) {
    acc_x[i] = __dadd_rn(acc_x[i], __ddiv_rn(kx, 3.0));
    acc_y[i] = __dadd_rn(acc_y[i], __ddiv_rn(ky, 3.0));
    acc_z[i] = __dadd_rn(acc_z[i], __ddiv_rn(kz, 3.0));
    acc_q[i] = __dadd_rn(acc_q[i], __ddiv_rn(kq, 3.0));
    double px, py, pz;
    if (which == 0) {
      px = __dadd_rn(x[i], __dmul_rn(0.5, kx));
      py = __dadd_rn(y[i], __dmul_rn(0.5, ky));
      pz = __dadd_rn(z[i], __dmul_rn(0.5, kz));
      qin[i] = __dadd_rn(q[i], __dmul_rn(0.5, kq));
    } else {
      px = __dadd_rn(x[i], kx);
      py = __dadd_rn(y[i], ky);
      pz = __dadd_rn(z[i], kz);
      qin[i] = __dadd_rn(q[i], kq);
    }
    if (renorm) project(radius, px, py, pz);
    xin[i] = px;
    yin[i] = py;
    zin[i] = pz;
  } else {
    double px = __dadd_rn(acc_x[i], __ddiv_rn(kx, 6.0));
    double py = __dadd_rn(acc_y[i], __ddiv_rn(ky, 6.0));
    double pz = __dadd_rn(acc_z[i], __ddiv_rn(kz, 6.0));
    if (renorm) project(radius, px, py, pz);
    x[i] = px;
    y[i] = py;
    z[i] = pz;
    q[i] = __dadd_rn(acc_q[i], __ddiv_rn(kq, 6.0));
  }
}

// Planar stages (PlaneIncompressibleSolver.f90:183-246): the same scheme on (x, y).
__global__ void plane_stage1_kernel(int64_t n, double dt, const double* x, const double* y,
                                    const double* u, const double* v, double* acc_x,
                                    double* acc_y, double* xin, double* yin) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double kx = __dmul_rn(dt, u[i]);
  const double ky = __dmul_rn(dt, v[i]);
  acc_x[i] = __dadd_rn(x[i], __ddiv_rn(kx, 6.0));
  acc_y[i] = __dadd_rn(y[i], __ddiv_rn(ky, 6.0));
  xin[i] = __dadd_rn(x[i], __dmul_rn(0.5, kx));
  yin[i] = __dadd_rn(y[i], __dmul_rn(0.5, ky));
}

__global__ void plane_stage_kernel(int64_t n, int which, double dt, double* x, double* y,
                                   const double* us, const double* vs, double* acc_x,
                                   double* acc_y, double* xin, double* yin) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double kx = __dmul_rn(dt, us[i]);
  const double ky = __dmul_rn(dt, vs[i]);
  if (which < 2) {
    acc_x[i] = __dadd_rn(acc_x[i], __ddiv_rn(kx, 3.0));
    acc_y[i] = __dadd_rn(acc_y[i], __ddiv_rn(ky, 3.0));
    if (which == 0) {
      xin[i] = __dadd_rn(x[i], __dmul_rn(0.5, kx));
      yin[i] = __dadd_rn(y[i], __dmul_rn(0.5, ky));
    } else {
      xin[i] = __dadd_rn(x[i], kx);
      yin[i] = __dadd_rn(y[i], ky);
    }
  } else {
    x[i] = __dadd_rn(acc_x[i], __ddiv_rn(kx, 6.0));
    y[i] = __dadd_rn(acc_y[i], __ddiv_rn(ky, 6.0));
  }
}

// Deterministic two-pass reduction of KE, enstrophy and circulation over active particles.
__global__ void diag_partial_kernel(int64_t n, const double* u, const double* v, const double* w,
                                    const double* q, const double* area, const int32_t* active,
                                    double* part) {
  __shared__ double sk[256], se[256], sc[256];
  double k = 0.0, e = 0.0, c = 0.0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (!active[i]) continue;
    const double m2 = u[i] * u[i] + v[i] * v[i] + (w ? w[i] * w[i] : 0.0);
    k += m2 * area[i];
    e += q[i] * q[i] * area[i];
    c += q[i] * area[i];
  }
  sk[threadIdx.x] = k;
  se[threadIdx.x] = e;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sk[threadIdx.x] += sk[threadIdx.x + s];
      se[threadIdx.x] += se[threadIdx.x + s];
      sc[threadIdx.x] += sc[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x + 0] = sk[0];
    part[3 * blockIdx.x + 1] = se[0];
    part[3 * blockIdx.x + 2] = sc[0];
  }
}

__global__ void diag_final_kernel(int nblocks, const double* part, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double k = 0.0, e = 0.0, c = 0.0;
  for (int b = 0; b < nblocks; ++b) {
    k += part[3 * b + 0];
    e += part[3 * b + 1];
    c += part[3 * b + 2];
  }
  out[0] = 0.5 * k;
  out[1] = 0.5 * e;
  out[2] = c;
}

constexpr int kDiagBlocks = 256;

}  // namespace

// ------------------------------------------------------------------ DeviceArena / SumScratch
int DeviceArena::alloc(size_t bytes, void** p) {
  void* q = nullptr;
  LPM_TRY(device_alloc(&q, bytes));
  ptrs.push_back(q);
  *p = q;
  return LPM_OK;
}

void DeviceArena::free(void* p) {
  if (!p) return;
  for (size_t i = 0; i < ptrs.size(); ++i) {
    if (ptrs[i] == p) {
      cudaFree(p);
      ptrs.erase(ptrs.begin() + static_cast<std::ptrdiff_t>(i));
      return;
    }
  }
}

void DeviceArena::release() {
  for (void* p : ptrs) cudaFree(p);
  ptrs.clear();
}

int SumScratch::init(DeviceArena& arena, int kind, int mode, int64_t ns, int64_t nt, int sm_count) {
  // sized for every sweep shape, so the autotuner can time them all in this scratch
  plan = plan_sum_max(kind, mode, ns, nt, sm_count);
  LPM_TRY(arena.alloc(plan.src_bytes, &src_buf));
  src_cap = plan.src_bytes;
  if (plan.partial_bytes) {
    void* p = nullptr;
    LPM_TRY(arena.alloc(plan.partial_bytes, &p));
    partial = static_cast<double*>(p);
  }
  partial_cap = plan.partial_bytes;
  return LPM_OK;
}

int SumScratch::fit(DeviceArena& arena, int kind, int mode, int64_t ns, int64_t nt, int sm_count) {
  plan = plan_sum_max(kind, mode, ns, nt, sm_count);
  if (plan.src_bytes > src_cap) {
    arena.free(src_buf);
    src_buf = nullptr;
    src_cap = 0;
    LPM_TRY(arena.alloc(plan.src_bytes, &src_buf));
    src_cap = plan.src_bytes;
  }
  if (plan.partial_bytes > partial_cap) {
    arena.free(partial);
    partial = nullptr;
    partial_cap = 0;
    void* p = nullptr;
    LPM_TRY(arena.alloc(plan.partial_bytes, &p));
    partial = static_cast<double*>(p);
    partial_cap = plan.partial_bytes;
  }
  return LPM_OK;
}

int64_t graph_kernel_nodes(cudaGraph_t graph) {
  size_t n = 0;
  if (cudaGraphGetNodes(graph, nullptr, &n) != cudaSuccess || n == 0) return 0;
  std::vector<cudaGraphNode_t> nodes(n);
  if (cudaGraphGetNodes(graph, nodes.data(), &n) != cudaSuccess) return 0;
  int64_t k = 0;
  for (size_t i = 0; i < n; ++i) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

std::vector<int32_t> active_list(int64_t n, const int32_t* active) {
  std::vector<int32_t> idx;
  for (int64_t j = 0; j < n; ++j)
    if (active[j]) idx.push_back(static_cast<int32_t>(j));
  return idx;
}

}  // namespace lpm

using namespace lpm;

// ====================================================================== BVE solver
struct lpm_bve_solver {
  Context* ctx = nullptr;
  cudaStream_t stream = nullptr;  // stream the work is enqueued on
  cudaStream_t own = nullptr;     // the solver's own stream (graphs are captured on it)
  DeviceArena arena;
  int64_t n = 0, ns = 0;
  int64_t cap_n = 0, cap_ns = 0;  // particles and sources the buffers hold
  int mode = LPM_MODE_FP64;
  double radius = 1.0, omega = 0.0;
  double *x, *y, *z, *q, *u, *v, *w, *area;
  double *ax, *ay, *az, *aq, *xin, *yin, *zin, *qin, *us, *vs, *ws;
  int32_t* idx = nullptr;
  int32_t* mask = nullptr;
  SumScratch scratch;
  double* diag_part = nullptr;
  double* diag_out = nullptr;
  int* status = nullptr;
  int* h_status = nullptr;
  // graph of one step
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double graph_dt = 0.0;
  int graph_renorm = -1;
  cudaEvent_t ev[8] = {};
  double kernel_ms = 0.0;
  int64_t kernel_launches = 0;
  int64_t step_kernels = 0;  // kernel nodes of the captured step graph
  bool timing = true;
  // FP32C: Hilbert-curve order of the sources, refreshed at the start of every step
  void* sort_scratch = nullptr;
  size_t sort_bytes = 0;
  int32_t* sorted = nullptr;
  // stream functions of the current state (allocated at the first request)
  SumScratch stream_scratch;
  double* absv = nullptr;
  double* psi = nullptr;  // psi_rel, psi_abs

  int sort_sources() {
    return curve_sort(stream, ns, idx, x, y, z, 1.0 / radius, sort_scratch, sort_bytes, sorted);
  }

  SumJob job(const double* px, const double* py, const double* pz, const double* pq, int kind,
             double* o0, double* o1, double* o2) const {
    SumJob j;
    j.kind = kind;
    j.mode = mode;
    j.n = n;
    j.x = px;
    j.y = py;
    j.z = pz;
    j.s1 = pq;
    j.area = area;
    j.src_idx = sorted ? sorted : idx;
    j.ns = ns;
    j.radius = radius;
    j.ib = 0;
    j.nt = n;
    j.out0 = o0;
    j.out1 = o1;
    j.out2 = o2;
    j.src_buf = scratch.src_buf;
    j.partial = scratch.partial;
    j.status = status;
    j.stream = stream;
    return j;
  }

  int velocity(const double* px, const double* py, const double* pz, const double* pq, double* o0, double* o1,
               double* o2, int kind = kSumBve) {
    if (ns == 0) {
      LPM_CUDA_TRY(cudaMemsetAsync(o0, 0, n * sizeof(double), stream));
      LPM_CUDA_TRY(cudaMemsetAsync(o1, 0, n * sizeof(double), stream));
      LPM_CUDA_TRY(cudaMemsetAsync(o2, 0, n * sizeof(double), stream));
      return LPM_OK;
    }
    return launch_sum(job(px, py, pz, pq, kind, o0, o1, o2), scratch.plan);
  }

  int enqueue_step(double dt, int renorm, bool with_events) {
    const unsigned g = static_cast<unsigned>(ceil_div(n, kStageThreads));
    if (sorted) LPM_TRY(sort_sources());
    const double two_dt_omega = (dt * 2.0) * omega;  // (dt*2)*Omega, as the Fortran associates it
    bve_stage1_kernel<<<g, kStageThreads, 0, stream>>>(n, renorm, dt, two_dt_omega, radius, x, y, z, q, u, v, w, ax,
                                                       ay, az, aq, xin, yin, zin, qin);
    LPM_CUDA_TRY(cudaGetLastError());
    for (int s = 0; s < 3; ++s) {
      if (with_events) LPM_CUDA_TRY(cudaEventRecordWithFlags(ev[2 * s], stream, cudaEventRecordExternal));
      LPM_TRY(velocity(xin, yin, zin, qin, us, vs, ws));
      if (with_events) LPM_CUDA_TRY(cudaEventRecordWithFlags(ev[2 * s + 1], stream, cudaEventRecordExternal));
      bve_stage_kernel<<<g, kStageThreads, 0, stream>>>(n, s, renorm, dt, two_dt_omega, radius, x, y, z, q, us, vs,
                                                        ws, ax, ay, az, aq, xin, yin, zin, qin);
      LPM_CUDA_TRY(cudaGetLastError());
    }
    if (with_events) LPM_CUDA_TRY(cudaEventRecordWithFlags(ev[6], stream, cudaEventRecordExternal));
    LPM_TRY(velocity(x, y, z, q, u, v, w));
    if (with_events) LPM_CUDA_TRY(cudaEventRecordWithFlags(ev[7], stream, cudaEventRecordExternal));
    return LPM_OK;
  }

  int capture(double dt, int renorm) {
    if (exec) {
      cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
    if (graph) {
      cudaGraphDestroy(graph);
      graph = nullptr;
    }
    // capture on the solver's own stream (a caller's stream may be the legacy default
    // stream, which cannot be captured), then launch on whichever stream is active
    LPM_CUDA_TRY(cudaStreamSynchronize(stream));
    cudaStream_t active = stream;
    stream = own;
    LPM_CUDA_TRY(cudaStreamBeginCapture(own, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_step(dt, renorm, true);
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamEndCapture(own, &gr);
    stream = active;
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
    cudaError_t e = cudaStreamSynchronize(stream);
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
    if (own) cudaStreamDestroy(own);
  }
};

namespace {

int upload(cudaStream_t s, double* d, const double* h, int64_t n) {
  LPM_CUDA_TRY(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, s));
  return LPM_OK;
}

int download(cudaStream_t s, double* h, const double* d, int64_t n) {
  if (h) LPM_CUDA_TRY(cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  return LPM_OK;
}

// Device buffers for up to ncap particles and nscap sources (everything but the pinned
// status word, the events and the stream).
int bve_alloc(lpm_bve_solver* S, int64_t ncap, int64_t nscap) {
  double** arrs[] = {&S->x, &S->y, &S->z, &S->q, &S->u, &S->v, &S->w, &S->area, &S->ax, &S->ay, &S->az,
                     &S->aq, &S->xin, &S->yin, &S->zin, &S->qin, &S->us, &S->vs, &S->ws};
  for (double** a : arrs) {
    void* p = nullptr;
    LPM_TRY(S->arena.alloc(ncap * sizeof(double), &p));
    *a = static_cast<double*>(p);
  }
  void* p = nullptr;
  LPM_TRY(S->arena.alloc((nscap > 0 ? nscap : 1) * sizeof(int32_t), &p));
  S->idx = static_cast<int32_t*>(p);
  LPM_TRY(S->arena.alloc(sizeof(int), &p));
  S->status = static_cast<int*>(p);
  LPM_TRY(S->arena.alloc(kDiagBlocks * 3 * sizeof(double), &p));
  S->diag_part = static_cast<double*>(p);
  LPM_TRY(S->arena.alloc(4 * sizeof(double), &p));
  S->diag_out = static_cast<double*>(p);
  LPM_TRY(S->scratch.init(S->arena, kSumBve, S->mode, nscap, ncap, S->ctx->sm_count));
  S->sort_scratch = nullptr;
  S->sorted = nullptr;
  S->sort_bytes = 0;
  if (nscap > 0 && sum_uses_sorted_sources(kSumBve, S->mode)) {
    S->sort_bytes = curve_sort_bytes(nscap);
    void* sorted = nullptr;
    LPM_TRY(S->arena.alloc(S->sort_bytes, &S->sort_scratch));
    LPM_TRY(S->arena.alloc(nscap * sizeof(int32_t), &sorted));
    S->sorted = static_cast<int32_t*>(sorted);
  }
  S->cap_n = ncap;
  S->cap_ns = nscap;
  return LPM_OK;
}

// Loads a particle set into buffers that hold it: uploads, source list, sweep plan (and the
// FP32C source order and sweep shape), and the initial velocity when u, v, w are NULL.
int bve_load(lpm_bve_solver* S, int64_t n, const std::vector<int32_t>& idx, const double* x, const double* y,
             const double* z, const double* q, const double* area, const double* u, const double* v,
             const double* w) {
  S->n = n;
  S->ns = static_cast<int64_t>(idx.size());
  LPM_CUDA_TRY(cudaMemsetAsync(S->status, 0, sizeof(int), S->stream));
  if (!idx.empty()) {
    LPM_CUDA_TRY(cudaMemcpyAsync(S->idx, idx.data(), idx.size() * sizeof(int32_t), cudaMemcpyHostToDevice, S->stream));
  }
  LPM_TRY(S->scratch.fit(S->arena, kSumBve, S->mode, S->ns, n, S->ctx->sm_count));
  LPM_TRY(upload(S->stream, S->x, x, n));
  LPM_TRY(upload(S->stream, S->y, y, n));
  LPM_TRY(upload(S->stream, S->z, z, n));
  LPM_TRY(upload(S->stream, S->q, q, n));
  LPM_TRY(upload(S->stream, S->area, area, n));
  if (S->ns > 0 && S->sorted) {
    // FP32C: the sources are ordered spatially at the start of every step (inside the step's
    // graph), so tiles stay compact as the particles move; the order only affects rounding
    LPM_TRY(S->sort_sources());
    // choose the sweep shape on this problem (the timing runs write into the stage buffers)
    int shape = 0;
    LPM_TRY(autotune_bve_shape(S->job(S->x, S->y, S->z, S->q, kSumBve, S->us, S->vs, S->ws), S->ctx->sm_count,
                               &shape));
    S->scratch.plan = plan_sum(kSumBve, S->mode, S->ns, n, S->ctx->sm_count, shape);
  }
  if (u && v && w) {
    LPM_TRY(upload(S->stream, S->u, u, n));
    LPM_TRY(upload(S->stream, S->v, v, n));
    LPM_TRY(upload(S->stream, S->w, w, n));
  } else {
    // SetVelocityOnMesh -> setVelocityFromVorticity (SphereBVE.f90:489-531)
    LPM_TRY(S->velocity(S->x, S->y, S->z, S->q, S->u, S->v, S->w, kSumBveMesh));
  }
  return LPM_OK;
}

int bve_create(lpm_bve_solver* S, int64_t n, const double* x, const double* y, const double* z, const double* q,
               const double* area, const int32_t* active, const double* u, const double* v, const double* w,
               double radius, double omega, int mode) {
  LPM_TRY(get_context(&S->ctx));
  S->mode = mode;
  S->radius = radius;
  S->omega = omega;
  LPM_CUDA_TRY(cudaStreamCreateWithFlags(&S->own, cudaStreamNonBlocking));
  S->stream = S->own;
  LPM_CUDA_TRY(cudaMallocHost(&S->h_status, sizeof(int)));
  for (auto& e : S->ev) LPM_CUDA_TRY(cudaEventCreate(&e));
  const std::vector<int32_t> idx = active_list(n, active);
  LPM_TRY(bve_alloc(S, n, static_cast<int64_t>(idx.size())));
  LPM_TRY(bve_load(S, n, idx, x, y, z, q, area, u, v, w));
  return S->check_status("lpm_bve_solver_create");
}

}  // namespace

extern "C" int lpm_bve_solver_create(lpm_bve_solver** out, int64_t n, const double* x, const double* y,
                                     const double* z, const double* relvort, const double* area,
                                     const int32_t* active, const double* u, const double* v, const double* w,
                                     double radius, double rotation_rate, int mode) {
  if (!out) return set_error(LPM_ERR_ARG, "null solver handle pointer");
  *out = nullptr;
  LPM_TRY(check_count(n));
  if (!x || !y || !z || !relvort || !area || !active) return set_error(LPM_ERR_ARG, "null input array");
  if (!(radius > 0.0)) return set_error(LPM_ERR_ARG, "radius must be positive");
  if (mode != LPM_MODE_FP64 && mode != LPM_MODE_FP32C) return set_error(LPM_ERR_ARG, "unknown mode %d", mode);
  if ((u == nullptr) != (v == nullptr) || (u == nullptr) != (w == nullptr))
    return set_error(LPM_ERR_ARG, "u, v, w must be all given or all NULL");
  lpm_bve_solver* S = new lpm_bve_solver();
  const int rc = bve_create(S, n, x, y, z, relvort, area, active, u, v, w, radius, rotation_rate, mode);
  if (rc != LPM_OK) {
    S->destroy();
    delete S;
    return rc;
  }
  *out = S;
  return LPM_OK;
}

extern "C" int lpm_bve_timestep(lpm_bve_solver* S, double dt, int n_steps, int renormalize) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  if (n_steps < 0) return set_error(LPM_ERR_ARG, "n_steps must be >= 0");
  if (!std::isfinite(dt)) return set_error(LPM_ERR_ARG, "dt must be finite");
  const int renorm = renormalize ? 1 : 0;
  if (!S->exec || S->graph_dt != dt || S->graph_renorm != renorm) LPM_TRY(S->capture(dt, renorm));
  for (int s = 0; s < n_steps; ++s) {
    LPM_CUDA_TRY(cudaGraphLaunch(S->exec, S->stream));
    // 4 stage kernels, 4 direct sums and (FP32C) the Hilbert-curve sort of the sources
    S->kernel_launches += S->step_kernels;
    if (!S->timing) continue;
    LPM_TRY(S->check_status("lpm_bve_timestep"));
    for (int k = 0; k < 4; ++k) {
      float ms = 0.f;
      LPM_CUDA_TRY(cudaEventElapsedTime(&ms, S->ev[2 * k], S->ev[2 * k + 1]));
      S->kernel_ms += ms;
    }
  }
  return S->timing ? LPM_OK : S->check_status("lpm_bve_timestep");
}

extern "C" int lpm_bve_get_state(lpm_bve_solver* S, double* x, double* y, double* z, double* relvort, double* u,
                                 double* v, double* w) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  LPM_TRY(download(S->stream, x, S->x, S->n));
  LPM_TRY(download(S->stream, y, S->y, S->n));
  LPM_TRY(download(S->stream, z, S->z, S->n));
  LPM_TRY(download(S->stream, relvort, S->q, S->n));
  LPM_TRY(download(S->stream, u, S->u, S->n));
  LPM_TRY(download(S->stream, v, S->v, S->n));
  LPM_TRY(download(S->stream, w, S->w, S->n));
  return S->check_status("lpm_bve_get_state");
}

extern "C" int lpm_bve_set_state(lpm_bve_solver* S, const double* x, const double* y, const double* z,
                                 const double* relvort, const double* u, const double* v, const double* w) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  if (!x || !y || !z || !relvort || !u || !v || !w) return set_error(LPM_ERR_ARG, "null state array");
  LPM_TRY(upload(S->stream, S->x, x, S->n));
  LPM_TRY(upload(S->stream, S->y, y, S->n));
  LPM_TRY(upload(S->stream, S->z, z, S->n));
  LPM_TRY(upload(S->stream, S->q, relvort, S->n));
  LPM_TRY(upload(S->stream, S->u, u, S->n));
  LPM_TRY(upload(S->stream, S->v, v, S->n));
  LPM_TRY(upload(S->stream, S->w, w, S->n));
  return S->check_status("lpm_bve_set_state");
}

extern "C" int lpm_bve_solver_remesh(lpm_bve_solver* S, int64_t n, const double* x, const double* y, const double* z,
                                     const double* relvort, const double* area, const int32_t* active, const double* u,
                                     const double* v, const double* w) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  LPM_TRY(check_count(n));
  if (!x || !y || !z || !relvort || !area || !active) return set_error(LPM_ERR_ARG, "null input array");
  if ((u == nullptr) != (v == nullptr) || (u == nullptr) != (w == nullptr))
    return set_error(LPM_ERR_ARG, "u, v, w must be all given or all NULL");
  LPM_CUDA_TRY(cudaStreamSynchronize(S->stream));
  // the step graph and the stream-function buffers are sized for the old particle set
  if (S->exec) cudaGraphExecDestroy(S->exec);
  if (S->graph) cudaGraphDestroy(S->graph);
  S->exec = nullptr;
  S->graph = nullptr;
  const std::vector<int32_t> idx = active_list(n, active);
  const int64_t ns = static_cast<int64_t>(idx.size());
  if (n > S->cap_n || ns > S->cap_ns) {
    // grow with 1/8 headroom, so that the next remeshes of a similar size reuse the buffers
    S->arena.release();
    S->mask = nullptr;
    S->absv = S->psi = nullptr;
    S->stream_scratch = SumScratch();
    S->scratch = SumScratch();
    LPM_TRY(bve_alloc(S, n + n / 8, ns + ns / 8));
  } else {
    S->arena.free(S->mask);  // the diagnostics' mask of the old set
    S->mask = nullptr;
  }
  if (S->psi) {
    S->arena.free(S->absv);
    S->arena.free(S->psi);
    S->arena.free(S->stream_scratch.src_buf);
    S->arena.free(S->stream_scratch.partial);
    S->absv = S->psi = nullptr;
    S->stream_scratch = SumScratch();
  }
  LPM_TRY(bve_load(S, n, idx, x, y, z, relvort, area, u, v, w));
  return S->check_status("lpm_bve_solver_remesh");
}

namespace {
int diagnostics(cudaStream_t s, int64_t n, const double* u, const double* v, const double* w, const double* q,
                const double* area, const int32_t* act_dev, double* part, double* out, double* ke, double* en,
                double* ci) {
  diag_partial_kernel<<<kDiagBlocks, 256, 0, s>>>(n, u, v, w, q, area, act_dev, part);
  diag_final_kernel<<<1, 32, 0, s>>>(kDiagBlocks, part, out);
  LPM_CUDA_TRY(cudaGetLastError());
  double h[3];
  LPM_CUDA_TRY(cudaMemcpyAsync(h, out, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  LPM_CUDA_TRY(cudaStreamSynchronize(s));
  if (ke) *ke = h[0];
  if (en) *en = h[1];
  if (ci) *ci = h[2];
  return LPM_OK;
}
}  // namespace

// The active mask for the diagnostics is kept as a per-particle int array built from idx.
__global__ void mask_from_idx_kernel(int64_t ns, const int32_t* idx, int32_t* mask) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < ns) mask[idx[k]] = 1;
}

static int mask_buffer(DeviceArena& arena, cudaStream_t s, int64_t n, int64_t ns, const int32_t* idx,
                       int32_t** mask) {
  if (*mask) return LPM_OK;
  void* p = nullptr;
  LPM_TRY(arena.alloc(n * sizeof(int32_t), &p));
  *mask = static_cast<int32_t*>(p);
  LPM_CUDA_TRY(cudaMemsetAsync(*mask, 0, n * sizeof(int32_t), s));
  if (ns) mask_from_idx_kernel<<<static_cast<unsigned>(ceil_div(ns, 256)), 256, 0, s>>>(ns, idx, *mask);
  LPM_CUDA_TRY(cudaGetLastError());
  return LPM_OK;
}

extern "C" int lpm_bve_diagnostics(lpm_bve_solver* S, double* ke, double* en, double* ci) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  LPM_TRY(mask_buffer(S->arena, S->stream, S->n, S->ns, S->idx, &S->mask));
  return diagnostics(S->stream, S->n, S->u, S->v, S->w, S->q, S->area, S->mask, S->diag_part, S->diag_out, ke, en,
                     ci);
}

namespace lpm {
// absolute vorticity of the current state: zeta + 2 Omega z / a (SphereBVE.f90:347)
__global__ void bve_absvort_kernel(int64_t n, const double* q, const double* z, double two_omega_over_a,
                                   double* out) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) out[i] = q[i] + two_omega_over_a * z[i];
}
}  // namespace lpm

extern "C" int lpm_bve_solver_stream_functions(lpm_bve_solver* S, const double* absvort, double* psi_rel,
                                               double* psi_abs) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  if (!psi_rel || !psi_abs) return set_error(LPM_ERR_ARG, "null output array");
  const size_t nb = static_cast<size_t>(S->n) * sizeof(double);
  if (!S->psi) {
    void* p = nullptr;
    LPM_TRY(S->arena.alloc(nb, &p));
    S->absv = static_cast<double*>(p);
    LPM_TRY(S->arena.alloc(2 * nb, &p));
    S->psi = static_cast<double*>(p);
    if (S->ns > 0)
      LPM_TRY(S->stream_scratch.init(S->arena, kSumSphereStream, S->mode, S->ns, S->n, S->ctx->sm_count));
  }
  if (absvort) {
    LPM_CUDA_TRY(cudaMemcpyAsync(S->absv, absvort, nb, cudaMemcpyHostToDevice, S->stream));
  } else {
    bve_absvort_kernel<<<static_cast<unsigned>(ceil_div(S->n, 256)), 256, 0, S->stream>>>(
        S->n, S->q, S->z, 2.0 * S->omega / S->radius, S->absv);
    LPM_CUDA_TRY(cudaGetLastError());
  }
  if (S->ns == 0) {
    LPM_CUDA_TRY(cudaMemsetAsync(S->psi, 0, 2 * nb, S->stream));
  } else {
    SumJob j = S->job(S->x, S->y, S->z, S->q, kSumSphereStream, S->psi, S->psi + S->n, nullptr);
    j.s2 = S->absv;
    j.src_buf = S->stream_scratch.src_buf;
    j.partial = S->stream_scratch.partial;
    LPM_TRY(launch_sum(j, S->stream_scratch.plan));
  }
  LPM_CUDA_TRY(cudaMemcpyAsync(psi_rel, S->psi, nb, cudaMemcpyDeviceToHost, S->stream));
  LPM_CUDA_TRY(cudaMemcpyAsync(psi_abs, S->psi + S->n, nb, cudaMemcpyDeviceToHost, S->stream));
  return S->check_status("lpm_bve_solver_stream_functions");
}

extern "C" int lpm_bve_kernel_timing(lpm_bve_solver* S, double* total_ms, int64_t* launches) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  if (total_ms) *total_ms = S->kernel_ms;
  if (launches) *launches = S->kernel_launches;
  return LPM_OK;
}

extern "C" int lpm_bve_solver_set_stream(lpm_bve_solver* S, void* stream) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  LPM_CUDA_TRY(cudaStreamSynchronize(S->stream));
  S->stream = stream ? static_cast<cudaStream_t>(stream) : S->own;
  return LPM_OK;
}

extern "C" int lpm_bve_solver_set_timing(lpm_bve_solver* S, int enable) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  S->timing = enable != 0;
  return LPM_OK;
}

extern "C" int lpm_bve_solver_destroy(lpm_bve_solver* S) {
  if (!S) return LPM_OK;
  S->destroy();
  delete S;
  return LPM_OK;
}

// ====================================================================== plane solver
struct lpm_plane_solver {
  Context* ctx = nullptr;
  cudaStream_t stream = nullptr;
  DeviceArena arena;
  int64_t n = 0, ns = 0;
  int64_t cap_n = 0, cap_ns = 0;  // particles and sources the buffers hold
  int mode = LPM_MODE_FP64;
  double delta = 0.0;
  double *x, *y, *om, *u, *v, *area, *ax, *ay, *xin, *yin, *us, *vs;
  int32_t* idx = nullptr;
  int32_t* mask = nullptr;
  SumScratch scratch;
  double* diag_part = nullptr;
  double* diag_out = nullptr;
  int* status = nullptr;
  int* h_status = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double graph_dt = 0.0;
  // FP32C: 2-D Hilbert-curve order of the sources, refreshed at the start of every step
  void* sort_scratch = nullptr;
  size_t sort_bytes = 0;
  int32_t* sorted = nullptr;

  int sort_sources() { return curve_sort2d(stream, ns, idx, x, y, sort_scratch, sort_bytes, sorted); }

  int velocity(const double* px, const double* py, double* o0, double* o1) {
    if (ns == 0) {
      LPM_CUDA_TRY(cudaMemsetAsync(o0, 0, n * sizeof(double), stream));
      LPM_CUDA_TRY(cudaMemsetAsync(o1, 0, n * sizeof(double), stream));
      return LPM_OK;
    }
    SumJob j;
    j.kind = kSumPlane;
    j.mode = mode;
    j.n = n;
    j.x = px;
    j.y = py;
    j.s1 = om;
    j.area = area;
    j.src_idx = sorted ? sorted : idx;
    j.ns = ns;
    j.delta = delta;
    j.ib = 0;
    j.nt = n;
    j.out0 = o0;
    j.out1 = o1;
    j.src_buf = scratch.src_buf;
    j.partial = scratch.partial;
    j.status = status;
    j.stream = stream;
    return launch_sum(j, scratch.plan);
  }

  int enqueue_step(double dt) {
    const unsigned g = static_cast<unsigned>(ceil_div(n, kStageThreads));
    if (sorted) LPM_TRY(sort_sources());
    plane_stage1_kernel<<<g, kStageThreads, 0, stream>>>(n, dt, x, y, u, v, ax, ay, xin, yin);
    LPM_CUDA_TRY(cudaGetLastError());
    for (int s = 0; s < 3; ++s) {
      LPM_TRY(velocity(xin, yin, us, vs));
      plane_stage_kernel<<<g, kStageThreads, 0, stream>>>(n, s, dt, x, y, us, vs, ax, ay, xin, yin);
      LPM_CUDA_TRY(cudaGetLastError());
    }
    return velocity(x, y, u, v);
  }

  int capture(double dt) {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    LPM_CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_step(dt);
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamEndCapture(stream, &gr);
    if (rc != LPM_OK) {
      if (gr) cudaGraphDestroy(gr);
      return rc;
    }
    if (e != cudaSuccess) return set_error(LPM_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(e));
    graph = gr;
    LPM_CUDA_TRY(cudaGraphInstantiate(&exec, graph, 0));
    graph_dt = dt;
    return LPM_OK;
  }

  int check_status(const char* what) {
    LPM_CUDA_TRY(cudaMemcpyAsync(h_status, status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    cudaError_t e = cudaStreamSynchronize(stream);
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
    if (h_status) cudaFreeHost(h_status);
    arena.release();
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {
// Device buffers for up to ncap particles and nscap sources.
int plane_alloc(lpm_plane_solver* S, int64_t ncap, int64_t nscap) {
  double** arrs[] = {&S->x, &S->y, &S->om, &S->u, &S->v, &S->area, &S->ax, &S->ay, &S->xin, &S->yin, &S->us, &S->vs};
  for (double** a : arrs) {
    void* p = nullptr;
    LPM_TRY(S->arena.alloc(ncap * sizeof(double), &p));
    *a = static_cast<double*>(p);
  }
  void* p = nullptr;
  LPM_TRY(S->arena.alloc((nscap > 0 ? nscap : 1) * sizeof(int32_t), &p));
  S->idx = static_cast<int32_t*>(p);
  LPM_TRY(S->arena.alloc(sizeof(int), &p));
  S->status = static_cast<int*>(p);
  LPM_TRY(S->arena.alloc(kDiagBlocks * 3 * sizeof(double), &p));
  S->diag_part = static_cast<double*>(p);
  LPM_TRY(S->arena.alloc(4 * sizeof(double), &p));
  S->diag_out = static_cast<double*>(p);
  LPM_TRY(S->scratch.init(S->arena, kSumPlane, S->mode, nscap, ncap, S->ctx->sm_count));
  S->sort_scratch = nullptr;
  S->sorted = nullptr;
  S->sort_bytes = 0;
  if (nscap > 0 && sum_uses_sorted_sources(kSumPlane, S->mode)) {
    S->sort_bytes = curve_sort2d_bytes(nscap);
    LPM_TRY(S->arena.alloc(S->sort_bytes, &S->sort_scratch));
    LPM_TRY(S->arena.alloc(nscap * sizeof(int32_t), &p));
    S->sorted = static_cast<int32_t*>(p);
  }
  S->cap_n = ncap;
  S->cap_ns = nscap;
  return LPM_OK;
}

// Loads a particle set into buffers that hold it (uploads, source list and order, plan, and
// the initial velocity when u, v are NULL).
int plane_load(lpm_plane_solver* S, int64_t n, const std::vector<int32_t>& idx, const double* x, const double* y,
               const double* om, const double* area, const double* u, const double* v) {
  S->n = n;
  S->ns = static_cast<int64_t>(idx.size());
  LPM_CUDA_TRY(cudaMemsetAsync(S->status, 0, sizeof(int), S->stream));
  if (!idx.empty()) {
    LPM_CUDA_TRY(cudaMemcpyAsync(S->idx, idx.data(), idx.size() * sizeof(int32_t), cudaMemcpyHostToDevice, S->stream));
  }
  LPM_TRY(S->scratch.fit(S->arena, kSumPlane, S->mode, S->ns, n, S->ctx->sm_count));
  LPM_TRY(upload(S->stream, S->x, x, n));
  LPM_TRY(upload(S->stream, S->y, y, n));
  LPM_TRY(upload(S->stream, S->om, om, n));
  LPM_TRY(upload(S->stream, S->area, area, n));
  if (S->sorted && S->ns > 0) LPM_TRY(S->sort_sources());
  if (u && v) {
    LPM_TRY(upload(S->stream, S->u, u, n));
    LPM_TRY(upload(S->stream, S->v, v, n));
  } else {
    LPM_TRY(S->velocity(S->x, S->y, S->u, S->v));
  }
  return LPM_OK;
}

int plane_create(lpm_plane_solver* S, int64_t n, const double* x, const double* y, const double* om,
                 const double* area, const int32_t* active, const double* u, const double* v, double delta,
                 int mode) {
  LPM_TRY(get_context(&S->ctx));
  S->mode = mode;
  S->delta = delta;
  LPM_CUDA_TRY(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
  LPM_CUDA_TRY(cudaMallocHost(&S->h_status, sizeof(int)));
  const std::vector<int32_t> idx = active_list(n, active);
  LPM_TRY(plane_alloc(S, n, static_cast<int64_t>(idx.size())));
  LPM_TRY(plane_load(S, n, idx, x, y, om, area, u, v));
  return S->check_status("lpm_plane_solver_create");
}
}  // namespace

extern "C" int lpm_plane_solver_create(lpm_plane_solver** out, int64_t n, const double* x, const double* y,
                                       const double* omega, const double* area, const int32_t* active,
                                       const double* u, const double* v, double delta, int mode) {
  if (!out) return set_error(LPM_ERR_ARG, "null solver handle pointer");
  *out = nullptr;
  LPM_TRY(check_count(n));
  if (!x || !y || !omega || !area || !active) return set_error(LPM_ERR_ARG, "null input array");
  if (!(delta >= 0.0)) return set_error(LPM_ERR_ARG, "delta must be >= 0");
  if (mode != LPM_MODE_FP64 && mode != LPM_MODE_FP32C) return set_error(LPM_ERR_ARG, "unknown mode %d", mode);
  if ((u == nullptr) != (v == nullptr)) return set_error(LPM_ERR_ARG, "u and v must be both given or both NULL");
  lpm_plane_solver* S = new lpm_plane_solver();
  const int rc = plane_create(S, n, x, y, omega, area, active, u, v, delta, mode);
  if (rc != LPM_OK) {
    S->destroy();
    delete S;
    return rc;
  }
  *out = S;
  return LPM_OK;
}

extern "C" int lpm_plane_timestep(lpm_plane_solver* S, double dt, int n_steps) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  if (n_steps < 0 || !std::isfinite(dt)) return set_error(LPM_ERR_ARG, "bad dt or n_steps");
  if (!S->exec || S->graph_dt != dt) LPM_TRY(S->capture(dt));
  for (int s = 0; s < n_steps; ++s) {
    LPM_CUDA_TRY(cudaGraphLaunch(S->exec, S->stream));
  }
  return S->check_status("lpm_plane_timestep");
}

extern "C" int lpm_plane_get_state(lpm_plane_solver* S, double* x, double* y, double* u, double* v) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  LPM_TRY(download(S->stream, x, S->x, S->n));
  LPM_TRY(download(S->stream, y, S->y, S->n));
  LPM_TRY(download(S->stream, u, S->u, S->n));
  LPM_TRY(download(S->stream, v, S->v, S->n));
  return S->check_status("lpm_plane_get_state");
}

extern "C" int lpm_plane_solver_remesh(lpm_plane_solver* S, int64_t n, const double* x, const double* y,
                                       const double* omega, const double* area, const int32_t* active,
                                       const double* u, const double* v) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  LPM_TRY(check_count(n));
  if (!x || !y || !omega || !area || !active) return set_error(LPM_ERR_ARG, "null input array");
  if ((u == nullptr) != (v == nullptr)) return set_error(LPM_ERR_ARG, "u and v must be both given or both NULL");
  LPM_CUDA_TRY(cudaStreamSynchronize(S->stream));
  if (S->exec) cudaGraphExecDestroy(S->exec);
  if (S->graph) cudaGraphDestroy(S->graph);
  S->exec = nullptr;
  S->graph = nullptr;
  const std::vector<int32_t> idx = active_list(n, active);
  const int64_t ns = static_cast<int64_t>(idx.size());
  if (n > S->cap_n || ns > S->cap_ns) {
    S->arena.release();  // grow with 1/8 headroom
    S->mask = nullptr;
    S->scratch = SumScratch();
    LPM_TRY(plane_alloc(S, n + n / 8, ns + ns / 8));
  } else {
    S->arena.free(S->mask);
    S->mask = nullptr;
  }
  LPM_TRY(plane_load(S, n, idx, x, y, omega, area, u, v));
  return S->check_status("lpm_plane_solver_remesh");
}

extern "C" int lpm_plane_diagnostics(lpm_plane_solver* S, double* ke, double* en, double* ci) {
  if (!S) return set_error(LPM_ERR_ARG, "null solver");
  LPM_TRY(mask_buffer(S->arena, S->stream, S->n, S->ns, S->idx, &S->mask));
  return diagnostics(S->stream, S->n, S->u, S->v, nullptr, S->om, S->area, S->mask, S->diag_part, S->diag_out, ke,
                     en, ci);
}

extern "C" int lpm_plane_solver_destroy(lpm_plane_solver* S) {
  if (!S) return LPM_OK;
  S->destroy();
  delete S;
  return LPM_OK;
}
