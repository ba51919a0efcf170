// noalloc.cu -- lpm_bve_velocity_noalloc: the sphere-BVE FP32C velocity sum with no device
// allocation at all.
//
// Who needs it: callers that cannot allocate device memory while they run.  Two common
// cases in codes that embed lpm-v2's solvers:
//  - the host application hands (almost) all of HBM to its own pool allocator when it
//    starts, so a cudaMalloc from a library either fails or fragments that pool;
//  - the caller runs a time loop next to other GPU work and cannot afford the device-wide
//    synchronisation that cudaMalloc/cudaFree may perform.
// Such a caller owns every input and output array (device pointers) and calls this entry
// point, which keeps its own scratch -- the source records and the FP64 partial sums -- in
// one file-scope __device__ array, g_noalloc_scratch, of kNoAllocScratchBytes (about
// 24 MiB).  That fixes the largest problem it accepts: n <= LPM_NOALLOC_MAX_PARTICLES.
// With CUDA's lazy module loading (the default since CUDA 12.2) the array is reserved when
// this file's module is first loaded on a device -- by the first call of this entry point
// there -- not when the library is loaded; from then on it is held until the context is
// destroyed (normally at process exit).  A caller whose pool takes most of HBM should make
// one call before its pool reserves the memory, or the first call can fail for lack of it.
//
// The sum is the FP32C one of lpm_bve_velocity (hi/lo positions, chord-form denominator,
// per-tile TwoSum accumulation, FP64 reduction), run over every particle as a source with
// zero strength for passive particles, so no compaction buffer is needed either.
//
// Rules of use:
//  - Host code must not pass g_noalloc_scratch itself to a kernel: in host code that name is
//    a host-side stand-in, not a device address.  The device address is looked up with
//    cudaGetSymbolAddress, with the device current, by the first call made in a CUDA context
//    (and again if that context is replaced, e.g. after cudaDeviceReset); make that first
//    call before any stream capture.
//  - Every call on a device shares the one array, which keeps the previous call's contents;
//    the call clears the status word it reads and overwrites every record and partial sum
//    before reading it.  Calls that overlap on the GPU (from several host threads or on
//    several streams) race on the array: serialise them.
//  - On an error return (a bounded device wait that gave up) u, v and w are left as they
//    were: the finish kernel writes nothing once the status word is set.
//  - The call is synchronous with respect to `stream` (it waits for the result status).
#include <cuda.h>

#include <mutex>

#include "bve_x2.cuh"
#include "engine.cuh"
#include "lpm_common.cuh"
#include "ops.cuh"
#include "sums.cuh"

namespace lpm {
namespace {

constexpr int kNaThreads = 128, kNaTpt = 4, kNaTile = 256, kNaMinB = 4;
constexpr int64_t kNaMaxParticles = LPM_NOALLOC_MAX_PARTICLES;
constexpr size_t kNaStatusBytes = 256;
constexpr size_t kNaRecBytes = static_cast<size_t>(kNaMaxParticles) * sizeof(BveX2::Rec);
constexpr size_t kNaPartialBytes = size_t(8) << 20;
constexpr size_t kNoAllocScratchBytes = kNaStatusBytes + kNaRecBytes + kNaPartialBytes;
static_assert(kNaMaxParticles % kNaTile == 0, "the record region holds whole tiles");

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNaMaxDevices = 64;
std::mutex g_na_mu;
// The scratch address per device, with the id of the CUDA context it was looked up in: a
// __device__ array lives in a module of one context, so a new context (cudaDeviceReset, or a
// context the caller made current) holds it at another address.
struct NaAddr {
  unsigned long long ctx_id = 0;
  void* ptr = nullptr;
};
NaAddr g_na_addr[kNaMaxDevices];

// Source records of every particle: passive particles get zero strength.
__global__ void noalloc_prep_kernel(int64_t n, int64_t npad, const double* x, const double* y, const double* z,
                                    const double* zeta, const double* area, const int32_t* active, double inv_a,
                                    double s_scale, BveX2::Rec* out) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= npad) return;
  BveX2::Rec r;
  if (k < n) {
    const double px = x[k] * inv_a, py = y[k] * inv_a, pz = z[k] * inv_a;
    float xh, xl, yh, yl, zh, zl;
    split2(px, xh, xl);
    split2(py, yh, yl);
    split2(pz, zh, zl);
    const float nc = __double2float_rn(-fma(px, px, fma(py, py, fma(pz, pz, -1.0))));
    const float s = active[k] ? __double2float_rn(zeta[k] * area[k] * s_scale) : 0.f;
    r.a = make_float4(-xh, -xh, -yh, -yh);
    r.b = make_float4(-zh, -zh, -xl, -xl);
    r.c = make_float4(-yl, -yl, -zl, -zl);
    r.d = make_float4(nc, nc, s, s);
  } else {
    r.a = r.b = r.c = r.d = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  out[k] = r;
}

__global__ void noalloc_finish_kernel(const double* partial, int64_t nsplit, int64_t nt, int64_t ib, const double* x,
                                      const double* y, const double* z, double inv_a, const int* status, double* u,
                                      double* v, double* w) {
  const int64_t il = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (il >= nt) return;
  if (*status != kDevOk) return;  // the sweep gave up: its partial sums are incomplete
  double d0 = 0.0, d1 = 0.0, d2 = 0.0;
  for (int64_t c = 0; c < nsplit; ++c) {
    d0 += partial[(c * 3 + 0) * nt + il];
    d1 += partial[(c * 3 + 1) * nt + il];
    d2 += partial[(c * 3 + 2) * nt + il];
  }
  const int64_t i = ib + il;
  const double px = x[i] * inv_a, py = y[i] * inv_a, pz = z[i] * inv_a;
  u[i] = d1 * pz - d2 * py;
  v[i] = d2 * px - d0 * pz;
  w[i] = d0 * py - d1 * px;
}

// Driver entry points for the identity of the current context, through the runtime (no
// link-time dependency on libcuda).
using PfnCtxGetCurrent = CUresult (*)(CUcontext*);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long*);

int current_context_id(int device, unsigned long long* id) {
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  if (!get_current || !get_id) {
    void* f0 = nullptr;
    void* f1 = nullptr;
    cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = cudaDriverEntryPointSymbolNotFound;
    const cudaError_t e0 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0);
    const cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1);
    if (e0 != cudaSuccess || e1 != cudaSuccess || q0 != cudaDriverEntryPointSuccess ||
        q1 != cudaDriverEntryPointSuccess || !f0 || !f1) {
      return set_error(LPM_ERR_CUDA, "cuCtxGetCurrent/cuCtxGetId are not available from the driver");
    }
    get_current = reinterpret_cast<PfnCtxGetCurrent>(f0);
    get_id = reinterpret_cast<PfnCtxGetId>(f1);
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS) return set_error(LPM_ERR_CUDA, "cuCtxGetCurrent failed");
  if (!ctx) {
    // no context bound to this thread yet: cudaSetDevice makes the device's primary one current
    LPM_CUDA_TRY(cudaSetDevice(device));
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return set_error(LPM_ERR_CUDA, "no current CUDA context");
  }
  if (get_id(ctx, id) != CUDA_SUCCESS) return set_error(LPM_ERR_CUDA, "cuCtxGetId failed");
  return LPM_OK;
}

// Device address of g_noalloc_scratch in the current context of `device` (looked up once
// per context; context ids are never reused within a process).
int scratch_address(int device, void** addr) {
  if (device < 0 || device >= kNaMaxDevices) return set_error(LPM_ERR_ARG, "device %d out of range", device);
  std::lock_guard<std::mutex> lock(g_na_mu);
  unsigned long long id = 0;
  LPM_TRY(current_context_id(device, &id));
  NaAddr& slot = g_na_addr[device];
  if (!slot.ptr || slot.ctx_id != id) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      slot.ptr = nullptr;
      return set_error(LPM_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch) failed on device %d: %s", device,
                       cudaGetErrorString(e));
    }
    slot.ptr = p;
    slot.ctx_id = id;
  }
  *addr = slot.ptr;
  return LPM_OK;
}

}  // namespace
}  // namespace lpm

extern "C" int lpm_bve_velocity_noalloc(int64_t n, const double* x, const double* y, const double* z,
                                        const double* zeta, const double* area, const int32_t* active,
                                        double radius, int64_t i_begin, int64_t i_end, double* u, double* v,
                                        double* w, void* stream_handle) {
  using namespace lpm;
  if (n <= 0) return set_error(LPM_ERR_ARG, "n must be positive (got %lld)", static_cast<long long>(n));
  if (n > kNaMaxParticles) {
    return set_error(LPM_ERR_ARG, "lpm_bve_velocity_noalloc accepts at most %lld particles (got %lld)",
                     static_cast<long long>(kNaMaxParticles), static_cast<long long>(n));
  }
  if (!x || !y || !z || !zeta || !area || !active || !u || !v || !w) return set_error(LPM_ERR_ARG, "null array");
  if (i_begin < 1 || i_end > n || i_begin > i_end) return set_error(LPM_ERR_ARG, "bad target range");
  if (!(radius > 0.0)) return set_error(LPM_ERR_ARG, "radius must be positive");
  cudaStream_t stream = static_cast<cudaStream_t>(stream_handle);
  int device = -1, sms = 0;
  LPM_CUDA_TRY(cudaGetDevice(&device));
  LPM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  void* base = nullptr;
  LPM_TRY(scratch_address(device, &base));
  int* status = static_cast<int*>(base);
  BveX2::Rec* recs = reinterpret_cast<BveX2::Rec*>(static_cast<unsigned char*>(base) + kNaStatusBytes);
  double* partial = reinterpret_cast<double*>(static_cast<unsigned char*>(base) + kNaStatusBytes + kNaRecBytes);

  const int64_t ib = i_begin - 1;
  const int64_t nt = i_end - i_begin + 1;
  const int64_t n_tiles = ceil_div(n, kNaTile);
  const int64_t npad = n_tiles * kNaTile;
  // split the sources so that the last wave is nearly full, within the partial-sum region
  const int64_t tblocks = ceil_div(nt, kNaThreads * kNaTpt);
  const int64_t cap = static_cast<int64_t>(kNaPartialBytes / (3 * sizeof(double) * static_cast<size_t>(nt)));
  int64_t nsplit = choose_split(tblocks, n_tiles, static_cast<int64_t>(sms) * kNaMinB, cap < 1 ? 1 : cap);
  const int64_t tpc = ceil_div(n_tiles, nsplit);
  nsplit = ceil_div(n_tiles, tpc);

  const double inv_a = 1.0 / radius;
  LPM_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), stream));  // the array keeps the last call's status
  noalloc_prep_kernel<<<static_cast<unsigned>(ceil_div(npad, 256)), 256, 0, stream>>>(
      n, npad, x, y, z, zeta, area, active, inv_a, -1.0 / (2.0 * 3.1415926535897932384626433832795027975 * radius),
      recs);
  SweepArgs<BveF32> a;
  a.p = BveF32::Params{x, y, z, inv_a};
  a.src = reinterpret_cast<const BveF32::Rec*>(recs);
  a.n_tiles = n_tiles;
  a.tiles_per_chunk = tpc;
  a.ib = ib;
  a.nt = nt;
  a.partial = partial;
  a.status = status;
  bve_sweep_x2_kernel<kNaThreads, kNaTpt, kNaTile, kNaMinB>
      <<<dim3(static_cast<unsigned>(tblocks), static_cast<unsigned>(nsplit)), kNaThreads, 0, stream>>>(a);
  noalloc_finish_kernel<<<static_cast<unsigned>(ceil_div(nt, 256)), 256, 0, stream>>>(partial, nsplit, nt, ib, x, y,
                                                                                        z, inv_a, status, u, v, w);
  LPM_CUDA_TRY(cudaGetLastError());
  int h_status = 0;
  LPM_CUDA_TRY(cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, stream));
  LPM_CUDA_TRY(cudaStreamSynchronize(stream));
  if (h_status != kDevOk) {
    return set_error(h_status == kDevTimeout ? LPM_ERR_TIMEOUT : LPM_ERR_CUDA, "device status %d", h_status);
  }
  return LPM_OK;
}
