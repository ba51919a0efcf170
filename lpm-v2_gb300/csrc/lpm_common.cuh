// lpm_common.cuh -- shared host/device infrastructure of liblpm_gpu.
//
// * status codes and the thread-local error string behind lpm_last_error_string()
// * the per-process device context: one non-blocking stream, a device status word that
//   bounded device-side waits set when they give up, and a growable workspace
// * PTX helpers: mbarrier waits with an iteration limit, 1-D TMA bulk copies
//   (cp.async.bulk) into shared memory, rcp.approx, TwoSum
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "lpm_gpu.h"

namespace lpm {

// ------------------------------------------------------------------ errors
int set_error(int code, const char* fmt, ...);
void clear_error();

#define LPM_CUDA_TRY(expr)                                                                    \
  do {                                                                                        \
    cudaError_t lpm_err_ = (expr);                                                            \
    if (lpm_err_ != cudaSuccess) {                                                            \
      return ::lpm::set_error(LPM_ERR_CUDA, "%s failed: %s (%s:%d)", #expr,                   \
                              cudaGetErrorString(lpm_err_), __FILE__, __LINE__);              \
    }                                                                                         \
  } while (0)

#define LPM_TRY(expr)              \
  do {                             \
    int lpm_rc_ = (expr);          \
    if (lpm_rc_ != LPM_OK) return lpm_rc_; \
  } while (0)

// device status word values (set by kernels, read by the host after a synchronize)
enum : int { kDevOk = 0, kDevTimeout = 1, kDevBadIndex = 2 };

// Largest particle count of a call: source lists, sort values and curve orders hold 32-bit
// particle indices.
constexpr int64_t kMaxParticles = 2147483647;

// LPM_ERR_ARG unless 0 < n <= kMaxParticles.
inline int check_count(int64_t n) {
  if (n <= 0) return set_error(LPM_ERR_ARG, "n must be positive (got %lld)", static_cast<long long>(n));
  if (n > kMaxParticles)
    return set_error(LPM_ERR_ARG, "n = %lld is above the %lld particles that 32-bit indices address",
                     static_cast<long long>(n), static_cast<long long>(kMaxParticles));
  return LPM_OK;
}

// ------------------------------------------------------------------ context / workspace
// A device buffer that only grows.  Growth synchronises the context stream first.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
};

struct Context {
  int device = -1;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  int* d_status = nullptr;     // device status word (kDev*)
  int* h_status = nullptr;     // pinned mirror
  std::vector<DevBuf> bufs;    // workspace slots, indexed by WorkSlot
  std::vector<int32_t> h_idx;  // host buffer of the active list of a host-buffer call
  std::mutex mu;               // one direct-sum call at a time per process
};

enum WorkSlot : int {
  kWsTargets = 0,   // target inputs (FP64 arrays)
  kWsSources,       // compacted source records
  kWsActive,        // active mask
  kWsScan,          // compaction block counts / offsets
  kWsPartial,       // split-K partial sums (FP64)
  kWsOutput,        // outputs before the copy back
  kWsCount
};

// Limits of the bounded waits of one sweep.  skip_tile >= 0 is a test hook: the copy of that
// source tile (an index into the record array) is never issued, so the waits for it run out
// and the sweep reports LPM_ERR_TIMEOUT without any fault.
struct WaitCfg {
  uint64_t ns;
  int64_t skip_tile;
};
__host__ __device__ constexpr WaitCfg default_wait() { return WaitCfg{1000000000ull, -1}; }

// Every device allocation of the library goes through here (cudaMalloc, or the failure that
// lpm_debug_fail_device_alloc armed).  Returns LPM_OK or LPM_ERR_ALLOC with the message set.
int device_alloc(void** p, size_t bytes);
// The wait limits for the next host-buffer sphere-BVE FP32C sweep: the ones that
// lpm_debug_inject_wait_timeout armed (once), else default_wait().
WaitCfg take_injected_wait();

// Returns the process context (initialising the device on first use).
int get_context(Context** ctx);
// Ensures workspace slot `slot` holds at least `bytes`; returns its pointer in *p.
int workspace(Context* ctx, int slot, size_t bytes, void** p);
// Synchronises ctx->stream, then converts a device status word into an LPM status.
int sync_and_check(Context* ctx, const char* what);

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline size_t align_up(size_t a, size_t b) { return (a + b - 1) / b * b; }

// ------------------------------------------------------------------ device helpers
#ifdef __CUDACC__

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// 2^x on the MUFU unit (PTX ex2.approx, flush-to-zero): relative error ~2^-22.
__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// TwoSum (Knuth): s + e == a + b exactly, with s = fl(a + b).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Adds t into the compensated pair (hi, lo).
__device__ __forceinline__ void comp_add(float& hi, float& lo, float t) {
  float s, e;
  two_sum(hi, t, s, e);
  hi = s;
  lo = __fadd_rn(lo, e);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// One arrival on an mbarrier (release semantics at CTA scope).
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Default limit of a bounded wait: 1 s of wall time.
constexpr uint64_t kWaitNs = 1000000000ull;

// Waits for `phase` of the mbarrier for at most `budget_ns` of wall time (and 2^30 polls).
// Returns false (after recording kDevTimeout in *status) when the limit is reached, so no
// wait can hang.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, int* status,
                                                  uint64_t budget_ns = kWaitNs) {
  if (mbar_try_wait(bar, phase)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, phase)) return true;
    if ((it & 255u) == 0u && global_ns() - t0 > budget_ns) break;
    if (it > (1u << 30)) break;
  }
  atomicExch(status, kDevTimeout);
  return false;
}

// 1-D bulk copy global -> shared (TMA), completion signalled on `bar` as tx bytes.
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void tma_load_1d(void* smem_dst, const void* gmem_src, uint32_t bytes,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(smem_dst)),
      "l"(gmem_src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

#endif  // __CUDACC__

}  // namespace lpm
