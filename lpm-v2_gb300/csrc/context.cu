// context.cu -- error reporting, the per-process device context and its workspace.
#include "lpm_common.cuh"

namespace lpm {

namespace {
thread_local std::string g_last_error;
Context* g_ctx = nullptr;
std::mutex g_ctx_mu;
// test hooks (lpm_debug_*): the countdown to an injected allocation failure, and wait limits
// armed for the next host-buffer sphere-BVE FP32C sweep
std::mutex g_hook_mu;
int64_t g_fail_alloc_in = 0;
bool g_wait_armed = false;
WaitCfg g_wait = default_wait();
}  // namespace

int device_alloc(void** p, size_t bytes) {
  *p = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_hook_mu);
    if (g_fail_alloc_in > 0 && --g_fail_alloc_in == 0) {
      return set_error(LPM_ERR_ALLOC, "device allocation of %zu bytes failed: injected failure "
                       "(lpm_debug_fail_device_alloc)", bytes);
    }
  }
  const cudaError_t e = cudaMalloc(p, bytes > 0 ? bytes : 16);
  if (e != cudaSuccess) {
    *p = nullptr;
    return set_error(LPM_ERR_ALLOC, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
  }
  return LPM_OK;
}

WaitCfg take_injected_wait() {
  std::lock_guard<std::mutex> lock(g_hook_mu);
  if (!g_wait_armed) return default_wait();
  g_wait_armed = false;
  return g_wait;
}

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

void clear_error() { g_last_error.clear(); }

int get_context(Context** out) {
  std::lock_guard<std::mutex> lock(g_ctx_mu);
  if (g_ctx) {
    int dev = -1;
    LPM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev != g_ctx->device) {
      return set_error(LPM_ERR_STATE,
                       "liblpm_gpu was initialised on device %d but device %d is current; "
                       "one process drives one GPU",
                       g_ctx->device, dev);
    }
    *out = g_ctx;
    return LPM_OK;
  }
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    return set_error(LPM_ERR_NO_DEVICE, "no CUDA device available (%s)",
                     e == cudaSuccess ? "device count is 0" : cudaGetErrorString(e));
  }
  Context* c = new Context();
  LPM_CUDA_TRY(cudaGetDevice(&c->device));
  LPM_CUDA_TRY(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device));
  LPM_CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  LPM_CUDA_TRY(cudaMalloc(&c->d_status, sizeof(int)));
  LPM_CUDA_TRY(cudaMemset(c->d_status, 0, sizeof(int)));
  LPM_CUDA_TRY(cudaMallocHost(&c->h_status, sizeof(int)));
  c->bufs.resize(kWsCount);
  g_ctx = c;
  *out = c;
  return LPM_OK;
}

int workspace(Context* ctx, int slot, size_t bytes, void** p) {
  DevBuf& b = ctx->bufs[slot];
  if (b.bytes < bytes) {
    LPM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (b.ptr) LPM_CUDA_TRY(cudaFree(b.ptr));
    b.ptr = nullptr;
    b.bytes = 0;
    const size_t want = align_up(bytes + bytes / 4, 1 << 20);
    LPM_TRY(device_alloc(&b.ptr, want));
    b.bytes = want;
  }
  *p = b.ptr;
  return LPM_OK;
}

int sync_and_check(Context* ctx, const char* what) {
  LPM_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    return set_error(LPM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
  const int st = *ctx->h_status;
  if (st != kDevOk) {
    LPM_CUDA_TRY(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
    LPM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (st == kDevTimeout) {
      return set_error(LPM_ERR_TIMEOUT, "%s: a bounded device-side wait gave up", what);
    }
    return set_error(LPM_ERR_CUDA, "%s: device status %d", what, st);
  }
  return LPM_OK;
}

}  // namespace lpm

extern "C" const char* lpm_last_error_string(void) { return lpm::g_last_error.c_str(); }

extern "C" int lpm_release_workspace(void) {
  using namespace lpm;
  Context* ctx = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_ctx_mu);
    ctx = g_ctx;
  }
  if (!ctx) return LPM_OK;  // nothing allocated yet
  std::lock_guard<std::mutex> lock(ctx->mu);
  LPM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  for (DevBuf& b : ctx->bufs) {
    if (b.ptr) LPM_CUDA_TRY(cudaFree(b.ptr));
    b.ptr = nullptr;
    b.bytes = 0;
  }
  std::vector<int32_t>().swap(ctx->h_idx);
  return LPM_OK;
}

extern "C" int lpm_debug_fail_device_alloc(int64_t k) {
  if (k < 0) return lpm::set_error(LPM_ERR_ARG, "k must be >= 0 (got %lld)", static_cast<long long>(k));
  std::lock_guard<std::mutex> lock(lpm::g_hook_mu);
  lpm::g_fail_alloc_in = k;
  return LPM_OK;
}

extern "C" int lpm_debug_inject_wait_timeout(int64_t skip_tile, int64_t budget_ns) {
  if (skip_tile < 0 || budget_ns <= 0 || budget_ns > 1000000000ll)
    return lpm::set_error(LPM_ERR_ARG, "need skip_tile >= 0 and 0 < budget_ns <= 1e9");
  std::lock_guard<std::mutex> lock(lpm::g_hook_mu);
  lpm::g_wait = lpm::WaitCfg{static_cast<uint64_t>(budget_ns), skip_tile};
  lpm::g_wait_armed = true;
  return LPM_OK;
}

extern "C" const char* lpm_version(void) { return "lpm_gpu 0.1 (sm_103a)"; }
