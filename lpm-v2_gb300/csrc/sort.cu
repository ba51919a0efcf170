// sort.cu -- spatial (Hilbert-curve) ordering of the source particles on the device.
//
// The FP32C sweeps store every source relative to the origin of its group (64 or 128
// consecutive sources), so groups must be spatially compact: sources are ordered by the 30-bit index, along a 3-D
// Hilbert curve over a 2^10 grid per axis, of the cell holding their unit-scaled position,
// with a device radix sort (CUB).  Consecutive Hilbert cells are face neighbours, so a group
// of consecutive sources forms one connected patch (a Hilbert-curve order jumps across the grid at
// its octant boundaries, which leaves some groups in two distant pieces).  The order only
// affects rounding (the FP32C sum is order-independent to its error bound); FP64 sums keep
// the reference's ascending order.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include "lpm_common.cuh"
#include "hilbert.cuh"
#include "sort.cuh"

namespace lpm {
namespace {

__device__ __forceinline__ uint32_t quant10(double p) {
  double t = (p + 1.0) * 512.0;
  t = t < 0.0 ? 0.0 : (t > 1023.0 ? 1023.0 : t);
  return static_cast<uint32_t>(t);
}

__device__ __forceinline__ uint32_t cell_key(double px, double py, double pz) {
  return hilbert_index30(quant10(px), quant10(py), quant10(pz));
}

__global__ void curve_keys_kernel(int64_t ns, const int32_t* idx, const double* x, const double* y,
                                   const double* z, double inv_a, uint32_t* keys, int32_t* vals) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= ns) return;
  const int32_t j = idx[k];
  keys[k] = cell_key(x[j] * inv_a, y[j] * inv_a, z ? z[j] * inv_a : 0.0);
  vals[k] = j;
}

// 64-bit keys: the group in the high bits, the curve index of the group-scaled position low.
__global__ void grouped_curve_keys_kernel(int64_t ns, const int32_t* idx, const int32_t* grp, const double* x,
                                           const double* y, const double* z, const double* inv_a, uint64_t* keys,
                                           int32_t* vals) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= ns) return;
  const int32_t j = idx[k];
  const int32_t g = grp[k];
  const double s = inv_a[g];
  keys[k] = (static_cast<uint64_t>(g) << 30) | cell_key(x[j] * s, y[j] * s, z[j] * s);
  vals[k] = j;
}

// Bounding box {x_min, y_min, x_max, y_max} of the listed points, in two launches: each block
// of bbox2d_partial_kernel reduces a grid-stride share of the points, and bbox2d_final_kernel
// reduces the blocks' boxes.  Minima and maxima are exact, so the box does not depend on the
// split.  (One block over every point was latency-bound: 81 us for 65,536 points.)
constexpr int kBoxThreads = 256;
constexpr int kBoxBlocksMax = 256;

int box_blocks(int64_t ns) {
  const int64_t b = ceil_div(ns, 4 * kBoxThreads);
  return static_cast<int>(b < 1 ? 1 : (b > kBoxBlocksMax ? kBoxBlocksMax : b));
}

__device__ __forceinline__ void box_reduce(double (&r)[4][kBoxThreads], double a, double b, double c, double d) {
  const int t = threadIdx.x;
  r[0][t] = a;
  r[1][t] = b;
  r[2][t] = c;
  r[3][t] = d;
  __syncthreads();
  for (int w = kBoxThreads / 2; w > 0; w >>= 1) {
    if (t < w) {
      r[0][t] = fmin(r[0][t], r[0][t + w]);
      r[1][t] = fmin(r[1][t], r[1][t + w]);
      r[2][t] = fmax(r[2][t], r[2][t + w]);
      r[3][t] = fmax(r[3][t], r[3][t + w]);
    }
    __syncthreads();
  }
}

// part[c * gridDim.x + block], c = 0..3
__global__ void __launch_bounds__(kBoxThreads) bbox2d_partial_kernel(int64_t ns, const int32_t* idx, const double* x,
                                                                     const double* y, double* part) {
  __shared__ double r[4][kBoxThreads];
  double a = 1e300, b = 1e300, c = -1e300, d = -1e300;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * kBoxThreads;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * kBoxThreads + threadIdx.x; k < ns; k += stride) {
    const int32_t j = idx[k];
    a = fmin(a, x[j]);
    b = fmin(b, y[j]);
    c = fmax(c, x[j]);
    d = fmax(d, y[j]);
  }
  box_reduce(r, a, b, c, d);
  if (threadIdx.x < 4) part[threadIdx.x * gridDim.x + blockIdx.x] = r[threadIdx.x][0];
}

__global__ void __launch_bounds__(kBoxThreads) bbox2d_final_kernel(int nb, const double* part, double* box) {
  __shared__ double r[4][kBoxThreads];
  const int t = threadIdx.x;
  const bool v = t < nb;
  box_reduce(r, v ? part[t] : 1e300, v ? part[nb + t] : 1e300, v ? part[2 * nb + t] : -1e300,
             v ? part[3 * nb + t] : -1e300);
  if (t < 4) box[t] = r[t][0];
}

// 2-D keys: the Hilbert index of the cell of a 2^16 grid laid over the bounding box (one
// scale for both axes, so cells are square).
__global__ void curve2d_keys_kernel(int64_t ns, const int32_t* idx, const double* x, const double* y,
                                    const double* box, uint32_t* keys, int32_t* vals) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= ns) return;
  const int32_t j = idx[k];
  const double ext = fmax(fmax(box[2] - box[0], box[3] - box[1]), 1e-300);
  const double s = 65535.0 / ext;
  double u = (x[j] - box[0]) * s, v = (y[j] - box[1]) * s;
  u = u < 0.0 ? 0.0 : (u > 65535.0 ? 65535.0 : u);
  v = v < 0.0 ? 0.0 : (v > 65535.0 ? 65535.0 : v);
  keys[k] = hilbert_index2d(static_cast<uint32_t>(u), static_cast<uint32_t>(v));
  vals[k] = j;
}

int end_bit_for(int n_groups) {
  int b = 0;
  while ((1 << b) < n_groups) ++b;
  return 30 + b;
}

}  // namespace

size_t grouped_curve_sort_bytes(int64_t ns, int n_groups) {
  size_t temp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, temp, static_cast<const uint64_t*>(nullptr), static_cast<uint64_t*>(nullptr),
                                  static_cast<const int32_t*>(nullptr), static_cast<int32_t*>(nullptr),
                                  static_cast<int>(ns), 0, end_bit_for(n_groups));
  return align_up(temp, 256) + 2 * align_up(static_cast<size_t>(ns) * 8, 256) + align_up(static_cast<size_t>(ns) * 4, 256);
}

int grouped_curve_sort(cudaStream_t stream, int64_t ns, int n_groups, const int32_t* idx, const int32_t* grp,
                        const double* x, const double* y, const double* z, const double* inv_a, void* scratch,
                        size_t scratch_bytes, int32_t* sorted) {
  if (ns <= 0) return LPM_OK;
  const int end_bit = end_bit_for(n_groups);
  size_t temp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, temp, static_cast<const uint64_t*>(nullptr), static_cast<uint64_t*>(nullptr),
                                  static_cast<const int32_t*>(nullptr), static_cast<int32_t*>(nullptr),
                                  static_cast<int>(ns), 0, end_bit);
  const size_t k8 = align_up(static_cast<size_t>(ns) * 8, 256);
  const size_t k4 = align_up(static_cast<size_t>(ns) * 4, 256);
  if (scratch_bytes < align_up(temp, 256) + 2 * k8 + k4) return set_error(LPM_ERR_STATE, "grouped sort scratch too small");
  char* base = static_cast<char*>(scratch);
  uint64_t* keys_in = reinterpret_cast<uint64_t*>(base + align_up(temp, 256));
  uint64_t* keys_out = reinterpret_cast<uint64_t*>(base + align_up(temp, 256) + k8);
  int32_t* vals_in = reinterpret_cast<int32_t*>(base + align_up(temp, 256) + 2 * k8);
  grouped_curve_keys_kernel<<<static_cast<unsigned>(ceil_div(ns, 256)), 256, 0, stream>>>(ns, idx, grp, x, y, z,
                                                                                           inv_a, keys_in, vals_in);
  LPM_CUDA_TRY(cudaGetLastError());
  LPM_CUDA_TRY(cub::DeviceRadixSort::SortPairs(base, temp, keys_in, keys_out, vals_in, sorted, static_cast<int>(ns), 0,
                                               end_bit, stream));
  return LPM_OK;
}

size_t curve_sort_bytes(int64_t ns) {
  size_t temp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, temp, static_cast<const uint32_t*>(nullptr), static_cast<uint32_t*>(nullptr),
                                  static_cast<const int32_t*>(nullptr), static_cast<int32_t*>(nullptr),
                                  static_cast<int>(ns), 0, 30);
  // keys in/out + values in
  return align_up(temp, 256) + 3 * align_up(static_cast<size_t>(ns) * 4, 256);
}

int curve_sort(cudaStream_t stream, int64_t ns, const int32_t* idx, const double* x, const double* y,
                const double* z, double inv_a, void* scratch, size_t scratch_bytes, int32_t* sorted) {
  if (ns <= 0) return LPM_OK;
  size_t temp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, temp, static_cast<const uint32_t*>(nullptr), static_cast<uint32_t*>(nullptr),
                                  static_cast<const int32_t*>(nullptr), static_cast<int32_t*>(nullptr),
                                  static_cast<int>(ns), 0, 30);
  const size_t arr = align_up(static_cast<size_t>(ns) * 4, 256);
  if (scratch_bytes < align_up(temp, 256) + 3 * arr)
    return set_error(LPM_ERR_STATE, "curve sort scratch too small");
  char* base = static_cast<char*>(scratch);
  void* d_temp = base;
  uint32_t* keys_in = reinterpret_cast<uint32_t*>(base + align_up(temp, 256));
  uint32_t* keys_out = reinterpret_cast<uint32_t*>(base + align_up(temp, 256) + arr);
  int32_t* vals_in = reinterpret_cast<int32_t*>(base + align_up(temp, 256) + 2 * arr);
  curve_keys_kernel<<<static_cast<unsigned>(ceil_div(ns, 256)), 256, 0, stream>>>(ns, idx, x, y, z, inv_a, keys_in,
                                                                                   vals_in);
  LPM_CUDA_TRY(cudaGetLastError());
  LPM_CUDA_TRY(cub::DeviceRadixSort::SortPairs(d_temp, temp, keys_in, keys_out, vals_in, sorted,
                                               static_cast<int>(ns), 0, 30, stream));
  return LPM_OK;
}

// The box and the blocks' partial boxes at the head of the 2-D sort's scratch.
constexpr size_t kBoxBytes = 256 + 4 * kBoxBlocksMax * sizeof(double);

size_t curve_sort2d_bytes(int64_t ns) {
  size_t temp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, temp, static_cast<const uint32_t*>(nullptr), static_cast<uint32_t*>(nullptr),
                                  static_cast<const int32_t*>(nullptr), static_cast<int32_t*>(nullptr),
                                  static_cast<int>(ns), 0, 32);
  // boxes, then the CUB temporary, keys in/out and values in
  return kBoxBytes + align_up(temp, 256) + 3 * align_up(static_cast<size_t>(ns) * 4, 256);
}

int curve_sort2d(cudaStream_t stream, int64_t ns, const int32_t* idx, const double* x, const double* y,
                 void* scratch, size_t scratch_bytes, int32_t* sorted) {
  if (ns <= 0) return LPM_OK;
  size_t temp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, temp, static_cast<const uint32_t*>(nullptr), static_cast<uint32_t*>(nullptr),
                                  static_cast<const int32_t*>(nullptr), static_cast<int32_t*>(nullptr),
                                  static_cast<int>(ns), 0, 32);
  const size_t arr = align_up(static_cast<size_t>(ns) * 4, 256);
  if (scratch_bytes < kBoxBytes + align_up(temp, 256) + 3 * arr)
    return set_error(LPM_ERR_STATE, "2-D curve sort scratch too small");
  char* base = static_cast<char*>(scratch);
  double* box = reinterpret_cast<double*>(base);
  double* part = reinterpret_cast<double*>(base + 256);
  void* d_temp = base + kBoxBytes;
  uint32_t* keys_in = reinterpret_cast<uint32_t*>(base + kBoxBytes + align_up(temp, 256));
  uint32_t* keys_out = reinterpret_cast<uint32_t*>(base + kBoxBytes + align_up(temp, 256) + arr);
  int32_t* vals_in = reinterpret_cast<int32_t*>(base + kBoxBytes + align_up(temp, 256) + 2 * arr);
  const int nb = box_blocks(ns);
  bbox2d_partial_kernel<<<nb, kBoxThreads, 0, stream>>>(ns, idx, x, y, part);
  bbox2d_final_kernel<<<1, kBoxThreads, 0, stream>>>(nb, part, box);
  curve2d_keys_kernel<<<static_cast<unsigned>(ceil_div(ns, 256)), 256, 0, stream>>>(ns, idx, x, y, box, keys_in,
                                                                                    vals_in);
  LPM_CUDA_TRY(cudaGetLastError());
  LPM_CUDA_TRY(cub::DeviceRadixSort::SortPairs(d_temp, temp, keys_in, keys_out, vals_in, sorted,
                                               static_cast<int>(ns), 0, 32, stream));
  return LPM_OK;
}

namespace {
__global__ void mark_kernel(int64_t ns, const int32_t* idx, uint8_t* mask) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < ns) mask[idx[k]] = 1;
}

__global__ void gather_flags_kernel(int64_t n, const int32_t* order, const uint8_t* mask, uint8_t* flags) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) flags[k] = mask[order[k]];
}

size_t select_temp_bytes(int64_t n) {
  size_t temp = 0;
  cub::DeviceSelect::Flagged(nullptr, temp, static_cast<const int32_t*>(nullptr), static_cast<const uint8_t*>(nullptr),
                             static_cast<int32_t*>(nullptr), static_cast<int64_t*>(nullptr), static_cast<int>(n));
  return temp;
}
}  // namespace

size_t select_in_order_bytes(int64_t n) {
  // mask and flags (n bytes each), the selected count, then the CUB temporary
  return 2 * align_up(static_cast<size_t>(n), 256) + 256 + align_up(select_temp_bytes(n), 256);
}

int select_in_order(cudaStream_t stream, int64_t n, const int32_t* order, int64_t ns, const int32_t* idx,
                    void* scratch, size_t scratch_bytes, int32_t* out) {
  if (n <= 0 || ns <= 0) return LPM_OK;
  const size_t temp = select_temp_bytes(n);
  const size_t nb = align_up(static_cast<size_t>(n), 256);
  if (scratch_bytes < 2 * nb + 256 + align_up(temp, 256)) return set_error(LPM_ERR_STATE, "select scratch too small");
  char* base = static_cast<char*>(scratch);
  uint8_t* mask = reinterpret_cast<uint8_t*>(base);
  uint8_t* flags = reinterpret_cast<uint8_t*>(base + nb);
  int64_t* count = reinterpret_cast<int64_t*>(base + 2 * nb);
  void* d_temp = base + 2 * nb + 256;
  LPM_CUDA_TRY(cudaMemsetAsync(mask, 0, static_cast<size_t>(n), stream));
  mark_kernel<<<static_cast<unsigned>(ceil_div(ns, 256)), 256, 0, stream>>>(ns, idx, mask);
  gather_flags_kernel<<<static_cast<unsigned>(ceil_div(n, 256)), 256, 0, stream>>>(n, order, mask, flags);
  LPM_CUDA_TRY(cudaGetLastError());
  size_t tb = temp;
  LPM_CUDA_TRY(cub::DeviceSelect::Flagged(d_temp, tb, order, flags, out, count, static_cast<int>(n), stream));
  return LPM_OK;
}

}  // namespace lpm
