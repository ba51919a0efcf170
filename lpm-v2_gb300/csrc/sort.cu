// sort.cu -- spatial (Hilbert-curve) ordering of the source particles on the device.
//
// The FP32C sphere sweep stores every source relative to the origin of its group of 64, so
// groups must be spatially compact: sources are ordered by the 30-bit index, along a 3-D
// Hilbert curve over a 2^10 grid per axis, of the cell holding their unit-scaled position,
// with a device radix sort (CUB).  Consecutive Hilbert cells are face neighbours, so 64
// consecutive sources form one connected patch (a Hilbert-curve order jumps across the grid at
// its octant boundaries, which leaves some groups in two distant pieces).  The order only
// affects rounding (the FP32C sum is order-independent to its error bound); FP64 sums keep
// the reference's ascending order.
#include <cub/device/device_radix_sort.cuh>

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

// Bounding box {x_min, y_min, x_max, y_max} of the listed points: one block, a fixed order.
__global__ void __launch_bounds__(1024) bbox2d_kernel(int64_t ns, const int32_t* idx, const double* x,
                                                      const double* y, double* box) {
  __shared__ double r[4][1024];
  double a = 1e300, b = 1e300, c = -1e300, d = -1e300;
  for (int64_t k = threadIdx.x; k < ns; k += 1024) {
    const int32_t j = idx[k];
    a = fmin(a, x[j]);
    b = fmin(b, y[j]);
    c = fmax(c, x[j]);
    d = fmax(d, y[j]);
  }
  r[0][threadIdx.x] = a;
  r[1][threadIdx.x] = b;
  r[2][threadIdx.x] = c;
  r[3][threadIdx.x] = d;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      r[0][threadIdx.x] = fmin(r[0][threadIdx.x], r[0][threadIdx.x + w]);
      r[1][threadIdx.x] = fmin(r[1][threadIdx.x], r[1][threadIdx.x + w]);
      r[2][threadIdx.x] = fmax(r[2][threadIdx.x], r[2][threadIdx.x + w]);
      r[3][threadIdx.x] = fmax(r[3][threadIdx.x], r[3][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) box[threadIdx.x] = r[threadIdx.x][0];
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

size_t curve_sort2d_bytes(int64_t ns) {
  size_t temp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, temp, static_cast<const uint32_t*>(nullptr), static_cast<uint32_t*>(nullptr),
                                  static_cast<const int32_t*>(nullptr), static_cast<int32_t*>(nullptr),
                                  static_cast<int>(ns), 0, 32);
  // box, then the CUB temporary, keys in/out and values in
  return 256 + align_up(temp, 256) + 3 * align_up(static_cast<size_t>(ns) * 4, 256);
}

int curve_sort2d(cudaStream_t stream, int64_t ns, const int32_t* idx, const double* x, const double* y,
                 void* scratch, size_t scratch_bytes, int32_t* sorted) {
  if (ns <= 0) return LPM_OK;
  size_t temp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, temp, static_cast<const uint32_t*>(nullptr), static_cast<uint32_t*>(nullptr),
                                  static_cast<const int32_t*>(nullptr), static_cast<int32_t*>(nullptr),
                                  static_cast<int>(ns), 0, 32);
  const size_t arr = align_up(static_cast<size_t>(ns) * 4, 256);
  if (scratch_bytes < 256 + align_up(temp, 256) + 3 * arr)
    return set_error(LPM_ERR_STATE, "2-D curve sort scratch too small");
  char* base = static_cast<char*>(scratch);
  double* box = reinterpret_cast<double*>(base);
  void* d_temp = base + 256;
  uint32_t* keys_in = reinterpret_cast<uint32_t*>(base + 256 + align_up(temp, 256));
  uint32_t* keys_out = reinterpret_cast<uint32_t*>(base + 256 + align_up(temp, 256) + arr);
  int32_t* vals_in = reinterpret_cast<int32_t*>(base + 256 + align_up(temp, 256) + 2 * arr);
  bbox2d_kernel<<<1, 1024, 0, stream>>>(ns, idx, x, y, box);
  curve2d_keys_kernel<<<static_cast<unsigned>(ceil_div(ns, 256)), 256, 0, stream>>>(ns, idx, x, y, box, keys_in,
                                                                                    vals_in);
  LPM_CUDA_TRY(cudaGetLastError());
  LPM_CUDA_TRY(cub::DeviceRadixSort::SortPairs(d_temp, temp, keys_in, keys_out, vals_in, sorted,
                                               static_cast<int>(ns), 0, 32, stream));
  return LPM_OK;
}

}  // namespace lpm
