// sums.cuh -- device-level launchers of the direct sums (shared by the host-buffer entry
// points and the device-resident solvers).  All pointers are device pointers; nothing here
// allocates, so the launches can be captured into CUDA graphs.
#pragma once

#include "lpm_common.cuh"

namespace lpm {

// Scratch layout of one direct-sum launch: compacted source records, then the split-K
// partial sums (FP32C only).
struct SumPlan {
  int64_t n_tiles = 0;       // source tiles (ns padded to a tile multiple)
  int64_t tiles_per_chunk = 0;
  int64_t nsplit = 1;        // split-K chunks (gridDim.y)
  size_t src_bytes = 0;      // bytes of the padded source-record array
  size_t partial_bytes = 0;  // bytes of the FP64 partial sums
  int shape = 0;             // sweep shape (sphere BVE FP32C; see bve_shape_count)
  int fp64_threads = 128;    // FP64 sequential sweep CTA size (32, 64 or 128: the best-balanced)
  bool fp64_small = false;   // fewer 128-thread CTAs than SMs: the split sweep where there is one
  int fp64_split_threads = 128;  // the split sweep's CTA size (32, 64 or 128)
  // a second sweep of the same job (the planar SWE surface-height Laplacian): its tiles and
  // split, its source records at src_buf + aux_src_offset; it reuses the partials
  int64_t aux_n_tiles = 0, aux_tiles_per_chunk = 0, aux_nsplit = 0;
  size_t aux_src_offset = 0;
  // FP32C PSE sums: the targets' curve order (two lists of nt int32: [ib, ib + nt) and its
  // sorted permutation) at src_buf + tperm_offset; 0 when the sweep takes targets in order
  size_t tperm_offset = 0;
};

enum SumKind : int {
  kSumBve = 0,        // sphere BVE velocity, BVESphereVelocity association
  kSumBveMesh,        // sphere BVE velocity, setVelocityFromVorticity association
  kSumPlane,          // planar Biot-Savart velocity
  kSumPseK8Geo,       // PSE Laplacian, K8 + great-circle distance
  kSumPseGaussChord,  // PSE Laplacian, Gaussian + chord distance
  kSumPseK8Chord,     // PSE Laplacian, K8 + chord distance (plane)
  kSumSphereStream,   // sphere stream functions
  kSumPlaneStream,    // planar stream function
  kSumPseGrad,        // PSE gradient on the sphere (K1 of the great-circle distance)
  kSumPseDiv,         // PSE divergence on the sphere
  kSumPsePlaneGrad,     // PSE gradient in the plane (FP64)
  kSumPsePlaneSecond,   // PSE second partials in the plane, from a gradient field (FP64)
  kSumPsePlaneDdot,     // PSE double dot product in the plane (FP64)
  kSumPseSphereDdot,    // PSE double dot product on the sphere (FP64)
  kSumPseInterpPlane,   // PSE interpolation at query points, chord distance (FP64)
  kSumPseInterpSphere,  // PSE interpolation at query points, great-circle distance (FP64)
  kSumSwePlane,         // planar SWE right-hand-side integrals (FP64)
  kSumSweSphere,        // sphere SWE right-hand-side integrals (FP64)
  kSumBetaPlane,        // beta-plane (x-periodic) velocity
  kSumBetaStream        // beta-plane stream functions (FP64)
};

// Kinds that have only the FP64 form.
inline bool sum_is_fp64_only(int kind) {
  return kind >= kSumPsePlaneGrad && kind <= kSumPseInterpSphere;
}

// Inputs of one direct sum over particles [0, n): sources are the ns particles listed (in
// ascending order) by src_idx; targets are particles ib .. ib+nt-1.
struct SumJob {
  int kind = kSumBve;
  int mode = LPM_MODE_FP64;  // LPM_MODE_FP64 or LPM_MODE_FP32C
  int64_t n = 0;
  const double *x = nullptr, *y = nullptr, *z = nullptr;
  const double* s1 = nullptr;  // zeta (BVE), omega (plane), f (PSE), relvort (stream)
  const double* s2 = nullptr;  // absvort (sphere stream), vy (PSE divergence), unused otherwise
  const double* s3 = nullptr;  // vz (PSE divergence), w (sphere double dot), surface height (SWE)
  const double* area = nullptr;
  const int32_t* src_idx = nullptr;
  int64_t ns = 0;
  double radius = 1.0;  // sphere radius (BVE, PSE, stream)
  double delta = 0.0;   // planar regularisation
  double eps = 1.0;     // PSE radius
  double radius2 = 1.0;  // SphereRadius of SphereDistance in the sphere SWE integrals
  int64_t ib = 0, nt = 0;
  double* out0 = nullptr;  // u / lap / psi_rel   (length nt)
  double* out1 = nullptr;  // v / psi_abs
  double* out2 = nullptr;  // w
  double* out3 = nullptr;  // lapSurf (SWE)
  // FP32C sphere BVE and planar sums: curve-sort src_idx into `sorted` with this scratch
  // before the sweep (sort_scratch == nullptr: src_idx is already spatially ordered and is
  // used as is)
  void* sort_scratch = nullptr;
  size_t sort_bytes = 0;
  int32_t* sorted = nullptr;
  // scratch (sizes from plan_sum)
  void* src_buf = nullptr;
  double* partial = nullptr;
  int* status = nullptr;
  cudaStream_t stream = nullptr;
  WaitCfg wait = default_wait();  // limits of the sweep's bounded waits (sphere BVE FP32C)
};

// Split-K factor for a sweep of `blocks` target blocks over `tiles` source tiles on `slots`
// resident CTA slots (SMs x CTAs per SM): the nsplit <= max_split that minimises
// waves x (tiles per chunk + one tile of per-CTA cost), where waves = ceil(blocks x nsplit /
// slots).  Equal-length CTAs run in lock-step waves, so a grid of 1.3 waves costs 2; this
// picks a split whose last wave is nearly full.  Ties go to the smaller split.
int64_t choose_split(int64_t blocks, int64_t tiles, int64_t slots, int64_t max_split);

// Decides tiles, split-K and (for the sphere BVE FP32C sweep) the CTA shape of a job on a
// device with sm_count SMs.
SumPlan plan_sum(int kind, int mode, int64_t ns, int64_t nt, int sm_count, int shape = 0);

// Number of sweep shapes of the sphere BVE FP32C sum.
int bve_shape_count();

// Autotuner: the shape of the sphere BVE FP32C sweep for a problem size, chosen once per
// size class by timing every shape on the job (its targets limited to a bounded subset) and
// cached for the process.  `job` must hold scratch sized for plan_sum_max(); results of the
// timing runs land in job.out*.  Returns the shape in *shape.
int autotune_bve_shape(const SumJob& job, int sm_count, int* shape);
// Plan with the largest scratch over all shapes (for allocating before tuning).
SumPlan plan_sum_max(int kind, int mode, int64_t ns, int64_t nt, int sm_count);
// Enqueues prep + sweep (+ finish) on job.stream.
int launch_sum(const SumJob& job, const SumPlan& plan);

// Whether the FP32C form of `kind` runs on curve-sorted, group-relative sources, and the
// scratch bytes of that sort for ns sources.
bool sum_uses_sorted_sources(int kind, int mode);
size_t sort_scratch_bytes(int kind, int64_t ns, int64_t nt);

}  // namespace lpm
