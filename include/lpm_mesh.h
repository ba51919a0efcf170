/*
 * lpm_mesh.h -- host-side workload generator: the uniformly refined lpm-v2 meshes.
 *
 * The direct sums take raw particle arrays; in lpm-v2 those arrays come from a PolyMesh2d
 * built by recursive refinement of a mesh seed (src/PolyMesh2d.f90:135-195).  This
 * generator restates that construction (seed tables, DivideTriFace, DivideQuadFace,
 * divideLinearEdge, face areas) so that benchmarks and tests run on the same particle
 * sets, in the same order, as the reference.  Adaptive refinement is not restated.
 * Host code only; it is not part of the GPU hot path.
 */
#ifndef LPM_MESH_H
#define LPM_MESH_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* seed identifiers, src/TypeDefs.f90:66-73 */
#define LPM_QUAD_RECT_SEED 202
#define LPM_ICOS_TRI_SPHERE_SEED 205
#define LPM_CUBED_SPHERE_SEED 206

typedef struct lpm_mesh lpm_mesh;

/* New(PolyMesh2d, meshSeed, initNest, maxNest, amrLimit=0, ampFactor),
 * src/PolyMesh2d.f90:135.  Returns 0 on success, a negative code on a bad argument. */
int lpm_mesh_create(lpm_mesh** mesh, int mesh_seed, int init_nest, double amp_factor);
void lpm_mesh_destroy(lpm_mesh* mesh);

int64_t lpm_mesh_n_particles(const lpm_mesh* mesh);
int64_t lpm_mesh_n_active(const lpm_mesh* mesh);
int64_t lpm_mesh_n_faces(const lpm_mesh* mesh);  /* all faces of the quadtree */
int64_t lpm_mesh_n_edges(const lpm_mesh* mesh);  /* all edges of the binary tree */
int64_t lpm_mesh_n_leaf_edges(const lpm_mesh* mesh);
int lpm_mesh_is_spherical(const lpm_mesh* mesh);

/* Copies the particle arrays (length n_particles).  z may be NULL for planar meshes
 * (planar particles have no z, src/Particles.f90:159-164); active is 1/0. */
int lpm_mesh_get_particles(const lpm_mesh* mesh, double* x, double* y, double* z,
                           double* area, int32_t* active);

/* MaxEdgeLength / AvgEdgeLength over leaf edges, src/Edges.f90:260-340 */
double lpm_mesh_max_edge_length(const lpm_mesh* mesh);
double lpm_mesh_avg_edge_length(const lpm_mesh* mesh);

#ifdef __cplusplus
}
#endif
#endif
