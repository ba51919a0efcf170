// mesh.cpp -- uniformly refined lpm-v2 meshes (host-side workload generator).
//
// Restates the mesh construction of lpm-v2 so the direct sums see the reference's particle
// sets, in the reference's order:
//   seed reading + initialisation   src/PolyMesh2d.f90:795-939
//   uniform refinement loop         src/PolyMesh2d.f90:179-190
//   DivideTriFace / DivideQuadFace  src/Faces.f90:701-858, :529-689
//   divideLinearEdge                src/Edges.f90:567-617
//   TriFaceArea / QuadFaceArea      src/Faces.f90:917-975
//   sphere/plane geometry helpers   src/SphereGeometry.f90:67-366, src/PlaneGeometry.f90
// Indices are 1-based internally (element 0 unused) because the refinement logic compares
// face indices stored in edges, exactly as the Fortran does.  Compiled with
// -ffp-contract=off so each product and sum rounds where the Fortran source rounds it.
#include "lpm_mesh.h"

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

namespace {

const double kPi = 3.1415926535897932384626433832795027975;

struct Vec3 {
  double x, y, z;
};

// ---------------------------------------------------------------- seed tables
// The seed connectivity has to match the reference's seed files exactly, because it fixes
// the particle insertion order of every later refinement level.  Values are those of
// icosTriSeed.dat, cubedSphereSeed.dat and quadRectSeed.dat (0-based, as in the files).

const double kIcosVerts[12][3] = {
    {0.0, 0.0, 1.0},
    {0.723606797749978969640917366873, 0.525731112119133606025669084848, 0.447213595499957939281834733746},
    {-0.276393202250021030359082633126, 0.850650808352039932181540497063, 0.447213595499957939281834733746},
    {-0.894427190999915878563669467492, 0.0, 0.447213595499957939281834733746},
    {-0.276393202250021030359082633127, -0.850650808352039932181540497063, 0.447213595499957939281834733746},
    {0.723606797749978969640917366873, -0.525731112119133606025669084848, 0.447213595499957939281834733746},
    {0.894427190999915878563669467492, 0.0, -0.447213595499957939281834733746},
    {0.276393202250021030359082633127, 0.850650808352039932181540497063, -0.447213595499957939281834733746},
    {-0.723606797749978969640917366873, 0.525731112119133606025669084848, -0.447213595499957939281834733746},
    {-0.723606797749978969640917366873, -0.525731112119133606025669084848, -0.447213595499957939281834733746},
    {0.276393202250021030359082633127, -0.850650808352039932181540497063, -0.447213595499957939281834733746},
    {0.0, 0.0, -1.0}};
const int kIcosEdges[30][4] = {
    {0, 1, 0, 4},   {1, 2, 0, 6},    {2, 0, 0, 1},    {2, 3, 1, 8},    {0, 3, 2, 1},
    {3, 4, 2, 10},  {4, 0, 2, 3},    {4, 5, 3, 12},   {5, 0, 3, 4},    {5, 1, 4, 14},
    {1, 6, 5, 14},  {6, 7, 5, 15},   {7, 1, 5, 6},    {7, 2, 6, 7},    {7, 8, 7, 16},
    {8, 2, 7, 8},   {8, 3, 8, 9},    {8, 9, 9, 17},   {3, 9, 10, 9},   {9, 4, 10, 11},
    {9, 10, 11, 18}, {10, 4, 11, 12}, {10, 5, 12, 13}, {10, 6, 13, 19}, {6, 5, 13, 14},
    {11, 6, 19, 15}, {11, 7, 15, 16}, {8, 11, 17, 16}, {11, 9, 17, 18}, {10, 11, 19, 18}};
const int kIcosFaceVerts[20][3] = {{0, 1, 2},   {0, 2, 3},  {0, 3, 4},  {0, 4, 5},   {0, 5, 1},
                                   {1, 6, 7},   {7, 2, 1},  {2, 7, 8},  {8, 3, 2},   {3, 8, 9},
                                   {9, 4, 3},   {4, 9, 10}, {10, 5, 4}, {5, 10, 6},  {6, 1, 5},
                                   {11, 7, 6},  {11, 8, 7}, {11, 9, 8}, {11, 10, 9}, {11, 6, 10}};
const int kIcosFaceEdges[20][3] = {{0, 1, 2},    {2, 3, 4},    {4, 5, 6},    {6, 7, 8},
                                   {8, 9, 0},    {10, 11, 12}, {13, 1, 12},  {13, 14, 15},
                                   {16, 3, 15},  {16, 17, 18}, {19, 5, 18},  {19, 20, 21},
                                   {22, 7, 21},  {22, 23, 24}, {10, 9, 24},  {26, 11, 25},
                                   {27, 14, 26}, {28, 17, 27}, {29, 20, 28}, {25, 23, 29}};

const double kCubeXYZ[14][3] = {
    {0.577350269189626, -0.577350269189626, 0.577350269189626},
    {0.577350269189626, -0.577350269189626, -0.577350269189626},
    {0.577350269189626, 0.577350269189626, -0.577350269189626},
    {0.577350269189626, 0.577350269189626, 0.577350269189626},
    {-0.577350269189626, 0.577350269189626, -0.577350269189626},
    {-0.577350269189626, 0.577350269189626, 0.577350269189626},
    {-0.577350269189626, -0.577350269189626, -0.577350269189626},
    {-0.577350269189626, -0.577350269189626, 0.577350269189626},
    {1.0, 0.0, 0.0},
    {0.0, 1.0, 0.0},
    {-1.0, 0.0, 0.0},
    {0.0, -1.0, 0.0},
    {0.0, 0.0, 1.0},
    {0.0, 0.0, -1.0}};
const int kCubeEdges[12][4] = {{0, 1, 0, 3}, {1, 2, 0, 6}, {2, 3, 0, 1}, {3, 0, 0, 4},
                               {2, 4, 1, 5}, {4, 5, 1, 2}, {5, 3, 1, 4}, {4, 6, 2, 5},
                               {6, 7, 2, 3}, {7, 5, 2, 4}, {6, 1, 3, 5}, {0, 7, 3, 4}};
const int kCubeFaceVerts[6][4] = {{0, 1, 2, 3}, {3, 2, 4, 5}, {5, 4, 6, 7},
                                  {7, 6, 1, 0}, {7, 0, 3, 5}, {1, 6, 4, 2}};
const int kCubeFaceEdges[6][4] = {{0, 1, 2, 3}, {2, 4, 5, 6}, {5, 7, 8, 9},
                                  {8, 10, 0, 11}, {11, 3, 6, 9}, {10, 7, 4, 1}};

const double kQuadXY[13][2] = {{-1.0, 1.0},  {-1.0, 0.0}, {-1.0, -1.0}, {0.0, -1.0}, {1.0, -1.0},
                               {1.0, 0.0},   {1.0, 1.0},  {0.0, 1.0},   {0.0, 0.0},  {-0.5, 0.5},
                               {-0.5, -0.5}, {0.5, -0.5}, {0.5, 0.5}};
const int kQuadEdges[12][4] = {{0, 1, 0, -1}, {1, 2, 1, -1}, {2, 3, 1, -1}, {3, 4, 2, -1},
                               {4, 5, 2, -1}, {5, 6, 3, -1}, {6, 7, 3, -1}, {7, 0, 0, -1},
                               {1, 8, 0, 1},  {8, 5, 3, 2},  {3, 8, 1, 2},  {8, 7, 0, 3}};
const int kQuadFaceVerts[4][4] = {{0, 1, 8, 7}, {1, 2, 3, 8}, {8, 3, 4, 5}, {7, 8, 5, 6}};
const int kQuadFaceEdges[4][4] = {{0, 8, 11, 7}, {1, 2, 10, 8}, {10, 3, 4, 9}, {11, 9, 5, 6}};

// ---------------------------------------------------------------- geometry
// Each helper follows the Fortran expression order (intrinsic sum() is a left-to-right sum).

double sum3sq(const Vec3& a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }

// SphereArcLengthVector, SphereGeometry.f90:141-160
double arc_length(const Vec3& a, const Vec3& b) {
  const double c1 = a.y * b.z - b.y * a.z;
  const double c2 = b.x * a.z - a.x * b.z;
  const double c3 = a.x * b.y - b.x * a.y;
  const double cn = std::sqrt((c1 * c1 + c2 * c2) + c3 * c3);
  const double dp = (a.x * b.x + a.y * b.y) + a.z * b.z;
  return std::atan2(cn, dp);
}

// SphereTriAreaVector, SphereGeometry.f90:347-366 (SphereRadius = radius)
double sphere_tri_area(const Vec3& a, const Vec3& b, const Vec3& c, double radius) {
  const double s1 = arc_length(a, b);
  const double s2 = arc_length(b, c);
  const double s3 = arc_length(c, a);
  const double hp = ((s1 + s2) + s3) / 2.0;
  const double zz = ((std::tan(hp / 2.0) * std::tan((hp - s1) / 2.0)) * std::tan((hp - s2) / 2.0)) *
                    std::tan((hp - s3) / 2.0);
  return ((4.0 * std::atan2(std::sqrt(zz), 1.0)) * radius) * radius;
}

// TriArea, PlaneGeometry.f90 (2-d shoelace form)
double plane_tri_area(const Vec3& a, const Vec3& b, const Vec3& c) {
  const double s = ((((-(b.x * a.y) + c.x * a.y) + a.x * b.y) - c.x * b.y) - a.x * c.y) + b.x * c.y;
  return 0.5 * std::fabs(s);
}

Vec3 normalise_to(const Vec3& c, double radius) {
  const double nrm = std::sqrt(sum3sq(c));
  return Vec3{(c.x / nrm) * radius, (c.y / nrm) * radius, (c.z / nrm) * radius};
}

// SphereMidpoint, SphereGeometry.f90:280-288
Vec3 sphere_midpoint(const Vec3& a, const Vec3& b, double radius) {
  return normalise_to(Vec3{(a.x + b.x) / 2.0, (a.y + b.y) / 2.0, (a.z + b.z) / 2.0}, radius);
}
// SphereTriCenter, SphereGeometry.f90:302-310
Vec3 sphere_tri_center(const Vec3& a, const Vec3& b, const Vec3& c, double radius) {
  return normalise_to(Vec3{((a.x + b.x) + c.x) / 3.0, ((a.y + b.y) + c.y) / 3.0,
                           ((a.z + b.z) + c.z) / 3.0},
                      radius);
}
// SphereQuadCenter, SphereGeometry.f90:325-333
Vec3 sphere_quad_center(const Vec3& a, const Vec3& b, const Vec3& c, const Vec3& d,
                        double radius) {
  return normalise_to(Vec3{(((a.x + b.x) + c.x) + d.x) / 4.0, (((a.y + b.y) + c.y) + d.y) / 4.0,
                           (((a.z + b.z) + c.z) + d.z) / 4.0},
                      radius);
}

}  // namespace

struct lpm_mesh {
  int seed = 0;
  int face_kind = 0;  // 3 or 4
  bool sphere = false;
  double radius = 1.0;  // SphereRadius used by the sphere geometry helpers
  // particles (1-based)
  std::vector<double> x, y, z, area;
  std::vector<char> active;
  // edges (1-based)
  std::vector<int> eorig, edest, eleft, eright, echild1, echild2;
  std::vector<char> ehas;
  // faces (1-based)
  std::vector<int> fcenter;
  std::vector<int> fverts, fedges;  // 4 slots per face, slot s of face f at 4*f + s (s 1-based -> s-1)
  std::vector<char> fhas;

  int np() const { return (int)x.size() - 1; }
  int ne() const { return (int)eorig.size() - 1; }
  int nf() const { return (int)fcenter.size() - 1; }

  Vec3 coord(int i) const { return Vec3{x[i], y[i], sphere ? z[i] : 0.0}; }

  int insert_particle(const Vec3& p) {  // InsertParticle, Particles.f90:497-517 (passive)
    x.push_back(p.x);
    y.push_back(p.y);
    z.push_back(sphere ? p.z : 0.0);
    area.push_back(0.0);
    active.push_back(0);
    return np();
  }
  int insert_edge(int o, int d, int l, int r) {  // insertPrivate, Edges.f90:211-233
    eorig.push_back(o);
    edest.push_back(d);
    eleft.push_back(l);
    eright.push_back(r);
    echild1.push_back(0);
    echild2.push_back(0);
    ehas.push_back(0);
    return ne();
  }
  int& fv(int f, int s) { return fverts[4 * f + (s - 1)]; }
  int& fe(int f, int s) { return fedges[4 * f + (s - 1)]; }
  int new_face() {
    fcenter.push_back(0);
    for (int s = 0; s < 4; ++s) {
      fverts.push_back(0);
      fedges.push_back(0);
    }
    fhas.push_back(0);
    return nf();
  }

  // divideLinearEdge, Edges.f90:567-617
  void divide_edge(int e) {
    const Vec3 v0 = coord(eorig[e]);
    const Vec3 v1 = coord(edest[e]);
    Vec3 mid;
    if (sphere) {
      mid = sphere_midpoint(v0, v1, radius);
    } else {
      mid = Vec3{0.5 * (v0.x + v1.x), 0.5 * (v0.y + v1.y), 0.0};
    }
    const int p = insert_particle(mid);
    const int orig = eorig[e], dest = edest[e], l = eleft[e], r = eright[e];
    const int c1 = insert_edge(orig, p, l, r);
    // Edges.f90:612 assigns rightFace(N+1) twice and never rightFace(N+2); child 2 keeps
    // the zero it was allocated with until the neighbouring face division sets it.
    const int c2 = insert_edge(p, dest, l, 0);
    ehas[e] = 1;
    echild1[e] = c1;
    echild2[e] = c2;
  }

  double face_area(int f) {  // TriFaceArea / QuadFaceArea, Faces.f90:917-975
    const Vec3 c = coord(fcenter[f]);
    double a = 0.0;
    for (int s = 1; s <= face_kind; ++s) {
      const Vec3 v1 = coord(fv(f, s));
      const Vec3 v2 = coord(fv(f, s % face_kind + 1));
      a = a + (sphere ? sphere_tri_area(v1, c, v2, radius) : plane_tri_area(v1, c, v2));
    }
    return a;
  }

  // DivideTriFace (Faces.f90:701-858) and DivideQuadFace (:529-689)
  void divide_face(int f) {
    const int nk = face_kind;
    int nv[5][5] = {};  // nv[slot][child]
    int nedge[5][5] = {};
    const int nf0 = nf();
    for (int i = 1; i <= nk; ++i) nv[i][i] = fv(f, i);
    for (int i = 1; i <= nk; ++i) {
      const int pe = fe(f, i);
      int c1, c2;
      if (ehas[pe]) {
        c1 = echild1[pe];
        c2 = echild2[pe];
      } else {
        c1 = ne() + 1;
        c2 = ne() + 2;
        divide_edge(pe);
      }
      const int inext = i % nk + 1;
      if (eleft[pe] == f) {  // positiveEdge, Edges.f90:678-685
        nedge[i][i] = c1;
        eleft[c1] = nf0 + i;
        nedge[i][inext] = c2;
        eleft[c2] = nf0 + inext;
      } else {
        nedge[i][i] = c2;
        eright[c2] = nf0 + i;
        nedge[i][inext] = c1;
        eright[c1] = nf0 + inext;
      }
      nv[inext][i] = edest[c1];
      nv[i][inext] = edest[c1];
    }
    if (nk == 3) {
      nv[1][4] = nv[3][2];
      nv[2][4] = nv[1][3];
      nv[3][4] = nv[2][1];
      int e = insert_edge(nv[1][4], nv[2][4], nf0 + 4, nf0 + 3);
      nedge[1][4] = e;
      nedge[1][3] = e;
      e = insert_edge(nv[2][4], nv[3][4], nf0 + 4, nf0 + 1);
      nedge[2][4] = e;
      nedge[2][1] = e;
      e = insert_edge(nv[3][4], nv[1][4], nf0 + 4, nf0 + 2);
      nedge[3][4] = e;
      nedge[3][2] = e;
    } else {
      const int pc = fcenter[f];
      for (int i = 1; i <= 4; ++i) nv[(i + 1) % 4 + 1][i] = pc;
      int e = insert_edge(nv[2][1], nv[3][1], nf0 + 1, nf0 + 2);
      nedge[2][1] = e;
      nedge[4][2] = e;
      e = insert_edge(nv[1][3], nv[4][3], nf0 + 4, nf0 + 3);
      nedge[4][3] = e;
      nedge[2][4] = e;
      e = insert_edge(nv[3][2], nv[4][2], nf0 + 2, nf0 + 3);
      nedge[3][2] = e;
      nedge[1][3] = e;
      e = insert_edge(nv[2][4], nv[1][4], nf0 + 1, nf0 + 4);
      nedge[1][4] = e;
      nedge[3][1] = e;
    }
    // child centres, computed for all 4 children from the slot-ordered vertices
    Vec3 centers[5];
    for (int c = 1; c <= 4; ++c) {
      const Vec3 a = coord(nv[1][c]), b = coord(nv[2][c]), d = coord(nv[3][c]);
      if (nk == 3) {
        if (sphere) {
          centers[c] = sphere_tri_center(a, b, d, radius);
        } else {
          centers[c] = Vec3{((a.x + b.x) + d.x) / 3.0, ((a.y + b.y) + d.y) / 3.0, 0.0};
        }
      } else {
        const Vec3 e4 = coord(nv[4][c]);
        if (sphere) {
          centers[c] = sphere_quad_center(a, b, d, e4, radius);
        } else {
          centers[c] = Vec3{0.25 * (((a.x + b.x) + d.x) + e4.x), 0.25 * (((a.y + b.y) + d.y) + e4.y), 0.0};
        }
      }
    }
    const int nnew = (nk == 3) ? 3 : 4;
    for (int c = 1; c <= nnew; ++c) {
      const int p = insert_particle(centers[c]);
      active[p] = 1;
      const int cf = new_face();
      fcenter[cf] = p;
      for (int s = 1; s <= nk; ++s) {
        fv(cf, s) = nv[s][c];
        fe(cf, s) = nedge[s][c];
      }
      area[p] = face_area(cf);
    }
    if (nk == 3) {
      // child 4 reuses the parent's centre particle (its position is not moved)
      const int cf = new_face();
      fcenter[cf] = fcenter[f];
      for (int s = 1; s <= 3; ++s) {
        fv(cf, s) = nv[s][4];
        fe(cf, s) = nedge[s][4];
      }
      area[fcenter[cf]] = face_area(cf);
    } else {
      active[fcenter[f]] = 0;  // MakeParticlePassive
      area[fcenter[f]] = 0.0;
    }
    fhas[f] = 1;
  }

  double edge_length(int e) const {  // EdgeLength, Edges.f90:282-297
    const Vec3 a = coord(eorig[e]), b = coord(edest[e]);
    if (sphere) {
      const double c1 = a.y * b.z - b.y * a.z;
      const double c2 = b.x * a.z - a.x * b.z;
      const double c3 = a.x * b.y - b.x * a.y;
      const double cn = std::sqrt((c1 * c1 + c2 * c2) + c3 * c3);
      const double dp = (a.x * b.x + a.y * b.y) + a.z * b.z;
      return std::atan2(cn, dp) * radius;
    }
    const double d1 = b.x - a.x, d2 = b.y - a.y, d3 = b.z - a.z;
    return std::sqrt((d1 * d1 + d2 * d2) + d3 * d3);
  }
};

extern "C" {

int lpm_mesh_create(lpm_mesh** out, int seed, int init_nest, double amp) {
  if (!out) return -1;
  *out = nullptr;
  if (init_nest < 0 || init_nest > 11) return -1;
  if (seed != LPM_ICOS_TRI_SPHERE_SEED && seed != LPM_CUBED_SPHERE_SEED && seed != LPM_QUAD_RECT_SEED)
    return -1;
  if (!(amp > 0.0)) return -1;
  lpm_mesh* m = new (std::nothrow) lpm_mesh();
  if (!m) return -5;
  m->seed = seed;
  m->sphere = (seed != LPM_QUAD_RECT_SEED);
  m->face_kind = (seed == LPM_ICOS_TRI_SPHERE_SEED) ? 3 : 4;
  m->radius = 1.0;  // SphereRadius (TypeDefs.f90:74) keeps its default 1.0 in the drivers
  // element 0 placeholders
  m->x.assign(1, 0.0);
  m->y.assign(1, 0.0);
  m->z.assign(1, 0.0);
  m->area.assign(1, 0.0);
  m->active.assign(1, 0);
  m->eorig.assign(1, 0);
  m->edest.assign(1, 0);
  m->eleft.assign(1, 0);
  m->eright.assign(1, 0);
  m->echild1.assign(1, 0);
  m->echild2.assign(1, 0);
  m->ehas.assign(1, 0);
  m->fcenter.assign(1, 0);
  m->fverts.assign(4, 0);
  m->fedges.assign(4, 0);
  m->fhas.assign(1, 0);

  // initializeMeshFromSeed, PolyMesh2d.f90:805-939
  std::vector<Vec3> xyz;
  int n_verts = 0, n_faces = 0;
  if (seed == LPM_ICOS_TRI_SPHERE_SEED) {
    n_verts = 12;
    n_faces = 20;
    for (int i = 0; i < 12; ++i) xyz.push_back(Vec3{kIcosVerts[i][0], kIcosVerts[i][1], kIcosVerts[i][2]});
    for (int f = 0; f < 20; ++f) {
      xyz.push_back(sphere_tri_center(xyz[kIcosFaceVerts[f][0]], xyz[kIcosFaceVerts[f][1]],
                                      xyz[kIcosFaceVerts[f][2]], m->radius));
    }
  } else if (seed == LPM_CUBED_SPHERE_SEED) {
    n_verts = 8;
    n_faces = 6;
    for (int i = 0; i < 14; ++i) xyz.push_back(Vec3{kCubeXYZ[i][0], kCubeXYZ[i][1], kCubeXYZ[i][2]});
  } else {
    n_verts = 9;
    n_faces = 4;
    for (int i = 0; i < 13; ++i) xyz.push_back(Vec3{kQuadXY[i][0], kQuadXY[i][1], 0.0});
  }
  for (auto& p : xyz) p = Vec3{amp * p.x, amp * p.y, amp * p.z};  // seedXYZ = ampFactor*seedXYZ
  for (const auto& p : xyz) m->insert_particle(p);
  const int n_edges = (seed == LPM_ICOS_TRI_SPHERE_SEED) ? 30 : 12;
  for (int e = 0; e < n_edges; ++e) {
    const int* row = (seed == LPM_ICOS_TRI_SPHERE_SEED) ? kIcosEdges[e]
                     : (seed == LPM_CUBED_SPHERE_SEED)  ? kCubeEdges[e]
                                                        : kQuadEdges[e];
    m->insert_edge(row[0] + 1, row[1] + 1, row[2] + 1, row[3] + 1);
  }
  for (int f = 0; f < n_faces; ++f) {
    const int cf = m->new_face();
    m->fcenter[cf] = n_verts + f + 1;
    for (int s = 1; s <= m->face_kind; ++s) {
      int v, e;
      if (seed == LPM_ICOS_TRI_SPHERE_SEED) {
        v = kIcosFaceVerts[f][s - 1];
        e = kIcosFaceEdges[f][s - 1];
      } else if (seed == LPM_CUBED_SPHERE_SEED) {
        v = kCubeFaceVerts[f][s - 1];
        e = kCubeFaceEdges[f][s - 1];
      } else {
        v = kQuadFaceVerts[f][s - 1];
        e = kQuadFaceEdges[f][s - 1];
      }
      m->fv(cf, s) = v + 1;
      m->fe(cf, s) = e + 1;
    }
    m->active[n_verts + f + 1] = 1;  // MakeParticleActive
  }
  for (int f = 1; f <= n_faces; ++f) m->area[m->fcenter[f]] = m->face_area(f);

  // uniform refinement, PolyMesh2d.f90:179-190
  int start = 1;
  for (int level = 1; level <= init_nest; ++level) {
    const int nold = m->nf();
    for (int f = start; f <= nold; ++f) m->divide_face(f);
    start = nold + 1;
  }
  *out = m;
  return 0;
}

void lpm_mesh_destroy(lpm_mesh* m) { delete m; }

int64_t lpm_mesh_n_particles(const lpm_mesh* m) { return m ? m->np() : 0; }
int64_t lpm_mesh_n_active(const lpm_mesh* m) {
  if (!m) return 0;
  int64_t c = 0;
  for (int i = 1; i <= m->np(); ++i) c += m->active[i] ? 1 : 0;
  return c;
}
int64_t lpm_mesh_n_faces(const lpm_mesh* m) { return m ? m->nf() : 0; }
int64_t lpm_mesh_n_edges(const lpm_mesh* m) { return m ? m->ne() : 0; }
int64_t lpm_mesh_n_leaf_edges(const lpm_mesh* m) {
  if (!m) return 0;
  int64_t c = 0;
  for (int e = 1; e <= m->ne(); ++e) c += m->ehas[e] ? 0 : 1;
  return c;
}
int lpm_mesh_is_spherical(const lpm_mesh* m) { return m && m->sphere ? 1 : 0; }

int lpm_mesh_get_particles(const lpm_mesh* m, double* x, double* y, double* z, double* area,
                           int32_t* active) {
  if (!m) return -1;
  const int n = m->np();
  for (int i = 1; i <= n; ++i) {
    if (x) x[i - 1] = m->x[i];
    if (y) y[i - 1] = m->y[i];
    if (z) z[i - 1] = m->z[i];
    if (area) area[i - 1] = m->area[i];
    if (active) active[i - 1] = m->active[i] ? 1 : 0;
  }
  return 0;
}

double lpm_mesh_max_edge_length(const lpm_mesh* m) {
  if (!m) return 0.0;
  double mx = 0.0;
  for (int e = 1; e <= m->ne(); ++e) {
    if (m->ehas[e]) continue;
    const double t = m->edge_length(e);
    if (t > mx) mx = t;
  }
  return mx;
}

double lpm_mesh_avg_edge_length(const lpm_mesh* m) {
  if (!m) return 0.0;
  double s = 0.0;
  int64_t nl = 0;
  for (int e = 1; e <= m->ne(); ++e) {
    if (m->ehas[e]) continue;
    s = s + m->edge_length(e);
    ++nl;
  }
  return nl ? s / (double)nl : 0.0;
}

}  // extern "C"
