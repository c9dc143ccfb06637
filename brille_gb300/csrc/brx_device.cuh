// Device-side tables and FP64 predicates of the brille query path.
//
// Every decision that selects an index (G shift, wedge operation, trellis
// node, tetrahedron, which weights are kept) is computed in FP64 with
// explicitly rounded operations (__dmul_rn / __dadd_rn / __dsub_rn are never
// contracted into FMAs), in the same order as the reference's C++
// (src/geometry.hpp, src/bz_move.cpp, src/trellis_poly.hpp,
// src/trellis_node.hpp), so that indices match the CPU restatement bit for bit.
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

namespace brx {

struct Tol {
  double rel, abs_;
};

// approx_float::tols for (double, double) (src/approx_float.hpp:79-100)
inline Tol make_tol(double Ttol, int tol) {
  Tol t;
  t.rel = DBL_EPSILON;
  t.abs_ = 5.0 / 1000000000000000.0;
  t.rel *= (double)tol * (double)10000;
  if (Ttol > t.rel) t.rel = Ttol;
  if (Ttol > t.abs_) t.abs_ = Ttol;
  return t;
}

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// approx_float::_scalar, same-type floating point (src/approx_float.hpp:171-177)
__device__ __forceinline__ bool approx(double a, double b, Tol t) {
  double x = fabs(dsub(a, b));
  return x <= dadd(t.abs_, dmul(t.rel, fabs(dadd(a, b)))) || x < DBL_MIN;
}
__device__ __forceinline__ bool cmp_ge(double a, double b, Tol t) { return approx(a, b, t) || a > b; }
__device__ __forceinline__ bool cmp_le(double a, double b, Tol t) { return approx(a, b, t) || a < b; }
__device__ __forceinline__ bool cmp_gt(double a, double b, Tol t) { return !approx(a, b, t) && a > b; }

// Σ_k m[3i+k]·v[k] with integer m, accumulated from 0 in k order
__device__ __forceinline__ void matvec_i(double out[3], const int32_t* m, const double v[3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) s = dadd(s, dmul((double)m[3 * i + k], v[k]));
    out[i] = s;
  }
}
// xyz = to_xyz · hkl where B's rows are the basis vectors
__device__ __forceinline__ void hkl_to_xyz(double out[3], const double* B, const double h[3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) s = dadd(s, dmul(B[3 * k + i], h[k]));
    out[i] = s;
  }
}
__device__ __forceinline__ double dot3(const double* a, const double* b) {
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) s = dadd(s, dmul(a[i], b[i]));
  return s;
}
// pseudo_orient3d = dot(a-d, cross(b-d, c-d)) (src/geometry.hpp:118-139)
__device__ __forceinline__ double orient3d(const double* a, const double* b, const double* c, const double* d) {
  double u0 = dsub(a[0], d[0]), u1 = dsub(a[1], d[1]), u2 = dsub(a[2], d[2]);
  double v0 = dsub(b[0], d[0]), v1 = dsub(b[1], d[1]), v2 = dsub(b[2], d[2]);
  double w0 = dsub(c[0], d[0]), w1 = dsub(c[1], d[1]), w2 = dsub(c[2], d[2]);
  double x0 = dsub(dmul(v1, w2), dmul(v2, w1));
  double x1 = dsub(dmul(v2, w0), dmul(v0, w2));
  double x2 = dsub(dmul(v0, w1), dmul(v1, w0));
  double s = 0.0;
  s = dadd(s, dmul(u0, x0));
  s = dadd(s, dmul(u1, x1));
  s = dadd(s, dmul(u2, x2));
  return s;
}

// Device copy of brx_geometry with device pointers.
struct DevGeom {
  double outer_B[9], prim_B[9];
  int32_t to_prim_6Pt[9], from_prim_invPt[9];
  int32_t is_primitive;
  int32_t n_faces;
  const double* face_abc;
  const double* face_normal;
  const int32_t* face_tau;
  const double* face_tau_len;
  int32_t n_wedge;
  const double* wedge_normal;
  int32_t wedge_le_ge;
  int32_t n_ops;
  const int32_t* ops;
  const int32_t* op_inverse;
  int32_t identity;
  int32_t n_knots[3];
  const double* knots[3];
  int64_t n_nodes;
  const int32_t* node_type;
  const int32_t* node_index;
  int32_t n_cube;
  long long n_tets;
  const int32_t* cube_vertices;
  // cube nodes in Morton order of their (i, j, k): group keys follow it, so
  // the gathers visit nodes that share vertices close together in time
  const int32_t* cube_rank;   // cube index → rank
  const int32_t* poly_tet_offset;
  const int32_t* tet_vertices;
  const double* tet_sphere;
  const double* tet_volume;
  const double* vertex_xyz;
  int32_t n_atoms;
  const int32_t* gamma_F0;
  const int32_t* gamma_vidx;
  const double* gamma_vectors;
  const double* rot_cart;   // n_ops × 9: L·W·L⁻¹ for Cartesian Γ data
  // FP32 screens (see brx_locate.cu): face planes n̂·x ≤ h with the o3d
  // tolerance band expressed as a distance, and wedge normals carried back
  // through every operation, m_ji = B⁻¹ W_j B n_i.
  const float* face_plane32;   // n_faces × 4: n̂, h
  const float* face_band32;    // n_faces: width of the tolerance band in distance
  const float* wedge_m32;      // (n_ops + 1) × n_wedge × 3 (last block: identity)
  float wedge_band32;          // width of the wedge tolerance band
  const float* tet_plane32;    // n_tets × 4 × (a_x, a_y, a_z, c): barycentric w_j(x) = a_j·x + c_j
  int32_t screen;              // 0 disables the screens (exact FP64 everywhere)
  // Every cube's corner i sits at corner 0's or corner 7's coordinate on
  // each axis d, bit d of 3-bit field i of cube_pattern choosing corner 7:
  // the cube weights then take |x_d − a_d| and |x_d − b_d| once per axis.
  int32_t cube_canon;
  int32_t cube_pattern;
  Tol t_main;               // (float_tolerance, digit)
  Tol t_def;                // (0, 1): the reference's default comparisons
};

// Per-q records written by the locate kernel, structure-of-arrays.
struct Records {
  double* q_ir;     // n × 3
  int32_t* tau;     // n × 3
  int32_t* rot;     // n × 2: R, R⁻¹
  int32_t* node;    // n × 2: node, tetrahedron (−1 for cube nodes)
  int32_t* nw;      // n
  int32_t* vidx;    // n × 8
  double* w;        // n × 8
  float* w32;       // n × 8: the weights rounded once to FP32 (for the FP32 gathers)
  int32_t* status;  // n
  int32_t* key;     // n: gather group (cube node or tetrahedron, and pivot slot)
};

// Group key of a located q: the vertex set it interpolates from (a cube
// node's 8 corners in weight order, or one tetrahedron's 4 vertices) and the
// slot of its pivot (first) vertex.  q with equal keys share every vertex
// row and every antiphase factor of the gather.
__host__ __device__ inline long long n_group_keys(int32_t n_cube, long long n_tets) {
  return 8LL * n_cube + 4LL * n_tets;
}

// Error summary shared by all kernels of one query.
struct ErrorWord {
  int32_t flags;         // OR of (1 << status)
  int32_t count;         // number of failing q
  long long first_bad;   // smallest failing q index
};

}  // namespace brx
