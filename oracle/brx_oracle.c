/*
 * brx_oracle.c — CPU oracle for the brille query path.  TEST INFRASTRUCTURE.
 *
 * This file restates, in plain C over the flat tables of include/brx.h, the
 * reference's FP64 algorithm for BrillouinZoneTrellis3::ir_interpolate_at and
 * interpolate_at.  It is the checker for the CUDA path: only tests, the smoke
 * check and the CPU-baseline leg of the benchmark load it.  The product never
 * calls it, and the product has no CPU fallback.
 *
 * Parity pinning: the reference itself cannot be built here (it needs the
 * HighFive/HDF5 library, which is absent, and a CMake-generated header), so
 * this restatement is pinned by the reference's own golden fixture
 * (wrap/tests/test_5_gamma.npz: NaCl, 48 symmetry images, 24 modes) and by its
 * known-answer tests (linear fields reproduced exactly, Q = q + τ with q inside
 * the zone).
 *
 * Arithmetic follows the reference operation by operation (build with
 * -ffp-contract=off so that no multiply-add is fused); geometry that the
 * reference evaluates through lattice metrics is evaluated here on Cartesian
 * coordinates, which is the same quantity up to rounding.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/brx.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#define TWO_PI 6.283185307179586476925286766559

/* ---------------------------------------------------------------------------
 * approx_float (src/approx_float.hpp:79-100, 171-177, 202-205)
 * ------------------------------------------------------------------------- */
typedef struct { double rel, abs_; } tol_t;

static tol_t tols(double Ttol, int tol) {
  tol_t t;
  t.rel = DBL_EPSILON;
  t.abs_ = 5.0 / 1000000000000000.0;
  t.rel *= (double)tol * (double)10000;
  if (Ttol > t.rel) t.rel = Ttol;
  if (Ttol > t.abs_) t.abs_ = Ttol;
  return t;
}

static int approx(double a, double b, tol_t t) {
  double x = fabs(a - b);
  return x <= t.abs_ + t.rel * fabs(a + b) || x < DBL_MIN;
}

/* Comparer(cmp::ge) and cmp::le (src/comparisons.hpp:84-91) */
static int cmp_ge(double a, double b, tol_t t) { return approx(a, b, t) || a > b; }
static int cmp_le(double a, double b, tol_t t) { return approx(a, b, t) || a < b; }
static int cmp_gt(double a, double b, tol_t t) { return !approx(a, b, t) && a > b; }

/* ---------------------------------------------------------------------------
 * small vector helpers, in the reference's summation order
 * ------------------------------------------------------------------------- */
/* multiply_matrix_vector / mul_arrays (src/utilities.tpp:48-55) */
static void matvec_i(double out[3], const int32_t m[9], const double v[3]) {
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s += (double)m[3 * i + k] * v[k];
    out[i] = s;
  }
}
/* xyz = to_xyz · hkl with to_xyz columns the basis vectors
 * (src/array_lvec_methods.tpp:41-50); B rows are the basis vectors */
static void hkl_to_xyz(double out[3], const double B[9], const double h[3]) {
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s += B[3 * k + i] * h[k];
    out[i] = s;
  }
}
static double dot3(const double* a, const double* b) {
  double s = 0.0;
  for (int i = 0; i < 3; ++i) s += a[i] * b[i];
  return s;
}
/* pseudo_orient3d: dot(a-d, cross(b-d, c-d)) (src/geometry.hpp:118-139) */
static double orient3d(const double* a, const double* b, const double* c, const double* d) {
  double u[3], v[3], w[3], x[3];
  for (int i = 0; i < 3; ++i) { u[i] = a[i] - d[i]; v[i] = b[i] - d[i]; w[i] = c[i] - d[i]; }
  x[0] = v[1] * w[2] - v[2] * w[1];
  x[1] = v[2] * w[0] - v[0] * w[2];
  x[2] = v[0] * w[1] - v[1] * w[0];
  return dot3(u, x);
}

/* point_inside_all_planes (src/geometry.hpp:414-418): the smallest orient3d
 * over all faces, then `> 0 || ≈ 0` with (float_tolerance, digit). */
static int inside_all_faces(const brx_geometry* g, const double* x, tol_t t) {
  double vmin = 0.0;
  for (int f = 0; f < g->n_faces; ++f) {
    const double* abc = g->face_abc + 9 * f;
    double o = orient3d(abc, abc + 3, abc + 6, x);
    if (f == 0 || o < vmin) vmin = o;
  }
  return vmin > 0 || approx(vmin, 0.0, t);
}

/* ---------------------------------------------------------------------------
 * Stage 1a: first-zone move, BrillouinZone::moveinto (src/bz_move.cpp:103-163)
 * with part_moveinto_prim (:14-53).  Returns 0 or BRX_ERR_MOVE_FAILED.
 * ------------------------------------------------------------------------- */
static int moveinto_one(const brx_geometry* g, const double Q[3], double q_out[3], int32_t tau_out[3]) {
  tol_t t = tols(g->float_tolerance, g->digit);
  double Qp[3], q[3], x[3];
  int32_t tau[3], last[3];
  /* parallel_transform_to_primitive: (6Pᵗ · Q) / 6 (src/transform.hpp:168-191) */
  if (g->is_primitive) {
    for (int i = 0; i < 3; ++i) Qp[i] = Q[i];
  } else {
    matvec_i(Qp, g->to_prim_6Pt, Q);
    for (int i = 0; i < 3; ++i) Qp[i] = Qp[i] / 6.0;
  }
  for (int i = 0; i < 3; ++i) {
    tau[i] = (int32_t)round(Qp[i]);
    q[i] = Qp[i] - (double)tau[i];
    last[i] = tau[i];
  }
  int max_count = g->n_faces;
  int count = 0;
  for (;;) {
    if (!(count++ < max_count)) break;
    hkl_to_xyz(x, g->prim_B, q);
    if (inside_all_faces(g, x, t)) break;
    /* N_hkl = round(q·n̂ / |τ|) and the anti-oscillation choice (:29-47) */
    int max_nm = 0, max_at = 0, any_pos = 0;
    double dmax_at = 0.0;
    for (int j = 0; j < g->n_faces; ++j) {
      double dj = dot3(x, g->face_normal + 3 * j);
      int nj = (int)round(dj / g->face_tau_len[j]);
      if (nj > 0) any_pos = 1;
      const int32_t* tj = g->face_tau + 3 * j;
      int back = (tj[0] + last[0]) != 0 || (tj[1] + last[1]) != 0 || (tj[2] + last[2]) != 0;
      if (nj > 0 && nj >= max_nm && (0 == max_nm || (back && dj > dmax_at))) {
        max_at = j;
        max_nm = nj;
        dmax_at = dj;
      }
    }
    if (any_pos) {
      const int32_t* tj = g->face_tau + 3 * max_at;
      for (int i = 0; i < 3; ++i) {
        q[i] -= (double)tj[i] * (double)max_nm;
        tau[i] += tj[i] * max_nm;
        last[i] = tj[i] * max_nm;
      }
    }
  }
  /* parallel_transform_from_primitive: (P⁻¹)ᵀ · q (src/transform.hpp:204-230) */
  if (g->is_primitive) {
    for (int i = 0; i < 3; ++i) { q_out[i] = q[i]; tau_out[i] = tau[i]; }
  } else {
    matvec_i(q_out, g->from_prim_invPt, q);
    for (int i = 0; i < 3; ++i) {
      int64_t s = 0;
      for (int k = 0; k < 3; ++k) s += (int64_t)g->from_prim_invPt[3 * i + k] * tau[k];
      tau_out[i] = (int32_t)s;
    }
  }
  /* isinside re-check in the outer lattice (:149-159) */
  hkl_to_xyz(x, g->outer_B, q_out);
  return inside_all_faces(g, x, t) ? 0 : BRX_ERR_MOVE_FAILED;
}

/* _inside_wedge_outer (src/bz.hpp:757-763; src/array2.tpp:665-672) */
static int inside_wedge(const brx_geometry* g, const double x[3]) {
  if (g->n_wedge == 0) return 1;
  if (g->wedge_le_ge) {
    tol_t t0 = tols(0.0, 1);
    int all_le = 1, all_ge = 1;
    for (int i = 0; i < g->n_wedge; ++i) {
      double d = dot3(g->wedge_normal + 3 * i, x);
      if (!cmp_le(d, 0.0, t0)) all_le = 0;
      if (!cmp_ge(d, 0.0, t0)) all_ge = 0;
    }
    return all_le || all_ge;
  }
  tol_t t = tols(g->float_tolerance, g->digit);
  for (int i = 0; i < g->n_wedge; ++i)
    if (!cmp_ge(dot3(g->wedge_normal + 3 * i, x), 0.0, t)) return 0;
  return 1;
}

/* Stage 1b: BrillouinZone::ir_moveinto wedge search (src/bz_move.cpp:257-285):
 * the first j with Wⱼᵀ q inside the wedge; invR = j, R = inverse(j). */
static int wedge_one(const brx_geometry* g, double q[3], int32_t rot[2]) {
  double x[3], qj[3];
  hkl_to_xyz(x, g->outer_B, q);
  if (inside_wedge(g, x)) {
    rot[0] = rot[1] = g->identity;
    return 0;
  }
  for (int j = 0; j < g->n_ops; ++j) {
    const int32_t* W = g->ops + 9 * j;
    int32_t Wt[9] = {W[0], W[3], W[6], W[1], W[4], W[7], W[2], W[5], W[8]};
    matvec_i(qj, Wt, q);
    hkl_to_xyz(x, g->outer_B, qj);
    if (inside_wedge(g, x)) {
      for (int i = 0; i < 3; ++i) q[i] = qj[i];
      rot[1] = j;
      rot[0] = g->op_inverse[j];
      return 0;
    }
  }
  return BRX_ERR_OUTSIDE_IR;
}

/* ---------------------------------------------------------------------------
 * Stage 2: trellis locate
 * ------------------------------------------------------------------------- */
/* find_bin (src/trellis_poly.hpp:67-73) */
static int find_bin(const double* edges, int n, double x) {
  int d = n;
  for (int i = 0; i < n; ++i) if (edges[i] > x) { d = i; break; }
  if (d > n - 1 && x < edges[0]) d = 0;
  return d > 0 ? d - 1 : d;
}
/* on_boundary (src/trellis_poly.hpp:75-81) */
static int on_boundary(const double* edges, int n, double x, int i) {
  tol_t t = tols(0.0, 1);
  if (i + 2 < n && approx(edges[i + 1], x, t)) return 1;
  if (i > 0 && approx(edges[i], x, t)) return -1;
  return 0;
}

static int sub_ok_not_null(const brx_geometry* g, const int s[3]) {
  for (int d = 0; d < 3; ++d) if (s[d] < 0 || s[d] >= g->n_knots[d] - 1) return 0;
  int64_t idx = s[0] + (int64_t)(g->n_knots[0] - 1) * (s[1] + (int64_t)(g->n_knots[1] - 1) * s[2]);
  return g->node_type[idx] != BRX_NODE_NULL;
}

/* node_subscript (src/trellis_poly.hpp:382-434); returns the linear index or
 * -1 when the subscript falls outside the trellis */
static int64_t node_subscript(const brx_geometry* g, const double x[3]) {
  int sub[3], close[3], ns[3];
  for (int d = 0; d < 3; ++d) sub[d] = find_bin(g->knots[d], g->n_knots[d], x[d]);
  int bad = !sub_ok_not_null(g, sub);
  if (bad) {
    int num_close = 0;
    for (int i = 0; i < 3; ++i) {
      close[i] = on_boundary(g->knots[i], g->n_knots[i], x[i], sub[i]);
      if (close[i]) ++num_close;
    }
    memcpy(ns, sub, sizeof ns);
    if (num_close > 0)
      for (int i = 0; i < 3 && bad; ++i) if (close[i]) {
        memcpy(ns, sub, sizeof ns);
        ns[i] += close[i];
        bad = !sub_ok_not_null(g, ns);
      }
    if (bad && num_close > 1)
      for (int i = 0; i < 3 && bad; ++i) if (close[i])
        for (int j = 0; j < 3 && bad; ++j) if (close[j]) {
          memcpy(ns, sub, sizeof ns);
          ns[i] += close[i];
          ns[j] += close[j];
          bad = !sub_ok_not_null(g, ns);
        }
    if (bad && num_close > 2) {
      for (int i = 0; i < 3; ++i) ns[i] = sub[i] + close[i];
      bad = !sub_ok_not_null(g, ns);
    }
    if (!bad) memcpy(sub, ns, sizeof ns);
  }
  for (int d = 0; d < 3; ++d) if (sub[d] < 0 || sub[d] >= g->n_knots[d] - 1) return -1;
  return sub[0] + (int64_t)(g->n_knots[0] - 1) * (sub[1] + (int64_t)(g->n_knots[1] - 1) * sub[2]);
}

/* tetrahedra_might_contain (src/trellis_node.hpp:349-364) */
static double tet_might_contain(const brx_geometry* g, int64_t t, const double x[3]) {
  tol_t t0 = tols(0.0, 1);
  const double* s = g->tet_sphere + 4 * t;
  double v[3] = {s[0] - x[0], s[1] - x[1], s[2] - x[2]};
  double d2 = 0.0, r2 = s[3] * s[3];
  for (int i = 0; i < 3; ++i) d2 += v[i] * v[i];
  return (d2 < r2 || approx(d2, r2, t0)) ? 0.0 : -d2;
}

/* tetrahedra_contains (src/trellis_node.hpp:319-339) */
static double tet_contains(const brx_geometry* g, int64_t t, const double x[3], double w[4], int shortcut) {
  tol_t t0 = tols(0.0, 1);
  if (shortcut) {
    double away = tet_might_contain(g, t, x);
    if (away < 0.0) return away;
  }
  const int32_t* vi = g->tet_vertices + 4 * t;
  const double* v0 = g->vertex_xyz + 3 * (int64_t)vi[0];
  const double* v1 = g->vertex_xyz + 3 * (int64_t)vi[1];
  const double* v2 = g->vertex_xyz + 3 * (int64_t)vi[2];
  const double* v3 = g->vertex_xyz + 3 * (int64_t)vi[3];
  double vol6 = g->tet_volume[t] * 6.0;
  w[0] = orient3d(x, v1, v2, v3) / vol6;
  w[1] = orient3d(v0, x, v2, v3) / vol6;
  w[2] = orient3d(v0, v1, x, v3) / vol6;
  w[3] = orient3d(v0, v1, v2, x) / vol6;
  int any_neg = 0;
  double mn = w[0];
  for (int j = 0; j < 4; ++j) {
    if (w[j] < 0.0 && !approx(w[j], 0.0, t0)) any_neg = 1;
    if (w[j] < mn) mn = w[j];
  }
  return any_neg ? mn : 0.0;
}

/* NodeContainer::indices_weights (src/trellis_node.hpp:586-614) with
 * CubeNode (:132-149) and PolyNode (:275-308), should_contain = true.
 * Returns the number of (vertex, weight) pairs or a negative brx_status. */
static int node_weights(const brx_geometry* g, int64_t node, const double x[3],
                        int32_t* tet_out, int32_t vidx[8], double w8[8]) {
  tol_t t0 = tols(0.0, 1);
  *tet_out = -1;
  int type = g->node_type[node];
  int32_t ni = g->node_index[node];
  if (type == BRX_NODE_CUBE) {
    const int32_t* cv = g->cube_vertices + 8 * (int64_t)ni;
    const double* a = g->vertex_xyz + 3 * (int64_t)cv[0];
    const double* b = g->vertex_xyz + 3 * (int64_t)cv[7];
    double vol = 1.0;
    for (int d = 0; d < 3; ++d) vol *= fabs(a[d] - b[d]);
    int n = 0;
    for (int i = 0; i < 8; ++i) {
      const double* v = g->vertex_xyz + 3 * (int64_t)cv[i];
      double p = 1.0;
      for (int d = 0; d < 3; ++d) p *= fabs(x[d] - v[d]);
      double wi = p / vol;
      if (cmp_gt(wi, 0.0, t0)) { vidx[n] = cv[7 - i]; w8[n] = wi; ++n; }
    }
    return n;
  }
  if (type == BRX_NODE_POLY) {
    int32_t t_begin = g->poly_tet_offset[ni], t_end = g->poly_tet_offset[ni + 1];
    double w[4] = {0, 0, 0, 0};
    double best = 0.0;
    int32_t best_i = -1;
    for (int32_t t = t_begin; t < t_end; ++t) {
      double mn = tet_contains(g, t, x, w, 1);
      if (mn >= 0.0) {
        int n = 0;
        const int32_t* vi = g->tet_vertices + 4 * (int64_t)t;
        for (int j = 0; j < 4; ++j) if (!approx(w[j], 0.0, t0)) { vidx[n] = vi[j]; w8[n] = w[j]; ++n; }
        *tet_out = t;
        return n;
      }
      if (best_i < 0 || mn > best) { best = mn; best_i = t; }
    }
    if (best_i < 0) return 0;
    /* escape hatch: the tetrahedron with the largest most-negative weight */
    double val = tet_contains(g, best_i, x, w, 0);
    if (val > 0.0) return -BRX_ERR_IMPOSSIBLE;
    int n = 0;
    const int32_t* vi = g->tet_vertices + 4 * (int64_t)best_i;
    for (int j = 0; j < 4; ++j) if (!approx(w[j], 0.0, t0)) { vidx[n] = vi[j]; w8[n] = w[j]; ++n; }
    *tet_out = best_i;
    return n;
  }
  return -BRX_ERR_NULL_NODE;
}

/* PolyTrellis::indices_weights (src/trellis_poly.hpp:246-255) */
static int locate_one(const brx_geometry* g, const double x[3], int32_t node_tet[2],
                      int32_t vidx[8], double w8[8]) {
  int64_t node = node_subscript(g, x);
  node_tet[0] = (int32_t)node;
  node_tet[1] = -1;
  if (node < 0) return -BRX_ERR_NOT_FOUND;
  int n = node_weights(g, node, x, &node_tet[1], vidx, w8);
  if (n == 0) return -BRX_ERR_NOT_FOUND;
  return n;
}

/* ---------------------------------------------------------------------------
 * Stage 3: gather and weighted sum (src/interpolator_at.tpp:92-127) with the
 * permutation lookup (src/interpolatordual.hpp:376-382,
 * src/permutation_table.hpp:193-198) and antiphase (src/utilities.tpp:567-578)
 * ------------------------------------------------------------------------- */
typedef struct orc_perm {
  int64_t n_keys;
  const int64_t* keys;
  const int32_t* ids;
  int32_t n_perms;
  int32_t n_branches;
  const int32_t* perms; /* n_perms × n_branches */
} orc_perm;

static const int32_t* perm_get(const orc_perm* p, int64_t nv, int64_t i, int64_t j) {
  if (!p || !p->n_keys || i == j) return NULL;
  int64_t key = i * nv + j, lo = 0, hi = p->n_keys;
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    if (p->keys[mid] < key) lo = mid + 1; else hi = mid;
  }
  if (lo < p->n_keys && p->keys[lo] == key) {
    int32_t id = p->ids[lo];
    if (id >= 0 && id < p->n_perms) return p->perms + (int64_t)id * p->n_branches;
  }
  return NULL;
}

static void gather_one(const brx_data* d, const orc_perm* perm, int64_t nv, int n,
                       const int32_t* vidx, const double* w, double* out, int phase_allowed) {
  int B = d->n_branches;
  int s = d->elements[0] + d->elements[1] + d->elements[2];
  int cplx = d->dtype == BRX_C128;
  int es = cplx ? 2 : 1;
  const double* data = (const double*)d->data;
  int64_t row = (int64_t)B * s * es;
  memset(out, 0, sizeof(double) * (size_t)row);
  const double* d0 = data + row * vidx[0];
  for (int x = 0; x < n; ++x) {
    const double* dx = data + row * vidx[x];
    const int32_t* pm = perm_get(perm, nv, vidx[0], vidx[x]);
    for (int b = 0; b < B; ++b) {
      int p = pm ? pm[b] : b;
      if (cplx) {
        double er = 1.0, ei = 0.0;
        if (phase_allowed) {
          const double* a = d0 + (int64_t)b * s * 2;
          const double* c = dx + (int64_t)p * s * 2;
          double real_dot = 0.0, imag_dot = 0.0;
          for (int i = 0; i < s; ++i) {
            double ar = a[2 * i], ai = a[2 * i + 1], br = c[2 * i], bi = c[2 * i + 1];
            real_dot += ar * br + ai * bi;
            imag_dot += ar * bi - ai * br;
          }
          double th = -1.0 * atan2(imag_dot, real_dot);
          er = cos(th);
          ei = sin(th);
        }
        /* (w · e^{-iθ}) · d */
        double wr = w[x] * er, wi = w[x] * ei;
        for (int i = 0; i < s; ++i) {
          double dr = dx[((int64_t)p * s + i) * 2], di = dx[((int64_t)p * s + i) * 2 + 1];
          out[((int64_t)b * s + i) * 2] += wr * dr - wi * di;
          out[((int64_t)b * s + i) * 2 + 1] += wr * di + wi * dr;
        }
      } else {
        for (int i = 0; i < s; ++i) out[(int64_t)b * s + i] += w[x] * dx[(int64_t)p * s + i];
      }
    }
  }
}

/* ---------------------------------------------------------------------------
 * Stage 4: rotate back by R (src/interpolator.hpp:387-428;
 * interpolator_real.tpp:19-64, interpolator_recip.tpp:19-64,
 * interpolator_axial.tpp:19-68, interpolator_gamma.tpp:49-139)
 * ------------------------------------------------------------------------- */
/* Γ-rotated 3×3 tensors: the reference takes Nmat = ⌊√n⌋/3 for n matrices
 * and rotates nothing at all unless n == 9·Nmat² (interpolator_gamma.tpp:
 * 62-68); when n == 9·Nmat² it rotates only Nmat² of the n blocks and copies
 * the rest from an uninitialised buffer.  That case is rejected here. */
static int gamma_matrices_ill_defined(const brx_data* d) {
  int nmat = d->elements[2] / 9;
  int Nmat = (int)sqrt((double)nmat) / 3;
  return nmat > 0 && nmat == 9 * Nmat * Nmat;
}

/* status of a (RotatesLike, LengthUnit, complex) combination */
int orc_rotation_supported(const brx_data* d) {
  int cplx = d->dtype == BRX_C128;
  switch (d->length_unit) {
    case BRX_LU_REAL_LATTICE:
      if (d->rotates_like == BRX_ROT_GAMMA && !cplx) return BRX_ERR_UNSUPPORTED;
      if (d->rotates_like == BRX_ROT_GAMMA && gamma_matrices_ill_defined(d)) return BRX_ERR_UNSUPPORTED;
      return (d->rotates_like >= 0 && d->rotates_like <= 2) ? BRX_OK : BRX_ERR_UNSUPPORTED;
    case BRX_LU_RECIPROCAL_LATTICE:
      return d->rotates_like == BRX_ROT_VECTOR ? BRX_OK : BRX_ERR_UNSUPPORTED;
    case BRX_LU_ANGSTROM:
      if (d->rotates_like != BRX_ROT_GAMMA) return BRX_ERR_UNSUPPORTED;
      if (gamma_matrices_ill_defined(d)) return BRX_ERR_UNSUPPORTED;
      return cplx ? BRX_OK : BRX_ERR_UNSUPPORTED;
    default:
      return BRX_ERR_UNSUPPORTED;
  }
}

/* out = M · v for a real 3×3 M applied to an element vector of stride es */
static void mv_real(double* out, const double* M, const double* v, int es) {
  for (int i = 0; i < 3; ++i)
    for (int c = 0; c < es; ++c) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += M[3 * i + k] * v[k * es + c];
      out[i * es + c] = s;
    }
}
/* C = A · B, 3×3, element stride es for the side that may be complex */
static void mm(double* C, const double* A, int ea, const double* B, int eb) {
  int ec = (ea > eb) ? ea : eb;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double sr = 0.0, si = 0.0;
      for (int k = 0; k < 3; ++k) {
        const double* a = A + (3 * i + k) * ea;
        const double* b = B + (3 * k + j) * eb;
        if (ea == 2 && eb == 2) { sr += a[0] * b[0] - a[1] * b[1]; si += a[0] * b[1] + a[1] * b[0]; }
        else if (ea == 2) { sr += a[0] * b[0]; si += a[1] * b[0]; }
        else if (eb == 2) { sr += a[0] * b[0]; si += a[0] * b[1]; }
        else { sr += a[0] * b[0]; }
      }
      C[(3 * i + j) * ec] = sr;
      if (ec == 2) C[(3 * i + j) * ec + 1] = si;
    }
}
static void op_real(const brx_geometry* g, int r, double M[9]) {
  for (int i = 0; i < 9; ++i) M[i] = (double)g->ops[9 * r + i];
}
static void op_cart(const brx_geometry* g, int r, double M[9]) {
  /* L · W · L⁻¹ (src/interpolator.hpp:413-419) */
  double W[9], t[9];
  op_real(g, r, W);
  mm(t, g->lattice_to_xyz, 1, W, 1);
  mm(M, t, 1, g->lattice_from_xyz, 1);
}
static int is_identity(const brx_geometry* g, int r) {
  static const int32_t I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int i = 0; i < 9; ++i) if (g->ops[9 * r + i] != I[i]) return 0;
  return 1;
}

static void rotate_one(const brx_geometry* g, const brx_data* d, const double q_ir[3],
                       int Rii, int iRii, double* x, double* tmp) {
  int B = d->n_branches;
  int s = d->elements[0] + d->elements[1] + d->elements[2];
  int es = d->dtype == BRX_C128 ? 2 : 1;
  int nsc = d->elements[0], nvec = d->elements[1] / 3, nmat = d->elements[2] / 9;
  if (nvec == 0 && nmat == 0) return;
  double R[9], Ri[9], RT[9], RiT[9], t0[18], t1[18];
  if (d->rotates_like == BRX_ROT_GAMMA) {
    int Nmat = (int)sqrt((double)nmat) / 3;
    if (nmat != 9 * Nmat * Nmat) return; /* interpolator_gamma.tpp:64-68 */
    if (d->length_unit == BRX_LU_ANGSTROM) { op_cart(g, Rii, R); op_cart(g, iRii, Ri); }
    else { op_real(g, Rii, R); op_real(g, iRii, Ri); }
    for (int b = 0; b < B; ++b) {
      double* xb = x + (int64_t)b * s * 2;
      int o = nsc;
      if (nvec > 0) {
        int o0 = o;
        for (int k = 0; k < nvec; ++k) {
          mv_real(t0, Ri, xb + o * 2, 2);
          int v0 = 3 * g->gamma_F0[k * g->n_ops + iRii];
          const double* dv = g->gamma_vectors + 3 * g->gamma_vidx[k * g->n_ops + iRii];
          double dq = 0.0;
          for (int c = 0; c < 3; ++c) dq += q_ir[c] * dv[c];
          double ph = TWO_PI * dq, pr = cos(ph), pi = sin(ph);
          for (int j = 0; j < 3; ++j) {
            tmp[(v0 + j) * 2] = pr * t0[2 * j] - pi * t0[2 * j + 1];
            tmp[(v0 + j) * 2 + 1] = pr * t0[2 * j + 1] + pi * t0[2 * j];
          }
          o += 3;
        }
        memcpy(xb + o0 * 2, tmp, sizeof(double) * 2 * 3 * nvec);
      }
    }
    return;
  }
  if (is_identity(g, Rii)) return;
  op_real(g, Rii, R);
  op_real(g, iRii, Ri);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) { RT[3 * i + j] = R[3 * j + i]; RiT[3 * i + j] = Ri[3 * j + i]; }
  double det = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) + R[2] * (R[3] * R[7] - R[4] * R[6]);
  for (int b = 0; b < B; ++b) {
    double* xb = x + (int64_t)b * s * es;
    int o = nsc;
    for (int v = 0; v < nvec; ++v) {
      double* p = xb + o * es;
      if (d->length_unit == BRX_LU_RECIPROCAL_LATTICE) mv_real(t0, RT, p, es);
      else if (d->rotates_like == BRX_ROT_PSEUDOVECTOR) {
        mv_real(t0, Ri, p, es);
        for (int j = 0; j < 3 * es; ++j) t0[j] = det * t0[j];
      } else mv_real(t0, R, p, es);
      memcpy(p, t0, sizeof(double) * 3 * es);
      o += 3;
    }
    for (int m = 0; m < nmat; ++m) {
      double* p = xb + o * es;
      if (d->length_unit == BRX_LU_RECIPROCAL_LATTICE) { mm(t0, p, es, RiT, 1); mm(t1, RT, 1, t0, es); }
      else if (d->rotates_like == BRX_ROT_PSEUDOVECTOR) { mm(t0, p, es, R, 1); mm(t1, Ri, 1, t0, es); }
      else { mm(t0, p, es, Ri, 1); mm(t1, R, 1, t0, es); }
      memcpy(p, t1, sizeof(double) * 9 * es);
      o += 9;
    }
  }
}

/* ---------------------------------------------------------------------------
 * exported entry points
 * ------------------------------------------------------------------------- */
static int set_threads(int threads) {
#ifdef _OPENMP
  int n = threads > 0 ? threads : omp_get_max_threads();
  omp_set_num_threads(n);
  return n;
#else
  (void)threads;
  return 1;
#endif
}

/* moveinto / ir_moveinto for every Q (serially, as the reference does) */
int orc_move(const brx_geometry* g, const double* Q, int64_t n, int ir, double* q, int32_t* tau,
             int32_t* rot, int32_t* status) {
  int worst = 0;
  for (int64_t i = 0; i < n; ++i) {
    int32_t r2[2] = {g->identity, g->identity};
    int st = moveinto_one(g, Q + 3 * i, q + 3 * i, tau + 3 * i);
    if (!st && ir) st = wedge_one(g, q + 3 * i, r2);
    if (rot) { rot[2 * i] = r2[0]; rot[2 * i + 1] = r2[1]; }
    status[i] = st;
    if (st && !worst) worst = st;
  }
  return worst;
}

/* move (ir or first zone, or none) then locate, per q, as the GPU's
 * locate stage does; writes every intermediate index */
int orc_move_locate(const brx_geometry* g, const double* Q, int64_t n, int ir, int no_move, double* q, int32_t* tau,
                    int32_t* rot, int32_t* node_tet, int32_t* nw, int32_t* vidx, double* w, int32_t* status) {
  int worst = 0;
  for (int64_t i = 0; i < n; ++i) {
    int32_t r2[2] = {g->identity, g->identity};
    int st = 0;
    tau[3 * i] = tau[3 * i + 1] = tau[3 * i + 2] = 0;
    if (no_move) {
      for (int k = 0; k < 3; ++k) q[3 * i + k] = Q[3 * i + k];
    } else {
      st = moveinto_one(g, Q + 3 * i, q + 3 * i, tau + 3 * i);
      if (!st && ir) st = wedge_one(g, q + 3 * i, r2);
    }
    rot[2 * i] = r2[0];
    rot[2 * i + 1] = r2[1];
    node_tet[2 * i] = node_tet[2 * i + 1] = -1;
    nw[i] = 0;
    for (int k = 0; k < 8; ++k) { vidx[8 * i + k] = 0; w[8 * i + k] = 0.0; }
    if (!st) {
      double x[3];
      hkl_to_xyz(x, g->outer_B, q + 3 * i);
      int k = locate_one(g, x, node_tet + 2 * i, vidx + 8 * i, w + 8 * i);
      if (k > 0) nw[i] = k; else st = -k;
    }
    status[i] = st;
    if (st && !worst) worst = st;
  }
  return worst;
}

/* locate at Cartesian points (parallel over q) */
int orc_locate(const brx_geometry* g, const double* xyz, int64_t n, int32_t* node_tet,
               int32_t* nw, int32_t* vidx, double* w, int32_t* status, int threads) {
  set_threads(threads);
  int worst = 0;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i) {
    int k = locate_one(g, xyz + 3 * i, node_tet + 2 * i, vidx + 8 * i, w + 8 * i);
    nw[i] = k > 0 ? k : 0;
    status[i] = k > 0 ? 0 : -k;
    if (k <= 0) {
#pragma omp critical
      if (!worst) worst = -k;
    }
  }
  return worst;
}

/* The whole query path.  ir: ir_interpolate_at (1) or interpolate_at (0).
 * values/vectors: brx_data with host pointers; outputs in the input dtype.
 * Mirrors the reference's threading: the move stage runs serially
 * (src/bz_move.cpp:135-141, 257-285), locate+gather and the rotation in
 * parallel over q (src/trellis_poly.hpp:330, interpolator_gamma.tpp:81). */
int orc_interpolate_at(const brx_geometry* g, const brx_data* vals, const brx_data* vecs,
                       const orc_perm* perm, const double* Q, int64_t n, int ir, int no_move,
                       double* vals_out, double* vecs_out, int32_t* status_out, int threads) {
  int64_t nv = g->n_vertices;
  double* q = (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
  int32_t* tau = (int32_t*)malloc(sizeof(int32_t) * 3 * (size_t)(n > 0 ? n : 1));
  int32_t* rot = (int32_t*)malloc(sizeof(int32_t) * 2 * (size_t)(n > 0 ? n : 1));
  int32_t* st = status_out;
  int worst = 0;
  if (no_move) {
    memcpy(q, Q, sizeof(double) * 3 * (size_t)n);
    for (int64_t i = 0; i < n; ++i) { rot[2 * i] = rot[2 * i + 1] = g->identity; st[i] = 0; }
  } else {
    worst = orc_move(g, Q, n, ir, q, tau, rot, st);
  }
  if (worst) goto done;
  if (ir) {
    int sv = orc_rotation_supported(vals);
    if (sv) { worst = sv; goto done; }
    if (vecs) { sv = orc_rotation_supported(vecs); if (sv) { worst = sv; goto done; } }
  }
  set_threads(threads);
  {
    int Bv = vals->n_branches, sv = vals->elements[0] + vals->elements[1] + vals->elements[2];
    int ev = vals->dtype == BRX_C128 ? 2 : 1;
    int64_t rv = (int64_t)Bv * sv * ev;
    int64_t rc = 0;
    int sc = 0, ec = 1;
    if (vecs) {
      sc = vecs->elements[0] + vecs->elements[1] + vecs->elements[2];
      ec = vecs->dtype == BRX_C128 ? 2 : 1;
      rc = (int64_t)vecs->n_branches * sc * ec;
    }
    int missing = 0;
#pragma omp parallel
    {
      double* tmp = (double*)malloc(sizeof(double) * (size_t)((rv > rc ? rv : rc) + 64));
#pragma omp for schedule(dynamic, 64) reduction(+ : missing)
      for (int64_t i = 0; i < n; ++i) {
        double x[3];
        int32_t nt[2], vi[8];
        double w[8];
        hkl_to_xyz(x, g->outer_B, q + 3 * i);
        int k = locate_one(g, x, nt, vi, w);
        if (k <= 0) {
          st[i] = -k;
          ++missing;
          continue;
        }
        gather_one(vals, perm, nv, k, vi, w, vals_out + rv * i, 0);
        if (vecs) gather_one(vecs, perm, nv, k, vi, w, vecs_out + rc * i, 1);
        if (ir) {
          rotate_one(g, vals, q + 3 * i, rot[2 * i], rot[2 * i + 1], vals_out + rv * i, tmp);
          if (vecs) rotate_one(g, vecs, q + 3 * i, rot[2 * i], rot[2 * i + 1], vecs_out + rc * i, tmp);
        }
      }
      free(tmp);
    }
    if (missing) {
      for (int64_t i = 0; i < n; ++i) if (st[i]) { worst = st[i]; break; }
    }
  }
done:
  free(q);
  free(tau);
  free(rot);
  return worst;
}

/* One rotation applied to already-gathered data (for stage-level tests). */
int orc_rotate(const brx_geometry* g, const brx_data* d, const double* q_ir, const int32_t* rot,
               int64_t n, double* x) {
  int s = d->elements[0] + d->elements[1] + d->elements[2];
  int es = d->dtype == BRX_C128 ? 2 : 1;
  int64_t row = (int64_t)d->n_branches * s * es;
  int sv = orc_rotation_supported(d);
  if (sv) return sv;
  double* tmp = (double*)malloc(sizeof(double) * (size_t)(row + 64));
  for (int64_t i = 0; i < n; ++i) rotate_one(g, d, q_ir + 3 * i, rot[2 * i], rot[2 * i + 1], x + row * i, tmp);
  free(tmp);
  return 0;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---------------------------------------------------------------------------
 * sort(): mode permutations of connected vertex pairs
 * (DualInterpolator::sort / determine_permutation_ij / cost_matrix,
 * src/interpolatordual.hpp:385-434; Interpolator::add_cost,
 * src/interpolator_cost.tpp:19-61; set_cost_info, src/interpolator.hpp:246-300;
 * utilities.tpp:249-431 for the cost functions, :567-598 for the antiphase).
 *
 * The cost arithmetic is the reference's, operation by operation: the phase
 * of y is aligned to x with polar(1, −atan2(Im, Re)) of the Hermitian
 * product over the whole branch, and every cost function runs on the phased
 * copy.  One departure: for REAL vectors the reference leaves the phased
 * copy uninitialised (inplace_antiphase is a no-op for real types,
 * utilities.tpp:530), so its costs read garbage; here y is used unchanged.
 *
 * The assignment is solved exactly by shortest augmenting paths with row and
 * column potentials (the Hungarian method in the form of Jonker and
 * Volgenant's augmentation step), where the reference runs LAPJV
 * (src/lapjv.hpp).  Both return an optimal assignment; they agree wherever
 * the optimum is unique.  The scan order and the tie rule (the lowest column
 * among equal reduced costs) are the ones the GPU kernel uses, so for equal
 * cost matrices the two give the same assignment.
 * ------------------------------------------------------------------------- */
typedef struct orc_sort_side {
  const void* data;   /* n_vertices × B × s doubles (complex: pairs) */
  int32_t cplx;
  int32_t s, e0, e1, e2;
  int32_t vf;         /* vector cost function (reference numbering) */
  int32_t phase;      /* align phases first (vectors of a DualInterpolator) */
  double w[3];
} orc_sort_side;

static double clamp_cos(double c, int* bad) {
  tol_t one = tols(0.0, 1);
  double act = fabs(c);
  if (approx(act, 1.0, one) && act > 1.0) {
    c /= act;
    act = fabs(c);
  }
  if (act > 1.0) *bad = 1;
  return c;
}

static double cos_ratio(double num, double nA, double nB, int* bad) {
  double c;
  if (nA != 0.0 && nB != 0.0) c = num / (nA * nB);
  else c = (nA != 0.0 || nB != 0.0) ? 0.0 : 1.0;
  return clamp_cos(c, bad);
}

/* vector cost of n complex elements (utilities.tpp:280-431) */
static double vec_cost_c(int vf, int n, const double* a, const double* b, int* bad) {
  if (vf == 1) { /* vector_distance */
    double s = 0.0;
    for (int i = 0; i < n; ++i) {
      double dr = a[2 * i] - b[2 * i], di = a[2 * i + 1] - b[2 * i + 1];
      s += dr * dr + di * di;
    }
    return sqrt(s);
  }
  if (vf == 3) { /* euclidean_angle */
    double AB = 0.0, nA = 0.0, nB = 0.0;
    for (int i = 0; i < n; ++i) {
      AB += a[2 * i] * b[2 * i] + a[2 * i + 1] * b[2 * i + 1];
      nA += a[2 * i] * a[2 * i] + a[2 * i + 1] * a[2 * i + 1];
      nB += b[2 * i] * b[2 * i] + b[2 * i + 1] * b[2 * i + 1];
    }
    return acos(cos_ratio(AB, sqrt(nA), sqrt(nB), bad));
  }
  /* hermitian_product(a, b), (a, a), (b, b) */
  double hr = 0.0, hi = 0.0, aa = 0.0, bb = 0.0;
  for (int i = 0; i < n; ++i) {
    hr += a[2 * i] * b[2 * i] + a[2 * i + 1] * b[2 * i + 1];
    hi += a[2 * i] * b[2 * i + 1] - a[2 * i + 1] * b[2 * i];
    aa += a[2 * i] * a[2 * i] + a[2 * i + 1] * a[2 * i + 1];
    bb += b[2 * i] * b[2 * i] + b[2 * i + 1] * b[2 * i + 1];
  }
  double vp = hr * hr + hi * hi; /* vector_product */
  if (vf == 2) return 1.0 - vp;
  double th = acos(cos_ratio(sqrt(vp), sqrt(aa), sqrt(bb), bad)); /* hermitian_angle */
  if (vf == 4) return th;
  double s = sin(th);
  return s * s;
}

/* vector cost of n real elements (utilities.tpp:249-278, 383-405) */
static double vec_cost_r(int vf, int n, const double* a, const double* b, int* bad) {
  if (vf == 1) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) {
      double d = a[i] - b[i];
      s += d * d;
    }
    return sqrt(s);
  }
  if (vf == 2) {
    double h = 0.0;
    for (int i = 0; i < n; ++i) h += a[i] * b[i];
    return 1.0 - h;
  }
  double AA = 0.0, BB = 0.0, AB = 0.0;
  for (int i = 0; i < n; ++i) {
    AA += a[i] * a[i];
    BB += b[i] * b[i];
    AB += a[i] * b[i];
  }
  double th = acos(cos_ratio(AB, sqrt(AA), sqrt(BB), bad)); /* vector_angle */
  if (vf == 3 || vf == 4) return th;
  double s = sin(th);
  return s * s;
}

/* add_cost for one (row x of vertex i, row y of vertex j); ph: scratch of s complex */
static double side_cost(const orc_sort_side* S, const double* x, const double* y, double* ph, int* bad) {
  const int e0 = S->e0, e1 = S->e1, e2 = S->e2, s = S->s;
  double sc = 0.0, vc = 0.0, mc = 0.0;
  if (S->cplx) {
    const double* yy = y;
    if (S->phase) { /* inplace_antiphase */
      double rd = 0.0, id = 0.0;
      for (int k = 0; k < s; ++k) {
        rd += x[2 * k] * y[2 * k] + x[2 * k + 1] * y[2 * k + 1];
        id += x[2 * k] * y[2 * k + 1] - x[2 * k + 1] * y[2 * k];
      }
      double t = -1.0 * atan2(id, rd);
      double er = cos(t), ei = sin(t);
      for (int k = 0; k < s; ++k) {
        ph[2 * k] = er * y[2 * k] - ei * y[2 * k + 1];
        ph[2 * k + 1] = er * y[2 * k + 1] + ei * y[2 * k];
      }
      yy = ph;
    }
    for (int k = 0; k < e0; ++k) {
      double dr = x[2 * k] - yy[2 * k], di = x[2 * k + 1] - yy[2 * k + 1];
      sc += sqrt(dr * dr + di * di);
    }
    if (e1) vc = vec_cost_c(S->vf, e1, x + 2 * e0, yy + 2 * e0, bad);
    for (int m = 0; m < e2 / 9; ++m) mc += vec_cost_c(1, 9, x + 2 * (e0 + e1 + 9 * m), yy + 2 * (e0 + e1 + 9 * m), bad);
  } else {
    for (int k = 0; k < e0; ++k) sc += fabs(x[k] - y[k]);
    if (e1) vc = vec_cost_r(S->vf, e1, x + e0, y + e0, bad);
    for (int m = 0; m < e2 / 9; ++m) mc += vec_cost_r(1, 9, x + e0 + e1 + 9 * m, y + e0 + e1 + 9 * m, bad);
  }
  return S->w[0] * sc + S->w[1] * vc + S->w[2] * mc;
}

/* cost_matrix(i, j): rows the modes of i, columns the modes of j */
static int cost_matrix(const orc_sort_side* sides, int n_sides, int B, int64_t i, int64_t j, double* C, double* ph) {
  int bad = 0;
  for (int q = 0; q < B * B; ++q) C[q] = 0.0;
  for (int sd = 0; sd < n_sides; ++sd) {
    const orc_sort_side* S = sides + sd;
    const int row = S->s * (S->cplx ? 2 : 1);
    const double* d = (const double*)S->data;
    for (int a = 0; a < B; ++a)
      for (int b = 0; b < B; ++b)
        C[a * B + b] += side_cost(S, d + ((size_t)i * B + a) * row, d + ((size_t)j * B + b) * row, ph, &bad);
  }
  return bad;
}

/* Exact assignment of the n×n matrix C: p[j] (1-based, j = 1..n) is the row
 * matched to column j.  Returns 0, or 1 when no finite column is reachable. */
int orc_assign(const double* C, int n, int32_t* p_out) {
  double* u = (double*)calloc((size_t)n + 1, sizeof(double));
  double* v = (double*)calloc((size_t)n + 1, sizeof(double));
  double* minv = (double*)malloc(sizeof(double) * ((size_t)n + 1));
  int* p = (int*)calloc((size_t)n + 1, sizeof(int));
  int* way = (int*)calloc((size_t)n + 1, sizeof(int));
  char* used = (char*)malloc((size_t)n + 1);
  int rc = 0;
  for (int i = 1; i <= n && !rc; ++i) {
    for (int j = 0; j <= n; ++j) {
      minv[j] = DBL_MAX;
      used[j] = 0;
    }
    p[0] = i;
    int j0 = 0;
    for (int step = 0;; ++step) {
      used[j0] = 1;
      int i0 = p[j0], j1 = 0;
      double delta = DBL_MAX;
      for (int j = 1; j <= n; ++j) {
        if (used[j]) continue;
        double cur = (C[(size_t)(i0 - 1) * n + (j - 1)] - u[i0]) - v[j];
        if (cur < minv[j]) {
          minv[j] = cur;
          way[j] = j0;
        }
        if (minv[j] < delta) {
          delta = minv[j];
          j1 = j;
        }
      }
      if (j1 == 0 || step > n) {
        rc = 1;
        break;
      }
      for (int j = 0; j <= n; ++j) {
        if (used[j]) {
          u[p[j]] += delta;
          v[j] -= delta;
        } else {
          minv[j] -= delta;
        }
      }
      j0 = j1;
      if (p[j0] == 0) break;
    }
    if (rc) break;
    do {
      int j1 = way[j0];
      p[j0] = p[j1];
      j0 = j1;
    } while (j0);
  }
  for (int j = 1; j <= n; ++j) p_out[j - 1] = p[j];
  free(u);
  free(v);
  free(minv);
  free(p);
  free(way);
  free(used);
  return rc;
}

static int64_t key_index(const int64_t* keys, int64_t n, int64_t key) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (keys[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return (lo < n && keys[lo] == key) ? lo : -1;
}

/* sort() over sorted keys: perm_out (n_keys × B) row k is the permutation of
 * key k (row → column for i < j, column → row for the reverse key).
 * cost_out, when given, receives the cost matrix of every key with i < j.
 * Returns 0, BRX_ERR_INVALID_ARGUMENT for a missing reverse key, or
 * BRX_ERR_IMPOSSIBLE (a cosine above 1, no finite assignment). */
int orc_sort(const orc_sort_side* sides, int n_sides, int B, int64_t nv, int64_t n_keys, const int64_t* keys,
             int32_t* perm_out, double* cost_out, int threads) {
  int rc = 0;
  set_threads(threads);
#pragma omp parallel
  {
    double* C = (double*)malloc(sizeof(double) * (size_t)B * B);
    int smax = 1;
    for (int sd = 0; sd < n_sides; ++sd)
      if (sides[sd].s > smax) smax = sides[sd].s;
    double* ph = (double*)malloc(sizeof(double) * 2 * (size_t)smax);
    int32_t* p = (int32_t*)malloc(sizeof(int32_t) * (size_t)B);
#pragma omp for schedule(dynamic, 64)
    for (int64_t k = 0; k < n_keys; ++k) {
      int64_t i = keys[k] / nv, j = keys[k] % nv;
      if (i >= j) continue;
      int64_t kr = key_index(keys, n_keys, j * nv + i);
      int e = 0;
      if (kr < 0) e = BRX_ERR_INVALID_ARGUMENT;
      else if (cost_matrix(sides, n_sides, B, i, j, C, ph) || orc_assign(C, B, p)) e = BRX_ERR_IMPOSSIBLE;
      if (e) {
#pragma omp critical
        if (!rc) rc = e;
        continue;
      }
      if (cost_out) memcpy(cost_out + (size_t)k * B * B, C, sizeof(double) * (size_t)B * B);
      for (int c = 0; c < B; ++c) {
        perm_out[(size_t)k * B + (p[c] - 1)] = c;
        perm_out[(size_t)kr * B + c] = p[c] - 1;
      }
    }
    free(C);
    free(ph);
    free(p);
  }
  return rc;
}
