// K1+K2: first-zone move, irreducible-wedge search and trellis locate.
//
// One thread per q.  The small per-zone tables (faces, wedge normals, point
// operations) are staged in shared memory once per CTA; trellis tables are
// read through the read-only path.  All predicates are FP64 (brx_device.cuh).
//
// Reference: BrillouinZone::moveinto / part_moveinto_prim
// (src/bz_move.cpp:14-53, 103-163), ir_moveinto (:257-285),
// _inside_wedge_outer (src/bz.hpp:757-763), PolyTrellis::node_subscript
// (src/trellis_poly.hpp:382-434), CubeNode/PolyNode::indices_weights
// (src/trellis_node.hpp:132-149, 275-364).
#include <cstdint>

#include "brx_device.cuh"
#include "brx_kernels.h"
#include "../../include/brx.h"

namespace brx {

// FP32 screens.  A face test or a wedge test evaluated in FP32 decides the
// exact FP64 predicate whenever the FP32 value lies outside an error margin
// around the predicate's tolerance band; only the undecided cases are
// evaluated exactly.  The decision is therefore the FP64 one in every case,
// and the first-match orders of the reference are kept.
//
// Margin: with unit normals and |x|₁ = Σ|x_i|, an FP32 dot product of
// rounded operands is within 8 ε₃₂ (|x|₁ + |h|) of the exact value; 3e-6
// covers that with a factor of over five.
__device__ __forceinline__ float screen_margin(float x1, float h) { return 3e-6f * (x1 + fabsf(h) + 1e-6f); }

struct SmemZone {
  float* plane;     // n_faces × 4
  float* band;      // n_faces
  float* wm;        // (n_ops + 1) × n_wedge × 3
  float* n32;       // n_faces × 3: face normals rounded to FP32
  float* tl32;      // n_faces: |τ| rounded to FP32
  double* abc;      // n_faces × 9
  double* normal;   // n_faces × 3
  double* tau_len;  // n_faces
  int32_t* tau;     // n_faces × 3
  double* wedge;    // n_wedge × 3
  int32_t* ops;     // n_ops × 9
  int32_t* opinv;   // n_ops
};

__device__ bool inside_all_faces_exact(const DevGeom& g, const SmemZone& z, const double x[3]) {
  double vmin = 0.0;
  for (int f = 0; f < g.n_faces; ++f) {
    const double* abc = z.abc + 9 * f;
    double o = orient3d(abc, abc + 3, abc + 6, x);
    if (f == 0 || o < vmin) vmin = o;
  }
  return vmin > 0 || approx(vmin, 0.0, g.t_main);
}

// point_inside_all_planes with the FP32 screen: −1 definitely outside,
// +1 definitely inside, 0 undecided
__device__ __forceinline__ int screen_faces(const DevGeom& g, const SmemZone& z, const double x[3]) {
  const float x0 = (float)x[0], x1 = (float)x[1], x2 = (float)x[2];
  const float xa = fabsf(x0) + fabsf(x1) + fabsf(x2);
  int all_in = 1;
  for (int f = 0; f < g.n_faces; ++f) {
    const float* P = z.plane + 4 * f;
    const float d = P[3] - (P[0] * x0 + P[1] * x1 + P[2] * x2);  // k_f·d = orient3d
    const float m = screen_margin(xa, P[3]);
    if (d < -(m + z.band[f])) return -1;
    if (!(d > m)) all_in = 0;
  }
  return all_in;
}

__device__ bool inside_all_faces(const DevGeom& g, const SmemZone& z, const double x[3]) {
  if (g.screen) {
    const int s = screen_faces(g, z, x);
    if (s) return s > 0;
  }
  return inside_all_faces_exact(g, z, x);
}

// One step of part_moveinto_prim's shift choice (src/bz_move.cpp:28-46) in
// FP32: n_j = round(n̂_j·x / |τ_j|) for every face, and the face of largest
// positive n_j, ties going to a later face only when it does not undo the
// last shift and lies further out.  Returns false, leaving the choice to the
// exact loop, whenever a quotient lies within its error bound of a rounding
// boundary or two candidate distances are too close to order; otherwise the
// choice is the FP64 one.  With unit normals |n̂·x|'s FP32 error is below
// 3e-7·|x|₁, so the 3e-6 margin of screen_margin covers it tenfold.
__device__ bool shift_screen(const DevGeom& g, const SmemZone& z, const double x[3], const int32_t last[3],
                             int* max_nm_out, int* max_at_out, int* any_pos_out) {
  const float x0 = (float)x[0], x1 = (float)x[1], x2 = (float)x[2];
  const float ed = screen_margin(fabsf(x0) + fabsf(x1) + fabsf(x2), 0.f);
  int max_nm = 0, max_at = 0, any_pos = 0;
  float dmax = 0.f;
  for (int j = 0; j < g.n_faces; ++j) {
    const float* n = z.n32 + 3 * j;
    const float d = n[0] * x0 + n[1] * x1 + n[2] * x2;
    const float tl = z.tl32[j];
    const float r = d / tl;
    const float mr = ed / tl + 1e-6f * fabsf(r) + 1e-30f;
    if (fabsf((r - floorf(r)) - 0.5f) <= mr) return false;
    const int nj = (int)roundf(r);
    if (nj > 0) any_pos = 1;
    const int32_t* tj = z.tau + 3 * j;
    const bool back = (tj[0] + last[0]) != 0 || (tj[1] + last[1]) != 0 || (tj[2] + last[2]) != 0;
    if (nj > 0 && nj >= max_nm) {
      bool take = max_nm == 0;
      if (!take && back) {
        if (fabsf(d - dmax) <= 2.f * ed) return false;
        take = d > dmax;
      }
      if (take) {
        max_at = j;
        max_nm = nj;
        dmax = d;
      }
    }
  }
  *max_nm_out = max_nm;
  *max_at_out = max_at;
  *any_pos_out = any_pos;
  return true;
}

// Returns 0 or BRX_ERR_MOVE_FAILED; q_out in conventional r.l.u.
__device__ int moveinto_one(const DevGeom& g, const SmemZone& z, const double Q[3], double q_out[3],
                            int32_t tau_out[3]) {
  double Qp[3], q[3], x[3];
  int32_t tau[3], last[3];
  if (g.is_primitive) {
    for (int i = 0; i < 3; ++i) Qp[i] = Q[i];
  } else {
    matvec_i(Qp, g.to_prim_6Pt, Q);
    for (int i = 0; i < 3; ++i) Qp[i] = __ddiv_rn(Qp[i], 6.0);
  }
  for (int i = 0; i < 3; ++i) {
    tau[i] = (int32_t)round(Qp[i]);
    q[i] = dsub(Qp[i], (double)tau[i]);
    last[i] = tau[i];
  }
  const int max_count = g.n_faces;
  int count = 0;
  for (;;) {
    if (!(count++ < max_count)) break;
    hkl_to_xyz(x, g.prim_B, q);
    if (inside_all_faces(g, z, x)) break;
    int max_nm = 0, max_at = 0, any_pos = 0;
    double dmax = 0.0;
    const bool screened = g.screen && shift_screen(g, z, x, last, &max_nm, &max_at, &any_pos);
    for (int j = 0; !screened && j < g.n_faces; ++j) {
      double dj = dot3(x, z.normal + 3 * j);
      int nj = (int)round(__ddiv_rn(dj, z.tau_len[j]));
      if (nj > 0) any_pos = 1;
      const int32_t* tj = z.tau + 3 * j;
      bool back = (tj[0] + last[0]) != 0 || (tj[1] + last[1]) != 0 || (tj[2] + last[2]) != 0;
      if (nj > 0 && nj >= max_nm && (0 == max_nm || (back && dj > dmax))) {
        max_at = j;
        max_nm = nj;
        dmax = dj;
      }
    }
    if (any_pos) {
      const int32_t* tj = z.tau + 3 * max_at;
      for (int i = 0; i < 3; ++i) {
        q[i] = dsub(q[i], dmul((double)tj[i], (double)max_nm));
        tau[i] += tj[i] * max_nm;
        last[i] = tj[i] * max_nm;
      }
    }
  }
  if (g.is_primitive) {
    for (int i = 0; i < 3; ++i) { q_out[i] = q[i]; tau_out[i] = tau[i]; }
  } else {
    matvec_i(q_out, g.from_prim_invPt, q);
    for (int i = 0; i < 3; ++i) {
      long long s = 0;
      for (int k = 0; k < 3; ++k) s += (long long)g.from_prim_invPt[3 * i + k] * tau[k];
      tau_out[i] = (int32_t)s;
    }
  }
  hkl_to_xyz(x, g.outer_B, q_out);
  return inside_all_faces(g, z, x) ? 0 : BRX_ERR_MOVE_FAILED;
}

__device__ bool inside_wedge(const DevGeom& g, const SmemZone& z, const double x[3]) {
  if (g.n_wedge == 0) return true;
  if (g.wedge_le_ge) {
    bool all_le = true, all_ge = true;
    for (int i = 0; i < g.n_wedge; ++i) {
      double d = dot3(z.wedge + 3 * i, x);
      if (!cmp_le(d, 0.0, g.t_def)) all_le = false;
      if (!cmp_ge(d, 0.0, g.t_def)) all_ge = false;
    }
    return all_le || all_ge;
  }
  for (int i = 0; i < g.n_wedge; ++i)
    if (!cmp_ge(dot3(z.wedge + 3 * i, x), 0.0, g.t_main)) return false;
  return true;
}

// Can W_jᵀ q (x its Cartesian form) be inside the wedge?  False only when
// some normal puts it outside by more than the margin and the tolerance band.
__device__ __forceinline__ bool wedge_candidate(const DevGeom& g, const float* m, float x0, float x1, float x2,
                                                float tol) {
  bool all_ge = true, all_le = true;
  for (int i = 0; i < g.n_wedge; ++i) {
    const float d = m[3 * i] * x0 + m[3 * i + 1] * x1 + m[3 * i + 2] * x2;
    if (d < -tol) all_ge = false;
    if (d > tol) all_le = false;
  }
  return all_ge || (g.wedge_le_ge && all_le);
}

// Is W_jᵀ q certainly inside the wedge?  True only when every normal puts
// it strictly on the inner side (or, for a mirrored wedge, every normal on
// the outer side) by more than the FP32 error margin: the exact dot products
// are then of that sign, and the exact test would accept.
__device__ __forceinline__ bool wedge_sure(const DevGeom& g, const float* m, float x0, float x1, float x2,
                                           float margin) {
  bool all_ge = true, all_le = true;
  for (int i = 0; i < g.n_wedge; ++i) {
    const float d = m[3 * i] * x0 + m[3 * i + 1] * x1 + m[3 * i + 2] * x2;
    if (!(d > margin)) all_ge = false;
    if (!(d < -margin)) all_le = false;
  }
  return all_ge || (g.wedge_le_ge && all_le);
}

__device__ int wedge_one(const DevGeom& g, const SmemZone& z, double q[3], int32_t rot[2]) {
  double x[3], qj[3];
  hkl_to_xyz(x, g.outer_B, q);
  if (g.screen && g.n_wedge > 0 && g.n_ops <= 64) {
    // FP32 screen of every operation first (the same work in every lane),
    // then exact tests of the survivors in the reference's order; each lane
    // walks its own candidate mask, so the exact tests run converged
    // an operation certainly inside needs no exact test either: the first
    // candidate in order that is certainly inside is the exact answer
    const float x0 = (float)x[0], x1 = (float)x[1], x2 = (float)x[2];
    const float margin = screen_margin(fabsf(x0) + fabsf(x1) + fabsf(x2), 0.f);
    const float tol = margin + g.wedge_band32;
    const float* wid = z.wm + 3 * g.n_wedge * g.n_ops;
    const bool id_cand = wedge_candidate(g, wid, x0, x1, x2, tol);
    unsigned long long mask = 0ull, sure = 0ull;
    for (int j = 0; j < g.n_ops; ++j)
      if (wedge_candidate(g, z.wm + 3 * g.n_wedge * j, x0, x1, x2, tol)) {
        mask |= 1ull << j;
        if (wedge_sure(g, z.wm + 3 * g.n_wedge * j, x0, x1, x2, margin)) sure |= 1ull << j;
      }
    if (id_cand && (wedge_sure(g, wid, x0, x1, x2, margin) || inside_wedge(g, z, x))) {
      rot[0] = rot[1] = g.identity;
      return 0;
    }
    while (mask) {
      const int j = __ffsll((long long)mask) - 1;
      mask &= mask - 1;
      const int32_t* W = z.ops + 9 * j;
      int32_t Wt[9] = {W[0], W[3], W[6], W[1], W[4], W[7], W[2], W[5], W[8]};
      matvec_i(qj, Wt, q);
      bool in = (sure >> j) & 1ull;
      if (!in) {
        double xj[3];
        hkl_to_xyz(xj, g.outer_B, qj);
        in = inside_wedge(g, z, xj);
      }
      if (in) {
        q[0] = qj[0]; q[1] = qj[1]; q[2] = qj[2];
        rot[1] = j;
        rot[0] = z.opinv[j];
        return 0;
      }
    }
    return BRX_ERR_OUTSIDE_IR;
  }
  if (inside_wedge(g, z, x)) {
    rot[0] = rot[1] = g.identity;
    return 0;
  }
  for (int j = 0; j < g.n_ops; ++j) {
    const int32_t* W = z.ops + 9 * j;
    int32_t Wt[9] = {W[0], W[3], W[6], W[1], W[4], W[7], W[2], W[5], W[8]};
    matvec_i(qj, Wt, q);
    hkl_to_xyz(x, g.outer_B, qj);
    if (inside_wedge(g, z, x)) {
      q[0] = qj[0]; q[1] = qj[1]; q[2] = qj[2];
      rot[1] = j;
      rot[0] = z.opinv[j];
      return 0;
    }
  }
  return BRX_ERR_OUTSIDE_IR;
}

// find_bin: the first knot greater than x (std::find_if in the reference)
// found by bisection, which gives the same index because knots increase
// strictly; a NaN compares false everywhere and lands past the end as there.
// The comparisons run on integer keys of the doubles (the bit pattern,
// negatives with their magnitude bits flipped), which order non-NaN values
// as IEEE does once x's −0 is taken as +0; a NaN x compares in FP64.
__device__ __forceinline__ long long order_key(long long b) { return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL); }

__device__ __forceinline__ int find_bin(const double* e, int n, double x, bool int_keys) {
  int lo = 0, hi = n;
  long long xb = __double_as_longlong(x);
  if (!int_keys || (xb & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL) {
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(e + mid) > x) hi = mid; else lo = mid + 1;
    }
  } else {
    if (xb == (long long)0x8000000000000000ULL) xb = 0;
    const long long xk = order_key(xb);
    const long long* eb = reinterpret_cast<const long long*>(e);
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (order_key(__ldg(eb + mid)) > xk) hi = mid; else lo = mid + 1;
    }
  }
  int d = lo;
  if (d > n - 1 && x < __ldg(e)) d = 0;
  return d > 0 ? d - 1 : d;
}

__device__ __forceinline__ int on_boundary(const DevGeom& g, const double* e, int n, double x, int i) {
  if (i + 2 < n && approx(__ldg(e + i + 1), x, g.t_def)) return 1;
  if (i > 0 && approx(__ldg(e + i), x, g.t_def)) return -1;
  return 0;
}

__device__ __forceinline__ bool sub_ok_not_null(const DevGeom& g, const int s[3]) {
  for (int d = 0; d < 3; ++d)
    if (s[d] < 0 || s[d] >= g.n_knots[d] - 1) return false;
  long long idx = s[0] + (long long)(g.n_knots[0] - 1) * (s[1] + (long long)(g.n_knots[1] - 1) * s[2]);
  return __ldg(g.node_type + idx) != BRX_NODE_NULL;
}

__device__ long long node_subscript(const DevGeom& g, const double x[3]) {
  int sub[3], close[3], ns[3];
  for (int d = 0; d < 3; ++d) sub[d] = find_bin(g.knots[d], g.n_knots[d], x[d], g.screen != 0);
  bool bad = !sub_ok_not_null(g, sub);
  if (bad) {
    int num_close = 0;
    for (int i = 0; i < 3; ++i) {
      close[i] = on_boundary(g, g.knots[i], g.n_knots[i], x[i], sub[i]);
      if (close[i]) ++num_close;
    }
    ns[0] = sub[0]; ns[1] = sub[1]; ns[2] = sub[2];
    if (num_close > 0)
      for (int i = 0; i < 3 && bad; ++i)
        if (close[i]) {
          ns[0] = sub[0]; ns[1] = sub[1]; ns[2] = sub[2];
          ns[i] += close[i];
          bad = !sub_ok_not_null(g, ns);
        }
    if (bad && num_close > 1)
      for (int i = 0; i < 3 && bad; ++i)
        if (close[i])
          for (int j = 0; j < 3 && bad; ++j)
            if (close[j]) {
              ns[0] = sub[0]; ns[1] = sub[1]; ns[2] = sub[2];
              ns[i] += close[i];
              ns[j] += close[j];
              bad = !sub_ok_not_null(g, ns);
            }
    if (bad && num_close > 2) {
      for (int i = 0; i < 3; ++i) ns[i] = sub[i] + close[i];
      bad = !sub_ok_not_null(g, ns);
    }
    if (!bad) { sub[0] = ns[0]; sub[1] = ns[1]; sub[2] = ns[2]; }
  }
  for (int d = 0; d < 3; ++d)
    if (sub[d] < 0 || sub[d] >= g.n_knots[d] - 1) return -1;
  return sub[0] + (long long)(g.n_knots[0] - 1) * (sub[1] + (long long)(g.n_knots[1] - 1) * sub[2]);
}

__device__ __forceinline__ void load3(double out[3], const double* p) {
  out[0] = __ldg(p); out[1] = __ldg(p + 1); out[2] = __ldg(p + 2);
}

// approx(w, 0, t_def) and cmp_gt(w, 0, t_def) from the bits of w where w is
// far from the tolerance band.  t_def has rel = 1e4·ε (2.2e-12) and abs =
// 5e-15, so approx(w, 0) — |w| ≤ 5e-15 + 2.2e-12·|w| in FP64 — holds for
// every |w| < 4e-15 and fails for every finite |w| > 1e-14; in between, and
// for infinities and NaN, the FP64 test runs.  Integer compares keep the
// FP64 pipe free.
__device__ __forceinline__ bool approx0_def(const DevGeom& g, double w) {
  if (g.screen) {
    const long long b = __double_as_longlong(w) & 0x7fffffffffffffffLL;
    if (b > __double_as_longlong(1e-14) && b < 0x7ff0000000000000LL) return false;
    if (b < __double_as_longlong(4e-15)) return true;
  }
  return approx(w, 0.0, g.t_def);
}
__device__ __forceinline__ bool gt0_def(const DevGeom& g, double w) {
  if (g.screen) {
    const long long b = __double_as_longlong(w);
    if (b < 0) return false;  // negative (or −NaN): w > 0 fails
    if (b > __double_as_longlong(1e-14) && b < 0x7ff0000000000000LL) return true;
    if (b < __double_as_longlong(4e-15)) return false;
  }
  return cmp_gt(w, 0.0, g.t_def);
}

__device__ double tet_contains(const DevGeom& g, long long t, const double x[3], double w[4], bool shortcut) {
  if (shortcut) {
    double s[4];
    const double* sp = g.tet_sphere + 4 * t;
    s[0] = __ldg(sp); s[1] = __ldg(sp + 1); s[2] = __ldg(sp + 2); s[3] = __ldg(sp + 3);
    double v0 = dsub(s[0], x[0]), v1 = dsub(s[1], x[1]), v2 = dsub(s[2], x[2]);
    double d2 = 0.0;
    d2 = dadd(d2, dmul(v0, v0));
    d2 = dadd(d2, dmul(v1, v1));
    d2 = dadd(d2, dmul(v2, v2));
    double r2 = dmul(s[3], s[3]);
    if (!(d2 < r2 || approx(d2, r2, g.t_def))) return -d2;
  }
  const int32_t* vi = g.tet_vertices + 4 * t;
  double a[3], b[3], c[3], d[3];
  load3(a, g.vertex_xyz + 3 * (long long)__ldg(vi));
  load3(b, g.vertex_xyz + 3 * (long long)__ldg(vi + 1));
  load3(c, g.vertex_xyz + 3 * (long long)__ldg(vi + 2));
  load3(d, g.vertex_xyz + 3 * (long long)__ldg(vi + 3));
  double vol6 = dmul(__ldg(g.tet_volume + t), 6.0);
  w[0] = __ddiv_rn(orient3d(x, b, c, d), vol6);
  w[1] = __ddiv_rn(orient3d(a, x, c, d), vol6);
  w[2] = __ddiv_rn(orient3d(a, b, x, d), vol6);
  w[3] = __ddiv_rn(orient3d(a, b, c, x), vol6);
  bool any_neg = false;
  double mn = w[0];
  for (int j = 0; j < 4; ++j) {
    if (w[j] < 0.0 && !approx0_def(g, w[j])) any_neg = true;
    if (w[j] < mn) mn = w[j];
  }
  return any_neg ? mn : 0.0;
}

// FP32 screen of one tetrahedron: true only when some barycentric weight is
// negative by more than a margin of 1e-5 of its magnitude scale (25× the FP32
// evaluation error), so that the exact test of tet_contains would find it
// negative beyond the default tolerance too.  NaN planes never screen out.
__device__ __forceinline__ bool tet_screened_out(const DevGeom& g, long long t, float x0, float x1, float x2,
                                                 float ax) {
  const float4* P = reinterpret_cast<const float4*>(g.tet_plane32) + 4 * t;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float4 p = __ldg(P + j);
    const float w = fmaf(p.x, x0, fmaf(p.y, x1, fmaf(p.z, x2, p.w)));
    const float m = 1e-5f * ((fabsf(p.x) + fabsf(p.y) + fabsf(p.z)) * ax + fabsf(p.w)) + 1e-12f;
    if (w < -m) return true;
  }
  return false;
}

// Returns the number of (vertex, weight) pairs, or −status.
__device__ int node_weights(const DevGeom& g, long long node, const double x[3], int32_t* tet_out,
                            int32_t vidx[8], double w8[8]) {
  *tet_out = -1;
  const int type = __ldg(g.node_type + node);
  const int32_t ni = __ldg(g.node_index + node);
  if (type == BRX_NODE_CUBE) {
    const int32_t* cv = g.cube_vertices + 8 * (long long)ni;
    int32_t ids[8];
    for (int i = 0; i < 8; ++i) ids[i] = __ldg(cv + i);
    double a[3], b[3];
    load3(a, g.vertex_xyz + 3 * (long long)ids[0]);
    load3(b, g.vertex_xyz + 3 * (long long)ids[7]);
    double vol = 1.0;
    for (int d = 0; d < 3; ++d) vol = dmul(vol, fabs(dsub(a[d], b[d])));
    int n = 0;
    if (g.cube_canon) {
      // corner i's factor on axis d is |x_d − a_d| or |x_d − b_d|, and
      // ((1·f0)·f1)·f2 = (f0·f1)·f2 exactly: the same products, formed once
      double da[3], db[3];
      for (int d = 0; d < 3; ++d) {
        da[d] = fabs(dsub(x[d], a[d]));
        db[d] = fabs(dsub(x[d], b[d]));
      }
      double p01[4];
      for (int k = 0; k < 4; ++k) p01[k] = dmul((k & 1) ? db[0] : da[0], (k & 2) ? db[1] : da[1]);
      for (int i = 0; i < 8; ++i) {
        const int bits = (g.cube_pattern >> (3 * i)) & 7;
        const double p = dmul(p01[bits & 3], (bits & 4) ? db[2] : da[2]);
        const double wi = __ddiv_rn(p, vol);
        if (gt0_def(g, wi)) { vidx[n] = ids[7 - i]; w8[n] = wi; ++n; }
      }
      return n;
    }
    for (int i = 0; i < 8; ++i) {
      double v[3];
      load3(v, g.vertex_xyz + 3 * (long long)ids[i]);
      double p = 1.0;
      for (int d = 0; d < 3; ++d) p = dmul(p, fabs(dsub(x[d], v[d])));
      double wi = __ddiv_rn(p, vol);
      if (gt0_def(g, wi)) { vidx[n] = ids[7 - i]; w8[n] = wi; ++n; }
    }
    return n;
  }
  if (type == BRX_NODE_POLY) {
    const int32_t tb = __ldg(g.poly_tet_offset + ni), te = __ldg(g.poly_tet_offset + ni + 1);
    double w[4] = {0, 0, 0, 0};
    if (g.screen) {
      // first containing tetrahedron in order, skipping those the FP32
      // screen rules out; none found: the exact loop below (with its
      // fallback) decides
      const float x0 = (float)x[0], x1 = (float)x[1], x2 = (float)x[2];
      const float ax = fabsf(x0) + fabsf(x1) + fabsf(x2);
      for (int32_t t = tb; t < te; ++t) {
        if (tet_screened_out(g, t, x0, x1, x2, ax)) continue;
        if (tet_contains(g, t, x, w, true) >= 0.0) {
          int n = 0;
          for (int j = 0; j < 4; ++j)
            if (!approx0_def(g, w[j])) { vidx[n] = __ldg(g.tet_vertices + 4 * (long long)t + j); w8[n] = w[j]; ++n; }
          *tet_out = t;
          return n;
        }
      }
    }
    double best = 0.0;
    int32_t best_i = -1;
    for (int32_t t = tb; t < te; ++t) {
      double mn = tet_contains(g, t, x, w, true);
      if (mn >= 0.0) {
        int n = 0;
        for (int j = 0; j < 4; ++j)
          if (!approx0_def(g, w[j])) { vidx[n] = __ldg(g.tet_vertices + 4 * (long long)t + j); w8[n] = w[j]; ++n; }
        *tet_out = t;
        return n;
      }
      if (best_i < 0 || mn > best) { best = mn; best_i = t; }
    }
    if (best_i < 0) return 0;
    double val = tet_contains(g, best_i, x, w, false);
    if (val > 0.0) return -BRX_ERR_IMPOSSIBLE;
    int n = 0;
    for (int j = 0; j < 4; ++j)
      if (!approx0_def(g, w[j])) { vidx[n] = __ldg(g.tet_vertices + 4 * (long long)best_i + j); w8[n] = w[j]; ++n; }
    *tet_out = best_i;
    return n;
  }
  return -BRX_ERR_NULL_NODE;
}

__device__ __forceinline__ void report(ErrorWord* err, long long i, int st) {
  atomicOr(&err->flags, 1 << st);
  atomicAdd(&err->count, 1);
  atomicMin(&err->first_bad, i + 0LL);
}

// Tables of one zone in shared memory (smem_d: locate_smem_bytes(g)).
__device__ __forceinline__ SmemZone stage_zone(const DevGeom& g, double* smem_d) {
  SmemZone z;
  double* p = smem_d;
  float* fp = reinterpret_cast<float*>(p);
  z.plane = fp; fp += 4 * g.n_faces;
  z.band = fp; fp += g.n_faces;
  z.wm = fp; fp += 3 * g.n_wedge * (g.n_ops + 1);
  z.n32 = fp; fp += 3 * g.n_faces;
  z.tl32 = fp; fp += g.n_faces;
  p = reinterpret_cast<double*>(((uintptr_t)fp + 15) & ~uintptr_t(15));
  z.abc = p; p += 9 * g.n_faces;
  z.normal = p; p += 3 * g.n_faces;
  z.tau_len = p; p += g.n_faces;
  z.wedge = p; p += 3 * g.n_wedge;
  int32_t* ip = reinterpret_cast<int32_t*>(p);
  z.tau = ip; ip += 3 * g.n_faces;
  z.ops = ip; ip += 9 * g.n_ops;
  z.opinv = ip;
  for (int i = threadIdx.x; i < 9 * g.n_faces; i += blockDim.x) z.abc[i] = g.face_abc[i];
  for (int i = threadIdx.x; i < 3 * g.n_faces; i += blockDim.x) {
    z.normal[i] = g.face_normal[i];
    z.tau[i] = g.face_tau[i];
  }
  for (int i = threadIdx.x; i < g.n_faces; i += blockDim.x) z.tau_len[i] = g.face_tau_len[i];
  for (int i = threadIdx.x; i < 3 * g.n_wedge; i += blockDim.x) z.wedge[i] = g.wedge_normal[i];
  for (int i = threadIdx.x; i < 9 * g.n_ops; i += blockDim.x) z.ops[i] = g.ops[i];
  for (int i = threadIdx.x; i < g.n_ops; i += blockDim.x) z.opinv[i] = g.op_inverse[i];
  if (g.screen) {
    for (int i = threadIdx.x; i < 4 * g.n_faces; i += blockDim.x) z.plane[i] = g.face_plane32[i];
    for (int i = threadIdx.x; i < g.n_faces; i += blockDim.x) z.band[i] = g.face_band32[i];
    for (int i = threadIdx.x; i < 3 * g.n_wedge * (g.n_ops + 1); i += blockDim.x) z.wm[i] = g.wedge_m32[i];
    for (int i = threadIdx.x; i < 3 * g.n_faces; i += blockDim.x) z.n32[i] = (float)g.face_normal[i];
    for (int i = threadIdx.x; i < g.n_faces; i += blockDim.x) z.tl32[i] = (float)g.face_tau_len[i];
  }
  return z;
}

// Node weights and the remaining records (node, tetrahedron, weights,
// status, group key) of the q at record index i whose trellis coordinates
// x lie in node (node < 0: not found).  Returns its status.
__device__ __forceinline__ int locate_finish(const DevGeom& g, long long node, const double x[3], long long i,
                                             const Records& r, int key_base, int key_fail) {
  int32_t nt[2] = {(int32_t)node, -1}, vi[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  double w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int nw = 0, st = 0;
  if (node < 0) {
    st = BRX_ERR_NOT_FOUND;
  } else {
    int k = node_weights(g, node, x, &nt[1], vi, w);
    if (k > 0) nw = k;
    else st = (k == 0) ? BRX_ERR_NOT_FOUND : -k;
  }
  r.node[2 * i] = nt[0]; r.node[2 * i + 1] = nt[1];
  r.nw[i] = nw;
#pragma unroll
  for (int k = 0; k < 8; ++k) { r.vidx[8 * i + k] = vi[k]; r.w[8 * i + k] = w[k]; }
  // FP64→FP32 conversions run on the FP64 pipe: once here, not per mode
  if (r.w32) {
    float4* w4 = reinterpret_cast<float4*>(r.w32 + 8 * i);
    w4[0] = make_float4((float)w[0], (float)w[1], (float)w[2], (float)w[3]);
    w4[1] = make_float4((float)w[4], (float)w[5], (float)w[6], (float)w[7]);
  }
  r.status[i] = st;
  int32_t key = (int32_t)n_group_keys(g.n_cube, g.n_tets);  // failed q: last bucket
  if (!st) {
    if (nt[1] < 0) {
      const int32_t ni = __ldg(g.node_index + node);
      const int32_t* cv = g.cube_vertices + 8 * (long long)ni;
      int slot = 0;
      for (int j = 0; j < 8; ++j)
        if (__ldg(cv + 7 - j) == vi[0]) { slot = j; break; }
      key = 8 * __ldg(g.cube_rank + ni) + slot;
    } else {
      const int32_t* tv = g.tet_vertices + 4 * (long long)nt[1];
      int slot = 0;
      for (int j = 0; j < 4; ++j)
        if (__ldg(tv + j) == vi[0]) { slot = j; break; }
      key = (int32_t)(8LL * g.n_cube + 4LL * nt[1] + slot);
    }
  }
  r.key[i] = st ? key_fail : key_base + key;
  return st;
}

// Failed move or wedge search: empty records with status st.
__device__ __forceinline__ void locate_failed(long long i, int st, const Records& r, int key_fail) {
  r.node[2 * i] = -1; r.node[2 * i + 1] = -1;
  r.nw[i] = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) { r.vidx[8 * i + k] = 0; r.w[8 * i + k] = 0.0; }
  if (r.w32) {
    float4* w4 = reinterpret_cast<float4*>(r.w32 + 8 * i);
    w4[0] = w4[1] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  r.status[i] = st;
  r.key[i] = key_fail;
}

// Move and wedge search of the q at Qq (records q_ir, τ, R at index i) and
// its trellis coordinates and node.  Returns the status of the move.
__device__ __forceinline__ int locate_front(const DevGeom& g, const SmemZone& z, const double* Qq, long long i,
                                            int mode, const Records& r, double x[3], long long* node) {
  double Qi[3] = {Qq[0], Qq[1], Qq[2]};
  double q[3];
  int32_t tau[3] = {0, 0, 0}, rot[2] = {g.identity, g.identity};
  int st = 0;
  if (mode == 2) {
    q[0] = Qi[0]; q[1] = Qi[1]; q[2] = Qi[2];
  } else {
    st = moveinto_one(g, z, Qi, q, tau);
    if (!st && mode == 1) st = wedge_one(g, z, q, rot);
  }
  r.q_ir[3 * i] = q[0]; r.q_ir[3 * i + 1] = q[1]; r.q_ir[3 * i + 2] = q[2];
  if (r.tau) { r.tau[3 * i] = tau[0]; r.tau[3 * i + 1] = tau[1]; r.tau[3 * i + 2] = tau[2]; }
  r.rot[2 * i] = rot[0]; r.rot[2 * i + 1] = rot[1];
  *node = -1;
  if (!st) {
    hkl_to_xyz(x, g.outer_B, q);
    *node = node_subscript(g, x);
  }
  return st;
}

// q whose node is a polyhedron wait in a CTA queue and are finished
// together, a full warp at a time: the tetrahedron path is long and taken
// by few q, and per-lane it would hold every warp that has one such q.
template <int CAP>
struct PolyQueue {
  int count;
  long long rec[CAP];   // record index
  long long qerr[CAP];  // index reported with an error
  long long node[CAP];
  double x[CAP][3];
};

template <int CAP>
__device__ __forceinline__ void poly_push(PolyQueue<CAP>& pq, long long i, long long qerr, long long node,
                                          const double x[3]) {
  const int k = atomicAdd(&pq.count, 1);
  pq.rec[k] = i;
  pq.qerr[k] = qerr;
  pq.node[k] = node;
  pq.x[k][0] = x[0]; pq.x[k][1] = x[1]; pq.x[k][2] = x[2];
}

// All threads of the CTA: finish every queued q, then empty the queue.
template <int CAP>
__device__ __forceinline__ void poly_drain(PolyQueue<CAP>& pq, const DevGeom& g, const Records& r, int key_base,
                                           int key_fail, ErrorWord* err) {
  __syncthreads();
  const int c = pq.count;
  for (int k = threadIdx.x; k < c; k += blockDim.x) {
    const double x[3] = {pq.x[k][0], pq.x[k][1], pq.x[k][2]};
    const int st = locate_finish(g, pq.node[k], x, pq.rec[k], r, key_base, key_fail);
    if (st) report(err, pq.qerr[k], st);
  }
  __syncthreads();
  if (threadIdx.x == 0) pq.count = 0;
  __syncthreads();
}

// One q: front, then either its cube (or failure) finished here or its
// polyhedron queued.
template <int CAP>
__device__ __forceinline__ void locate_step(const DevGeom& g, const SmemZone& z, PolyQueue<CAP>& pq, const double* Qq,
                                            long long i, long long qerr, int mode, const Records& r, int key_base,
                                            int key_fail, ErrorWord* err) {
  double x[3] = {0.0, 0.0, 0.0};
  long long node = -1;
  int st = locate_front(g, z, Qq, i, mode, r, x, &node);
  if (st) {
    locate_failed(i, st, r, key_fail);
  } else if (node >= 0 && __ldg(g.node_type + node) == BRX_NODE_POLY) {
    poly_push(pq, i, qerr, node, x);
    return;
  } else {
    st = locate_finish(g, node, x, i, r, key_base, key_fail);
  }
  if (st) report(err, qerr, st);
}

constexpr int kPolyCap = 2 * kLocateThreads;

// mode: 0 interpolate_at (moveinto), 1 ir_interpolate_at (ir_moveinto),
// 2 no move (Q already in the trellis domain)
__global__ void __launch_bounds__(kLocateThreads)
locate_kernel(DevGeom g, const double* __restrict__ Q, long long n, long long base, int mode,
              Records r, ErrorWord* err) {
  extern __shared__ double smem_d[];
  __shared__ PolyQueue<kPolyCap> pq;
  const SmemZone z = stage_zone(g, smem_d);
  if (threadIdx.x == 0) pq.count = 0;
  __syncthreads();
  const int key_fail = (int)n_group_keys(g.n_cube, g.n_tets);
  // rounds of one q per thread, the same count for every thread of the CTA
  for (long long i0 = blockIdx.x * (long long)blockDim.x; i0 < n; i0 += (long long)gridDim.x * blockDim.x) {
    const long long i = i0 + threadIdx.x;
    if (i < n) locate_step(g, z, pq, Q + 3 * i, i, base + i, mode, r, 0, key_fail, err);
    __syncthreads();
    if (pq.count >= (int)blockDim.x) poly_drain(pq, g, r, 0, key_fail, err);
  }
  poly_drain(pq, g, r, 0, key_fail, err);
}

// Many trellises in one persistent launch.  Work comes in tiles of one
// item's q (tiles[t] = item, first q, count); a CTA restages the zone
// tables whenever its next tile belongs to another item.  Records are
// batch-wide (item i's q start at q_off[i]); each item reads its Q through
// Qptr[i] and reports errors into err[i] with item-local q indices.
template <int THREADS>
__global__ void __launch_bounds__(THREADS, 512 / THREADS)
locate_batch_kernel(const DevGeom* __restrict__ geoms, const long long* __restrict__ q_off,
                    const int32_t* __restrict__ key_off, int key_fail, const int4* __restrict__ tiles, int n_tiles,
                    const double* const* __restrict__ Qptr, int mode, Records r, ErrorWord* err) {
  extern __shared__ double smem_d[];
  __shared__ DevGeom s_geom;
  __shared__ PolyQueue<2 * THREADS> pq;
  int cur = -1;
  SmemZone z{};
  if (threadIdx.x == 0) pq.count = 0;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const int4 tile = tiles[t];
    if (tile.x != cur) {
      __syncthreads();  // the previous item's tables are no longer read
      for (int w = threadIdx.x; w < (int)(sizeof(DevGeom) / sizeof(int)); w += THREADS)
        reinterpret_cast<int*>(&s_geom)[w] = reinterpret_cast<const int*>(geoms + tile.x)[w];
      __syncthreads();
      z = stage_zone(s_geom, smem_d);
      __syncthreads();
      cur = tile.x;
    }
    const DevGeom& g = s_geom;
    const double* Q = Qptr[cur];
    const long long qo = q_off[cur];
    const int kb = key_off[cur];
    for (int k0 = 0; k0 < tile.z; k0 += THREADS) {
      const int k = k0 + threadIdx.x;
      const long long il = (long long)tile.y + k;
      if (k < tile.z) locate_step(g, z, pq, Q + 3 * il, qo + il, il, mode, r, kb, key_fail, err + cur);
      __syncthreads();
      if (pq.count >= THREADS) poly_drain(pq, g, r, kb, key_fail, err + cur);
    }
    // the queue holds this item's q only
    poly_drain(pq, g, r, kb, key_fail, err + cur);
  }
}

cudaError_t preload_locate_kernel() {
  cudaFuncAttributes a;
  return cudaFuncGetAttributes(&a, locate_kernel);
}

void launch_locate_batch(const DevGeom* geoms, const long long* q_off, const int32_t* key_off, int key_fail,
                         const int4* tiles, int n_tiles, const double* const* Qptr, int mode, const Records& r,
                         ErrorWord* err, size_t smem, int threads, int grid, cudaStream_t s) {
  if (n_tiles <= 0) return;
  if (grid > n_tiles) grid = n_tiles;
  switch (threads) {
    case 64:
      locate_batch_kernel<64><<<grid, 64, smem, s>>>(geoms, q_off, key_off, key_fail, tiles, n_tiles, Qptr, mode, r, err);
      break;
    case 256:
      locate_batch_kernel<256><<<grid, 256, smem, s>>>(geoms, q_off, key_off, key_fail, tiles, n_tiles, Qptr, mode, r, err);
      break;
    default:
      locate_batch_kernel<128><<<grid, 128, smem, s>>>(geoms, q_off, key_off, key_fail, tiles, n_tiles, Qptr, mode, r, err);
      break;
  }
}

size_t locate_smem_bytes(const DevGeom& g) {
  return sizeof(float) * (9 * (size_t)g.n_faces + 3 * (size_t)g.n_wedge * (g.n_ops + 1)) + 16 +
         sizeof(double) * (13 * (size_t)g.n_faces + 3 * (size_t)g.n_wedge) +
         sizeof(int32_t) * (3 * (size_t)g.n_faces + 10 * (size_t)g.n_ops) + 16;
}

void launch_locate(const DevGeom& g, const double* Q, long long n, long long base, int mode, const Records& r,
                   ErrorWord* err, int num_sms, cudaStream_t s) {
  if (n <= 0) return;
  long long blocks = (n + kLocateThreads - 1) / kLocateThreads;
  long long cap = (long long)num_sms * 8;
  if (blocks > cap) blocks = cap;
  locate_kernel<<<(unsigned)blocks, kLocateThreads, locate_smem_bytes(g), s>>>(g, Q, n, base, mode, r, err);
}

}  // namespace brx
