// brx_sort: sort() — the mode permutation between every pair of trellis
// vertices that share a node, on the GPU.
//
// The reference builds, for each unordered pair (i < j) among its permutation
// keys, a B×B cost matrix between the modes of vertex i (rows) and vertex j
// (columns) and solves the linear assignment problem on it with LAPJV
// (DualInterpolator::sort / determine_permutation_ij,
// src/interpolatordual.hpp:398-434; cost_matrix :385-396; Interpolator::add_cost,
// src/interpolator_cost.tpp:19-61; cost functions src/interpolator.hpp:246-300,
// src/utilities.tpp:249-431,567-598).  The row → column assignment becomes
// the permutation of key i·N+j and the column → row assignment that of j·N+i.
//
// Here one CTA owns one pair at a time (four warps, one per scheduler, or
// one warp when B < 16), over a contiguous run of keys so that consecutive
// pairs of one vertex keep its rows staged:
//  1. both vertices' rows of values and vectors are copied into the CTA's
//     shared memory (FP64 storage as double, FP32/BF16 storage as float),
//     rows padded to an odd stride so that lanes reading different rows hit
//     different banks;
//  2. the cost matrix is formed in FP64 with the threads over (row, column)
//     pairs.  The antiphase e^{-iθ} of the vectors is conj(h)/|h| of the
//     Hermitian product h over the whole branch, and the vector-part costs
//     use |⟨x, e·y⟩| = |⟨x, y⟩| and Re⟨x, e·y⟩ = Re(e·⟨x, y⟩), which equal the
//     reference's costs up to rounding; scalars, matrices and the distance
//     cost are formed element by element against e·y as the reference does;
//  3. warp 0 solves the assignment exactly by the shortest augmenting path
//     method with row and column potentials: lanes scan columns, a shuffle argmin
//     (ties to the lower column) picks the next column, lanes update the
//     potentials of their columns, lane 0 walks the augmenting path.  The
//     optimum is the one LAPJV finds wherever it is unique;
//  4. lanes scatter both permutations; a ballot flags non-identity pairs.
// The host then gives non-identity permutations ids in key order and a
// second kernel copies their rows into the handle's table; identity pairs
// keep id −1, which the gathers read as the identity, as
// PermutationTable::safe_get does for unset keys.  Every loop is bounded:
// the augmenting search stops with an error when no finite column is left
// (NaN or infinite costs) or after B+1 steps.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <string>
#include <vector>

#include "../../include/brx.h"
#include "brx_handle.h"
#include "brx_kernels.h"

using namespace brx_detail;

namespace {

constexpr int kPairWarps = 4;  // warps of a CTA that owns a pair with B ≥ 16
constexpr unsigned kFull = 0xffffffffu;

// one interpolator (values or vectors) as the cost kernel sees it
struct SortSide {
  const void* data;  // device, n_vertices × B × s elements (complex: pairs)
  int store;         // ST_F64 / ST_F32 / ST_BF16
  int cplx;
  int s, e0, e1, e2;
  int vf;            // vector cost function, reference numbering
  int phase;         // align the phase of y to x first (complex vectors)
  double w0, w1, w2;
  int reals;         // reals per row: s, or 2s for complex
  int rs;            // padded row stride in staged units (odd)
  int off_i, off_j;  // staged rows of vertex i / j: byte offsets in the warp region
  int off_ni, off_nj;  // per row of i / j: vector-part |x|², |x| and 1/|x|² (0 for a zero row), B doubles each
};

struct SortParams {
  SortSide side[2];
  int n_sides;
  int B;
  long long n_vertices;
  long long n_keys;
  const long long* keys;
  int32_t* perm_out;  // n_keys × B
  int32_t* nonid;     // n_keys
  int32_t* status;    // [0] brx_status of the first failure, [1] its key index
  int off_c;          // B×B cost matrix (double)
  int off_lap;        // u, v, minv (double, B+1 each), then p, way, used (int, B+1 each)
  brx::Tol one;       // approx_float::scalar(·, 1.0) tolerance
};

__device__ __forceinline__ void record(const SortParams& P, int st, long long k) {
  if (atomicCAS(P.status, 0, st) == 0) P.status[1] = (int32_t)k;
}

template <typename T>
__device__ __forceinline__ T load_elem(const void* base, int store, long long idx) {
  if (store == brx::ST_F64) return (T) static_cast<const double*>(base)[idx];
  if (store == brx::ST_F32) return (T) static_cast<const float*>(base)[idx];
  return (T)__bfloat162float(static_cast<const __nv_bfloat16*>(base)[idx]);
}

// cos θ from a numerator and two norms, with the reference's zero-norm rule
// and its snap of |cos θ| ≈ 1 (src/utilities.tpp:249-280,357-380)
__device__ __forceinline__ double cos_of(double num, double na, double nb, const brx::Tol& one, bool* bad) {
  double c;
  if (na != 0.0 && nb != 0.0) c = num / (na * nb);
  else c = (na != 0.0 || nb != 0.0) ? 0.0 : 1.0;
  double act = fabs(c);
  if (brx::approx(act, 1.0, one) && act > 1.0) {
    c = c / act;
    act = fabs(c);
  }
  if (act > 1.0) *bad = true;
  return c;
}

// Vector-part norms of one row: |x|², |x| and 1/|x|² (0 for a zero row).
struct RowNorm {
  double n2, n, inv2;
};

// sin² of the angle whose cosine has the square num2·inv2x·inv2y (the
// reference's sin(acos(c))², src/interpolator.hpp:287-294, as 1 − c²): the
// zero-norm rule and the snap of c ≈ ±1 are the reference's; only where c²
// exceeds 1 is c itself formed to decide between the snap and an error.
__device__ __forceinline__ double sin2_of(double num2, const RowNorm& x, const RowNorm& y, const brx::Tol& one,
                                          bool* bad) {
  if (x.n2 == 0.0 || y.n2 == 0.0) return (x.n2 != 0.0 || y.n2 != 0.0) ? 1.0 : 0.0;
  const double c2 = num2 * x.inv2 * y.inv2;
  if (c2 <= 1.0) return 1.0 - c2;
  const double c = cos_of(sqrt(num2), x.n, y.n, one, bad);
  return 1.0 - c * c;
}

// Interpolator::add_cost for one (row a of vertex i, row b of vertex j)
// (src/interpolator_cost.tpp:19-61): w0·scalar + w1·vector + w2·matrix cost.
template <typename T>
__device__ double pair_cost(const SortSide& S, const T* x, const T* y, const RowNorm& nx, const RowNorm& ny,
                            const brx::Tol& one, bool* bad) {
  double sc = 0.0, vc = 0.0, mc = 0.0;
  const int e0 = S.e0, e1 = S.e1, e2 = S.e2, s = S.s;
  if (S.cplx) {
    // Hermitian products ⟨x, y⟩ over the vector part (v) and over the other
    // elements (o); the phase comes from their sum over the whole branch
    double orr = 0.0, oi = 0.0, vr = 0.0, vi = 0.0;
    auto hprod = [&](int k, double& re, double& im) {
      const double xr = (double)x[2 * k], xi = (double)x[2 * k + 1];
      const double yr = (double)y[2 * k], yi = (double)y[2 * k + 1];
      re = fma(xr, yr, re);
      re = fma(xi, yi, re);
      im = fma(xr, yi, im);
      im = fma(-xi, yr, im);
    };
    for (int k = 0; k < e0; ++k) hprod(k, orr, oi);
    for (int k = e0; k < e0 + e1; ++k) hprod(k, vr, vi);
    for (int k = e0 + e1; k < s; ++k) hprod(k, orr, oi);
    const double hr = orr + vr, hi = oi + vi;
    double er = 1.0, ei = 0.0;  // e^{-iθ}, θ = arg⟨x, y⟩ (utilities.tpp:567-578)
    if (S.phase) {
      const double hm = sqrt(hr * hr + hi * hi);
      if (hm > 0.0) {
        er = hr / hm;
        ei = -hi / hm;
      }
    }
    // |x_k − e·y_k| for element k
    auto dist2 = [&](int k) {
      const double yr = (double)y[2 * k], yi = (double)y[2 * k + 1];
      const double dr = (double)x[2 * k] - (er * yr - ei * yi);
      const double di = (double)x[2 * k + 1] - (er * yi + ei * yr);
      return dr * dr + di * di;
    };
    for (int k = 0; k < e0; ++k) sc += sqrt(dist2(k));
    if (e1) {
      switch (S.vf) {
        case 1: {  // vector_distance
          double d = 0.0;
          for (int k = e0; k < e0 + e1; ++k) d += dist2(k);
          vc = sqrt(d);
          break;
        }
        case 2:  // 1 − |⟨x, e·y⟩|²
          vc = 1.0 - (vr * vr + vi * vi);
          break;
        case 3:  // Euclidean angle of the 2n-real vectors x and e·y
          vc = acos(cos_of(er * vr - ei * vi, nx.n, ny.n, one, bad));
          break;
        case 4:  // Hermitian angle
          vc = acos(cos_of(sqrt(vr * vr + vi * vi), nx.n, ny.n, one, bad));
          break;
        default:  // sin² of the Hermitian angle
          vc = sin2_of(vr * vr + vi * vi, nx, ny, one, bad);
      }
    }
    for (int m = 0; m < e2 / 9; ++m) {
      double d = 0.0;
      for (int k = e0 + e1 + 9 * m; k < e0 + e1 + 9 * m + 9; ++k) d += dist2(k);
      mc += sqrt(d);
    }
  } else {
    for (int k = 0; k < e0; ++k) sc += fabs((double)x[k] - (double)y[k]);
    if (e1) {
      if (S.vf == 1) {
        double d = 0.0;
        for (int k = e0; k < e0 + e1; ++k) {
          const double t = (double)x[k] - (double)y[k];
          d += t * t;
        }
        vc = sqrt(d);
      } else {
        double ab = 0.0;
        for (int k = e0; k < e0 + e1; ++k) ab += (double)x[k] * (double)y[k];
        if (S.vf == 2) vc = 1.0 - ab;
        else if (S.vf == 3 || S.vf == 4) vc = acos(cos_of(ab, nx.n, ny.n, one, bad));
        else vc = sin2_of(ab * ab, nx, ny, one, bad);
      }
    }
    for (int m = 0; m < e2 / 9; ++m) {
      double d = 0.0;
      for (int k = e0 + e1 + 9 * m; k < e0 + e1 + 9 * m + 9; ++k) {
        const double t = (double)x[k] - (double)y[k];
        d += t * t;
      }
      mc += sqrt(d);
    }
  }
  return (S.w0 * sc + S.w1 * vc) + S.w2 * mc;
}

// Copy the B rows of one vertex into padded shared-memory rows (four loads
// in flight per thread) and form the norms of their vector parts; all
// threads of the CTA take part.
template <typename T>
__device__ void stage_rows(const SortSide& S, int B, long long vtx, T* dst, RowNorm* nrm) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const long long base = vtx * (long long)B * S.reals;
  const int total = B * S.reals;
  for (int i0 = tid; i0 < total; i0 += 4 * nt) {
    T v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (i0 + nt * u < total) v[u] = load_elem<T>(S.data, S.store, base + i0 + nt * u);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int idx = i0 + nt * u;
      if (idx < total) {
        const int r = idx / S.reals;
        dst[r * S.rs + (idx - r * S.reals)] = v[u];
      }
    }
  }
  __syncthreads();
  const int m = S.cplx ? 2 : 1;
  for (int r = tid; r < B; r += nt) {
    double n2 = 0.0;
    const T* row = dst + r * S.rs;
    for (int k = m * S.e0; k < m * (S.e0 + S.e1); ++k) n2 += (double)row[k] * (double)row[k];
    nrm[r].n2 = n2;
    nrm[r].n = sqrt(n2);
    nrm[r].inv2 = n2 > 0.0 ? 1.0 / n2 : 0.0;
  }
}

// Exact assignment for the n×n cost matrix C (row-major) by shortest
// augmenting paths with potentials; columns 1..n belong to lanes, column 0 is
// the virtual start.  On return p[j] (j = 1..n) is the 1-based row matched to
// column j.  Returns false when no finite column can be reached.
__device__ bool assign_warp(const double* C, int n, double* u, double* v, double* minv, int* p, int* way,
                            int* used, int lane) {
  for (int j = lane; j <= n; j += 32) {
    u[j] = 0.0;
    v[j] = 0.0;
    p[j] = 0;
    way[j] = 0;
  }
  __syncwarp();
  for (int i = 1; i <= n; ++i) {
    for (int j = lane; j <= n; j += 32) {
      minv[j] = DBL_MAX;
      used[j] = 0;
    }
    __syncwarp();
    if (lane == 0) p[0] = i;
    int j0 = 0;
    for (int step = 0;; ++step) {
      if (lane == 0) used[j0] = 1;
      __syncwarp();
      const int i0 = p[j0];
      const double ui0 = u[i0];
      const double* row = C + (size_t)(i0 - 1) * n;
      double best = DBL_MAX;
      int bj = 0;
      for (int j = 1 + lane; j <= n; j += 32) {
        if (!used[j]) {
          const double cur = (row[j - 1] - ui0) - v[j];
          double mv = minv[j];
          if (cur < mv) {
            mv = cur;
            minv[j] = cur;
            way[j] = j0;
          }
          if (mv < best) {
            best = mv;
            bj = j;
          }
        }
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const double ob = __shfl_xor_sync(kFull, best, o);
        const int oj = __shfl_xor_sync(kFull, bj, o);
        if (ob < best || (ob == best && oj < bj)) {
          best = ob;
          bj = oj;
        }
      }
      if (bj == 0 || step > n) return false;
      const double delta = best;
      __syncwarp();
      for (int j = lane; j <= n; j += 32) {
        if (used[j]) {
          u[p[j]] += delta;
          v[j] -= delta;
        } else {
          minv[j] -= delta;
        }
      }
      __syncwarp();
      j0 = bj;
      if (p[j0] == 0) break;
    }
    if (lane == 0) {
      int jj = j0;
      for (int guard = 0; jj != 0 && guard <= n; ++guard) {
        const int j1 = way[jj];
        p[jj] = p[j1];
        jj = j1;
      }
    }
    __syncwarp();
  }
  return true;
}

__device__ long long find_key(const long long* keys, long long n, long long key) {
  long long lo = 0, hi = n;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (keys[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return (lo < n && keys[lo] == key) ? lo : -1;
}

// One vertex pair at a time per CTA (one warp for B < 16, else four: one per
// scheduler, so that the FP64 cost matrix keeps every FP64 pipe of the SM
// fed); warp 0 then solves the assignment and writes both permutations.
template <typename T>
__global__ void __launch_bounds__(32 * kPairWarps) sort_pairs_kernel(SortParams P) {
  extern __shared__ __align__(16) unsigned char region[];
  const int tid = threadIdx.x, lane = tid & 31;
  const int B = P.B;
  double* C = reinterpret_cast<double*>(region + P.off_c);
  double* u = reinterpret_cast<double*>(region + P.off_lap);
  double* v = u + (B + 1);
  double* minv = v + (B + 1);
  int* p = reinterpret_cast<int*>(minv + (B + 1));
  int* way = p + (B + 1);
  int* used = way + (B + 1);
  // each CTA takes a contiguous run of keys: consecutive keys share vertex
  // i, whose rows stay staged
  const long long per = (P.n_keys + gridDim.x - 1) / gridDim.x;
  const long long k_end = min(P.n_keys, ((long long)blockIdx.x + 1) * per);
  long long staged_i = -1;
  for (long long k = (long long)blockIdx.x * per; k < k_end; ++k) {
    const long long key = P.keys[k];
    const long long i = key / P.n_vertices, j = key - i * P.n_vertices;
    // every key needs its reverse (the reference's overwrite of j·N+i fails without it)
    const long long kr = find_key(P.keys, P.n_keys, j * P.n_vertices + i);
    if (kr < 0) {
      if (tid == 0) record(P, BRX_ERR_INVALID_ARGUMENT, k);
      continue;
    }
    if (i >= j) continue;
    __syncthreads();  // the previous pair's assignment is done with the shared rows
    for (int sd = 0; sd < P.n_sides; ++sd) {
      const SortSide& S = P.side[sd];
      if (i != staged_i)
        stage_rows<T>(S, B, i, reinterpret_cast<T*>(region + S.off_i), reinterpret_cast<RowNorm*>(region + S.off_ni));
      stage_rows<T>(S, B, j, reinterpret_cast<T*>(region + S.off_j), reinterpret_cast<RowNorm*>(region + S.off_nj));
    }
    staged_i = i;
    __syncthreads();
    bool bad = false;
    for (int q = tid; q < B * B; q += blockDim.x) {
      const int a = q / B, b = q - a * B;
      double c = 0.0;
      for (int sd = 0; sd < P.n_sides; ++sd) {
        const SortSide& S = P.side[sd];
        const T* x = reinterpret_cast<const T*>(region + S.off_i) + a * S.rs;
        const T* y = reinterpret_cast<const T*>(region + S.off_j) + b * S.rs;
        const RowNorm nx = reinterpret_cast<const RowNorm*>(region + S.off_ni)[a];
        const RowNorm ny = reinterpret_cast<const RowNorm*>(region + S.off_nj)[b];
        c += pair_cost<T>(S, x, y, nx, ny, P.one, &bad);
      }
      C[q] = c;
    }
    if (__syncthreads_or(bad)) {  // also the barrier after which C is complete
      if (tid == 0) record(P, BRX_ERR_IMPOSSIBLE, k);
      continue;
    }
    if (tid < 32) {
      if (!assign_warp(C, B, u, v, minv, p, way, used, lane)) {
        if (lane == 0) record(P, BRX_ERR_IMPOSSIBLE, k);
      } else {
        bool moved = false, unmatched = false;
        for (int jj = 1 + lane; jj <= B; jj += 32) {
          const int r = p[jj] - 1;
          if (r < 0 || r >= B) {
            unmatched = true;
            continue;
          }
          P.perm_out[k * B + r] = jj - 1;   // row (mode of i) → column (mode of j)
          P.perm_out[kr * B + jj - 1] = r;  // column → row
          moved |= (r != jj - 1);
        }
        if (__any_sync(kFull, unmatched) && lane == 0) record(P, BRX_ERR_IMPOSSIBLE, k);
        const bool any = __any_sync(kFull, moved);
        if (lane == 0) {
          P.nonid[k] = any;
          P.nonid[kr] = any;
        }
      }
    }
  }
}

__global__ void compact_perms_kernel(const int32_t* ids, const int32_t* perm_out, long long n_keys, int B,
                                     int32_t* perms) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n_keys * B; t += stride) {
    const long long k = t / B;
    const int id = ids[k];
    if (id >= 0) perms[(long long)id * B + (t - k * B)] = perm_out[t];
  }
}

brx_status side_from(brx_handle* h, const Interp& d, const brx_sort_cost* c, bool vectors, SortSide* S) {
  S->data = d.data.p;
  S->store = d.store;
  S->cplx = d.cplx;
  S->s = d.s;
  S->e0 = d.el[0];
  S->e1 = d.el[1];
  S->e2 = d.el[2];
  S->vf = c ? c->vector_fn : 0;
  S->phase = vectors && d.cplx;
  S->w0 = c ? c->weight[0] : 1.0;
  S->w1 = c ? c->weight[1] : 1.0;
  S->w2 = c ? c->weight[2] : 1.0;
  S->reals = d.s * (d.cplx ? 2 : 1);
  S->rs = S->reals | 1;
  if (c && c->scalar_fn != 0)
    return fail(h, BRX_ERR_UNSUPPORTED, "scalar cost function " + std::to_string(c->scalar_fn) +
                                            " is not defined; the reference's only one is 0 (sum of |a-b|)");
  return BRX_OK;
}

}  // namespace

extern "C" brx_status brx_sort(brx_handle* h, int64_t n_keys, const int64_t* keys, const brx_sort_cost* values_cost,
                               const brx_sort_cost* vectors_cost, void* stream) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (!h->filled) return fail(h, BRX_ERR_NOT_FILLED, "The interpolation data must be filled before sorting.");
  if (n_keys < 0 || (n_keys > 0 && !keys)) return fail(h, BRX_ERR_INVALID_ARGUMENT, "invalid permutation keys");
  const long long N = h->host_geom.n_vertices;
  const int B = h->vals.B;
  // keys: strictly increasing, each a pair of distinct vertices; the kernel
  // checks that (j, i) is listed for every (i, j) (the reference's overwrite
  // of j·N+i fails on a missing key, permutation_table.hpp:173-184)
  for (long long k = 0; k < n_keys; ++k) {
    if (k && keys[k] <= keys[k - 1]) return fail(h, BRX_ERR_INVALID_ARGUMENT, "permutation keys must be strictly increasing");
    const long long i = keys[k] / N, j = keys[k] - (keys[k] / N) * N;
    if (keys[k] < 0 || i >= N || i == j)
      return fail(h, BRX_ERR_INVALID_ARGUMENT, "permutation key " + std::to_string(keys[k]) + " is not a pair of distinct vertices");
  }
  SortParams P{};
  P.B = B;
  P.n_vertices = N;
  P.n_keys = n_keys;
  P.n_sides = h->vecs.present ? 2 : 1;
  brx_status st = side_from(h, h->vals, values_cost, false, &P.side[0]);
  if (st) return st;
  if (P.n_sides == 2) {
    st = side_from(h, h->vecs, vectors_cost, true, &P.side[1]);
    if (st) return st;
  }
  P.one = brx::make_tol(0.0, 1);
  // staged precision: double for FP64 storage, float otherwise
  const bool f64 = h->vals.store == ST_F64;
  const size_t esz = f64 ? sizeof(double) : sizeof(float);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    off = (off + 15) & ~(size_t)15;
    const size_t o = off;
    off += bytes;
    return (int)o;
  };
  for (int sd = 0; sd < P.n_sides; ++sd) {
    SortSide& S = P.side[sd];
    S.off_i = take(esz * B * S.rs);
    S.off_j = take(esz * B * S.rs);
    S.off_ni = take(3 * sizeof(double) * B);
    S.off_nj = take(3 * sizeof(double) * B);
  }
  P.off_c = take(sizeof(double) * B * B);
  P.off_lap = take(sizeof(double) * 3 * (B + 1) + sizeof(int) * 3 * (B + 1));
  const size_t pair_bytes = (off + 15) & ~(size_t)15;
  if (pair_bytes > h->smem_optin)
    return fail(h, BRX_ERR_UNSUPPORTED,
                "sort: one vertex pair needs " + std::to_string(pair_bytes) + " bytes of shared memory (more than " +
                    std::to_string(h->smem_optin) + "); use FP32 storage or fewer branches");
  BRX_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t cs = stream ? static_cast<cudaStream_t>(stream) : h->sc[0].stream;
  h->n_keys = 0;
  h->n_perms = 0;
  // the antiphase table follows the permutations: until it is rebuilt the
  // gather forms its factors per group
  h->ph_valid = false;
  if (n_keys == 0) return build_phase_table(h);
  // transient buffers of this call, released on every return
  struct Transient {
    DevBuf out, flag, status;
    ~Transient() {
      out.release();
      flag.release();
      status.release();
    }
  } tr;
  DevBuf& d_out = tr.out;
  DevBuf& d_flag = tr.flag;
  DevBuf& d_status = tr.status;
  BRX_CUDA(h, h->perm_keys.ensure(sizeof(int64_t) * n_keys));
  BRX_CUDA(h, h->perm_ids.ensure(sizeof(int32_t) * n_keys));
  BRX_CUDA(h, d_out.ensure(sizeof(int32_t) * (size_t)n_keys * B));
  BRX_CUDA(h, d_flag.ensure(sizeof(int32_t) * n_keys));
  BRX_CUDA(h, d_status.ensure(sizeof(int32_t) * 2));
  BRX_CUDA(h, cudaMemcpyAsync(h->perm_keys.p, keys, sizeof(int64_t) * n_keys, cudaMemcpyHostToDevice, cs));
  BRX_CUDA(h, cudaMemsetAsync(d_flag.p, 0, sizeof(int32_t) * n_keys, cs));
  BRX_CUDA(h, cudaMemsetAsync(d_status.p, 0, sizeof(int32_t) * 2, cs));
  P.keys = static_cast<const long long*>(h->perm_keys.p);
  P.perm_out = static_cast<int32_t*>(d_out.p);
  P.nonid = static_cast<int32_t*>(d_flag.p);
  P.status = static_cast<int32_t*>(d_status.p);
  // one pair per CTA: four warps (one per scheduler) once the cost matrix
  // has enough entries to share, one below
  const int warps = B * B >= 256 ? kPairWarps : 1;
  const size_t dyn = pair_bytes;
  const void* fn = f64 ? (const void*)sort_pairs_kernel<double> : (const void*)sort_pairs_kernel<float>;
  BRX_CUDA(h, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  int per_sm = 0;
  BRX_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * warps, dyn));
  long long grid = (long long)std::max(1, per_sm) * h->num_sms;
  grid = std::max<long long>(1, std::min<long long>(grid, n_keys));
  if (f64) sort_pairs_kernel<double><<<(unsigned)grid, 32 * warps, dyn, cs>>>(P);
  else sort_pairs_kernel<float><<<(unsigned)grid, 32 * warps, dyn, cs>>>(P);
  BRX_CUDA(h, cudaGetLastError());
  h->launches += 1;
  std::vector<int32_t> flag(n_keys);
  int32_t status[2] = {0, 0};
  BRX_CUDA(h, cudaMemcpyAsync(flag.data(), d_flag.p, sizeof(int32_t) * n_keys, cudaMemcpyDeviceToHost, cs));
  BRX_CUDA(h, cudaMemcpyAsync(status, d_status.p, sizeof(status), cudaMemcpyDeviceToHost, cs));
  BRX_CUDA(h, cudaStreamSynchronize(cs));
  if (status[0]) {
    const long long k = status[1];
    const long long key = (k >= 0 && k < n_keys) ? keys[k] : -1;
    const std::string pair = "(" + std::to_string(key / N) + ", " + std::to_string(key % N) + ")";
    if (status[0] == BRX_ERR_INVALID_ARGUMENT) return fail(h, BRX_ERR_INVALID_ARGUMENT, "Can not overwrite a non-existant key");
    return fail(h, (brx_status)status[0],
                "sort: vertex pair " + pair + " gives a cosine above 1 or a cost matrix without a finite assignment");
  }
  // ids of the non-identity permutations in key order
  int32_t n_perm = 0;
  for (long long k = 0; k < n_keys; ++k) flag[k] = flag[k] ? n_perm++ : -1;
  BRX_CUDA(h, cudaMemcpyAsync(h->perm_ids.p, flag.data(), sizeof(int32_t) * n_keys, cudaMemcpyHostToDevice, cs));
  if (n_perm > 0) {
    BRX_CUDA(h, h->perms.ensure(sizeof(int32_t) * (size_t)n_perm * B));
    const long long total = n_keys * B;
    const int threads = 256;
    const long long blocks = std::min<long long>((total + threads - 1) / threads, (long long)h->num_sms * 16);
    compact_perms_kernel<<<(unsigned)blocks, threads, 0, cs>>>(static_cast<const int32_t*>(h->perm_ids.p),
                                                               static_cast<const int32_t*>(d_out.p), n_keys, B,
                                                               static_cast<int32_t*>(h->perms.p));
    BRX_CUDA(h, cudaGetLastError());
    h->launches += 1;
  }
  BRX_CUDA(h, cudaStreamSynchronize(cs));
  h->n_keys = n_keys;
  h->n_perms = n_perm;
  return build_phase_table(h);
}

extern "C" brx_status brx_get_permutations(brx_handle* h, int64_t n_keys, int64_t* keys_out, int32_t* perms_out) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (n_keys != h->n_keys)
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "the handle holds " + std::to_string(h->n_keys) + " permutation keys");
  if (n_keys == 0) return BRX_OK;
  if (!keys_out || !perms_out) return fail(h, BRX_ERR_INVALID_ARGUMENT, "output buffers must be provided");
  const int B = h->vals.B;
  BRX_CUDA(h, cudaSetDevice(h->device));
  std::vector<int32_t> ids(n_keys), perms((size_t)h->n_perms * B);
  BRX_CUDA(h, cudaMemcpy(keys_out, h->perm_keys.p, sizeof(int64_t) * n_keys, cudaMemcpyDeviceToHost));
  BRX_CUDA(h, cudaMemcpy(ids.data(), h->perm_ids.p, sizeof(int32_t) * n_keys, cudaMemcpyDeviceToHost));
  if (h->n_perms)
    BRX_CUDA(h, cudaMemcpy(perms.data(), h->perms.p, sizeof(int32_t) * perms.size(), cudaMemcpyDeviceToHost));
  for (long long k = 0; k < n_keys; ++k) {
    const int id = ids[k];
    for (int b = 0; b < B; ++b)
      perms_out[k * B + b] = (id >= 0 && id < h->n_perms) ? perms[(size_t)id * B + b] : b;
  }
  return BRX_OK;
}

extern "C" int64_t brx_permutation_count(const brx_handle* h) { return h ? h->n_keys : 0; }
