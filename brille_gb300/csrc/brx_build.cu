// Trellis construction on the GPU: node classification of the knot grid and
// the tetrahedra of the cells the irreducible polyhedron's surface cuts.
//
// The reference builds its PolyTrellis on the host (PolyTrellis::construct,
// src/trellis_poly_parallel.tpp:74-482): cells wholly inside the polyhedron
// are cube nodes, cells it cuts are intersected with it and tetrahedralised
// by TetGen, the rest are null.  Here every cell is one thread:
//
//   classify_kernel   the 8 corners' signed distances to the polyhedron's
//                     planes: cube, null (all corners outside one plane) or
//                     cut;
//   cut_cell_kernel   the corners of cell ∩ polyhedron (cell corners
//                     inside, polyhedron vertices in the cell, cell edges
//                     through planes, polyhedron edges through cell faces),
//                     merged within tol and clamped to the cell, kept if
//                     they span a volume; a count pass, then a write pass
//                     at scanned offsets;
//   fan_kernel        the convex polytope split into tetrahedra: a fan from
//                     its first corner over every facet (a plane holding ≥ 3
//                     corners, the first corner not among them), each facet
//                     polygon ordered by angle and fanned from its first
//                     corner.  Pyramids from one corner over the facets that
//                     do not contain it tile a convex polytope exactly.
//
// All arithmetic is FP64.  The host merges the cut cells' corners with the
// knot points of the cube nodes into one vertex list (that merge is global
// and needs a spatial index; brille_gb300.trellis does it).
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/brx.h"

namespace {

constexpr int kMaxPoints = 128;  // corners of one cut polytope
constexpr int kMaxPlanes = 64;   // planes of the polyhedron
constexpr int kMaxTets = 512;    // tetrahedra of one cut polytope

// corner c of a cell: bit pattern (x, y, z) in the cube-node order
// (000)(100)(110)(010)(101)(001)(011)(111)
__constant__ int c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                   {1, 0, 1}, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}};
// the 12 cell edges as corner pairs
__constant__ int c_edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {5, 4}, {4, 7},
                                  {7, 6}, {6, 5}, {0, 5}, {1, 4}, {2, 7}, {3, 6}};

struct BuildArgs {
  const double* kn[3];
  int nk[3];
  int nv, np, ne;
  const double* verts;   // nv × 3
  const double* planes;  // np × 4
  const int32_t* edges;  // ne × 2
  double tol;
  int always_triangulate;
};

__device__ __forceinline__ double plane_dist(const double* pl, const double* x) {
  return pl[0] * x[0] + pl[1] * x[1] + pl[2] * x[2] + pl[3];
}

__device__ __forceinline__ void cell_box(const BuildArgs& a, long long cell, double lo[3], double hi[3]) {
  const int nx = a.nk[0] - 1, ny = a.nk[1] - 1;
  const int sub[3] = {(int)(cell % nx), (int)((cell / nx) % ny), (int)(cell / ((long long)nx * ny))};
  for (int d = 0; d < 3; ++d) {
    lo[d] = a.kn[d][sub[d]];
    hi[d] = a.kn[d][sub[d] + 1];
  }
}

// 0 null, 1 cube, 3 cut
__global__ void classify_kernel(BuildArgs a, long long n_cells, int32_t* type) {
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < n_cells;
       cell += (long long)gridDim.x * blockDim.x) {
    double lo[3], hi[3];
    cell_box(a, cell, lo, hi);
    bool all_in = true;
    unsigned long long out_all = ~0ULL;  // planes every corner lies outside of
    for (int c = 0; c < 8; ++c) {
      const double x[3] = {c_corner[c][0] ? hi[0] : lo[0], c_corner[c][1] ? hi[1] : lo[1],
                           c_corner[c][2] ? hi[2] : lo[2]};
      unsigned long long out = 0;
      for (int h = 0; h < a.np; ++h) {
        const double d = plane_dist(a.planes + 4 * h, x);
        if (d > a.tol) {
          out |= 1ULL << h;
          all_in = false;
        }
      }
      out_all &= out;
    }
    int t = 3;
    if (out_all) t = 0;
    else if (all_in && !a.always_triangulate) t = 1;
    type[cell] = t;
  }
}

// The corners of cell ∩ polyhedron, merged within tol and clamped to the
// cell; 0 when fewer than 4 or flat.  Returns -1 when more than kMaxPoints.
__device__ int cut_points(const BuildArgs& a, long long cell, double (*pts)[3]) {
  double lo[3], hi[3];
  cell_box(a, cell, lo, hi);
  const double tol = a.tol;
  double cx[8][3];
  for (int c = 0; c < 8; ++c)
    for (int d = 0; d < 3; ++d) cx[c][d] = c_corner[c][d] ? hi[d] : lo[d];
  int n = 0;
  bool over = false;
  auto push = [&](const double* x) {
    // merged within tol with what is already there
    for (int i = 0; i < n; ++i) {
      const double dx = x[0] - pts[i][0], dy = x[1] - pts[i][1], dz = x[2] - pts[i][2];
      if (sqrt(dx * dx + dy * dy + dz * dz) < tol) return;
    }
    if (n == kMaxPoints) {
      over = true;
      return;
    }
    for (int d = 0; d < 3; ++d) pts[n][d] = x[d];
    ++n;
  };
  auto inside = [&](const double* x) {
    for (int h = 0; h < a.np; ++h)
      if (plane_dist(a.planes + 4 * h, x) > tol) return false;
    return true;
  };
  // cell corners inside the polyhedron
  for (int c = 0; c < 8; ++c)
    if (inside(cx[c])) push(cx[c]);
  // polyhedron vertices inside the cell
  for (int v = 0; v < a.nv; ++v) {
    const double* x = a.verts + 3 * v;
    bool in = true;
    for (int d = 0; d < 3; ++d) in = in && x[d] >= lo[d] - tol && x[d] <= hi[d] + tol;
    if (in) push(x);
  }
  // cell edges crossing polyhedron planes
  for (int e = 0; e < 12; ++e) {
    const double* pa = cx[c_edge[e][0]];
    const double* pb = cx[c_edge[e][1]];
    for (int h = 0; h < a.np; ++h) {
      const double da = plane_dist(a.planes + 4 * h, pa), db = plane_dist(a.planes + 4 * h, pb);
      if ((da < -tol && db > tol) || (da > tol && db < -tol)) {
        const double t = da / (da - db);
        double x[3];
        for (int d = 0; d < 3; ++d) x[d] = pa[d] + t * (pb[d] - pa[d]);
        if (inside(x)) push(x);
      }
    }
  }
  // polyhedron edges crossing cell faces
  for (int e = 0; e < a.ne; ++e) {
    const double* pa = a.verts + 3 * a.edges[2 * e];
    const double* pb = a.verts + 3 * a.edges[2 * e + 1];
    for (int ax = 0; ax < 3; ++ax)
      for (int side = 0; side < 2; ++side) {
        const double plane = side ? hi[ax] : lo[ax];
        const double ua = pa[ax] - plane, ub = pb[ax] - plane;
        if ((ua < -tol && ub > tol) || (ua > tol && ub < -tol)) {
          const double t = ua / (ua - ub);
          double x[3];
          for (int d = 0; d < 3; ++d) x[d] = pa[d] + t * (pb[d] - pa[d]);
          x[ax] = plane;
          bool in = true;
          for (int d = 0; d < 3; ++d) in = in && x[d] >= lo[d] - tol && x[d] <= hi[d] + tol;
          if (in) push(x);
        }
      }
  }
  if (over) return -1;
  if (n < 4) return 0;
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) pts[i][d] = fmin(fmax(pts[i][d], lo[d]), hi[d]);
  // flat: no corner off the plane through three spread corners by more
  // than 1e-9 of the cell's size
  const double span = fmax(hi[0] - lo[0], fmax(hi[1] - lo[1], hi[2] - lo[2]));
  int i1 = 0;
  double best = 0;
  for (int i = 1; i < n; ++i) {
    const double dx = pts[i][0] - pts[0][0], dy = pts[i][1] - pts[0][1], dz = pts[i][2] - pts[0][2];
    const double r = dx * dx + dy * dy + dz * dz;
    if (r > best) { best = r; i1 = i; }
  }
  double u[3] = {pts[i1][0] - pts[0][0], pts[i1][1] - pts[0][1], pts[i1][2] - pts[0][2]};
  int i2 = 0;
  best = 0;
  double nrm[3] = {0, 0, 0};
  for (int i = 1; i < n; ++i) {
    const double w[3] = {pts[i][0] - pts[0][0], pts[i][1] - pts[0][1], pts[i][2] - pts[0][2]};
    const double c[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
    const double r = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
    if (r > best) { best = r; i2 = i; nrm[0] = c[0]; nrm[1] = c[1]; nrm[2] = c[2]; }
  }
  if (i2 == 0) return 0;
  const double nn = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
  double off = 0;
  for (int i = 1; i < n; ++i) {
    const double w[3] = {pts[i][0] - pts[0][0], pts[i][1] - pts[0][1], pts[i][2] - pts[0][2]};
    off = fmax(off, fabs(w[0] * nrm[0] + w[1] * nrm[1] + w[2] * nrm[2]) / nn);
  }
  if (off <= 1e-9 * span) return 0;
  return n;
}

// pass 0: counts[i] = corners of cut cell cells[i] (0 if none, -1 if too
// many); pass 1: writes them at point offset[i]
__global__ void cut_cell_kernel(BuildArgs a, const int64_t* cells, long long n, int pass, int32_t* counts,
                                const int64_t* offset, double* out, int32_t* err) {
  double pts[kMaxPoints][3];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int m = cut_points(a, cells[i], pts);
    if (pass == 0) {
      counts[i] = m < 0 ? 0 : m;
      if (m < 0) atomicExch(err, 1);
      continue;
    }
    // the write pass recomputes the corners; it writes no more than the
    // count pass gave this cell, and flags any difference
    if (m != (m < 0 ? -1 : counts[i])) atomicExch(err, 3);
    const int w = min(m, counts[i]);
    if (w <= 0) continue;
    double* o = out + 3 * offset[i];
    for (int k = 0; k < w; ++k)
      for (int d = 0; d < 3; ++d) o[3 * k + d] = pts[k][d];
  }
}

// Tetrahedra of one convex polytope (corners p[0..n)) in the cell [lo, hi]:
// pyramids from corner 0 over every facet that does not contain it, each
// facet fanned from its first corner by angle.  Writes local index quads to
// out (if not null) and returns their count, or -1 past cap.
__device__ int fan_tets(const BuildArgs& a, const double (*p)[3], int n, const double lo[3], const double hi[3],
                        int32_t* out, int cap) {
  const double tol = a.tol;
  const double span = fmax(hi[0] - lo[0], fmax(hi[1] - lo[1], hi[2] - lo[2]));
  const double vol_eps = 1e-12 * span * span * span;
  int nt = 0;
  int mem[kMaxPoints];
  double ang[kMaxPoints];
  const int np = 6 + a.np;
  for (int f = 0; f < np; ++f) {
    double nrm[3], off;  // plane n·x + off = 0
    if (f < 6) {
      const int ax = f >> 1;
      nrm[0] = nrm[1] = nrm[2] = 0;
      nrm[ax] = 1;
      off = -((f & 1) ? hi[ax] : lo[ax]);
    } else {
      const double* pl = a.planes + 4 * (f - 6);
      nrm[0] = pl[0];
      nrm[1] = pl[1];
      nrm[2] = pl[2];
      off = pl[3];
      // a polyhedron plane that is one of the cell's own planes is that facet already
      bool dup = false;
      for (int ax = 0; ax < 3 && !dup; ++ax) {
        if (fabs(fabs(nrm[ax]) - 1.0) > 1e-12) continue;
        const double x = -off / nrm[ax];
        dup = fabs(x - lo[ax]) <= tol || fabs(x - hi[ax]) <= tol;
      }
      if (dup) continue;
    }
    int k = 0;
    bool has0 = false;
    for (int i = 0; i < n; ++i)
      if (fabs(nrm[0] * p[i][0] + nrm[1] * p[i][1] + nrm[2] * p[i][2] + off) <= tol) {
        if (i == 0) has0 = true;
        mem[k++] = i;
      }
    if (has0 || k < 3) continue;
    // order the facet's corners by angle about their centroid
    double c[3] = {0, 0, 0};
    for (int i = 0; i < k; ++i)
      for (int d = 0; d < 3; ++d) c[d] += p[mem[i]][d];
    for (int d = 0; d < 3; ++d) c[d] /= k;
    double u[3] = {p[mem[0]][0] - c[0], p[mem[0]][1] - c[1], p[mem[0]][2] - c[2]};
    const double un = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    if (!(un > 0)) continue;
    for (int d = 0; d < 3; ++d) u[d] /= un;
    const double w[3] = {nrm[1] * u[2] - nrm[2] * u[1], nrm[2] * u[0] - nrm[0] * u[2], nrm[0] * u[1] - nrm[1] * u[0]};
    for (int i = 0; i < k; ++i) {
      const double r[3] = {p[mem[i]][0] - c[0], p[mem[i]][1] - c[1], p[mem[i]][2] - c[2]};
      ang[i] = atan2(r[0] * w[0] + r[1] * w[1] + r[2] * w[2], r[0] * u[0] + r[1] * u[1] + r[2] * u[2]);
    }
    for (int i = 1; i < k; ++i) {  // insertion sort by angle
      const double av = ang[i];
      const int mv = mem[i];
      int j = i - 1;
      while (j >= 0 && ang[j] > av) {
        ang[j + 1] = ang[j];
        mem[j + 1] = mem[j];
        --j;
      }
      ang[j + 1] = av;
      mem[j + 1] = mv;
    }
    for (int i = 1; i + 1 < k; ++i) {
      const double* q0 = p[0];
      const double* q1 = p[mem[0]];
      const double* q2 = p[mem[i]];
      const double* q3 = p[mem[i + 1]];
      const double e1[3] = {q1[0] - q0[0], q1[1] - q0[1], q1[2] - q0[2]};
      const double e2[3] = {q2[0] - q0[0], q2[1] - q0[1], q2[2] - q0[2]};
      const double e3[3] = {q3[0] - q0[0], q3[1] - q0[1], q3[2] - q0[2]};
      const double vol = e1[0] * (e2[1] * e3[2] - e2[2] * e3[1]) - e1[1] * (e2[0] * e3[2] - e2[2] * e3[0]) +
                         e1[2] * (e2[0] * e3[1] - e2[1] * e3[0]);
      if (fabs(vol) <= vol_eps) continue;
      if (nt == cap) return -1;
      if (out) {
        out[4 * nt] = 0;
        out[4 * nt + 1] = mem[0];
        out[4 * nt + 2] = mem[i];
        out[4 * nt + 3] = mem[i + 1];
      }
      ++nt;
    }
  }
  return nt;
}

// pass 0: counts[i] = tetrahedra of polytope i; pass 1: writes them at
// tet offset[i]
__global__ void fan_kernel(BuildArgs a, const int64_t* cells, const int64_t* point_offset, const double* points,
                           long long n, int pass, int32_t* counts, const int64_t* offset, int32_t* out,
                           int32_t* err) {
  double p[kMaxPoints][3];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(point_offset[i + 1] - point_offset[i]);
    for (int k = 0; k < m; ++k)
      for (int d = 0; d < 3; ++d) p[k][d] = points[3 * (point_offset[i] + k) + d];
    double lo[3], hi[3];
    cell_box(a, cells[i], lo, hi);
    // the write pass writes no more than the count pass gave this polytope
    const int t = pass == 1 ? fan_tets(a, p, m, lo, hi, out + 4 * offset[i], counts[i])
                            : fan_tets(a, p, m, lo, hi, nullptr, kMaxTets);
    if (pass == 0) {
      if (t < 0) atomicExch(err, 2);
      counts[i] = t < 0 ? 0 : t;
    } else if (t != counts[i]) {
      atomicExch(err, 3);
    }
  }
}

struct DevMem {
  std::vector<void*> ptrs;
  ~DevMem() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) ptrs.push_back(q);
    *p = static_cast<T*>(q);
    return e;
  }
};

template <typename T>
cudaError_t upload(DevMem& m, const T* src, size_t count, T** dst) {
  cudaError_t e = m.alloc(dst, count);
  if (e == cudaSuccess && count) e = cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice);
  return e;
}

unsigned grid_for(long long n) {
  long long b = (n + 127) / 128;
  return (unsigned)std::max<long long>(1, std::min<long long>(b, 65536));
}

}  // namespace

#define BUILD_CUDA(call)                                 \
  do {                                                   \
    if ((call) != cudaSuccess) {                         \
      cudaGetLastError();                                \
      brx_trellis_cells_free(out);                       \
      return BRX_ERR_CUDA;                               \
    }                                                    \
  } while (0)

extern "C" {

void brx_trellis_cells_free(brx_trellis_cells* out) {
  if (!out) return;
  std::free(out->node_type);
  std::free(out->poly_node);
  std::free(out->point_offset);
  std::free(out->points);
  std::free(out->tet_offset);
  std::free(out->tets);
  std::memset(out, 0, sizeof *out);
}

brx_status brx_trellis_cells_build(const brx_trellis_in* in, int32_t device, brx_trellis_cells* out) {
  if (!in || !out) return BRX_ERR_INVALID_ARGUMENT;
  std::memset(out, 0, sizeof *out);
  if (in->n_planes < 4 || in->n_planes > kMaxPlanes || in->n_vertices < 4 || in->n_edges < 6 || !in->planes ||
      !in->vertices || !in->edges || !(in->tol >= 0))
    return in->n_planes > kMaxPlanes ? BRX_ERR_UNSUPPORTED : BRX_ERR_INVALID_ARGUMENT;
  for (int d = 0; d < 3; ++d) {
    if (in->n_knots[d] < 2 || !in->knots[d]) return BRX_ERR_INVALID_ARGUMENT;
    for (int i = 1; i < in->n_knots[d]; ++i)
      if (!(in->knots[d][i] > in->knots[d][i - 1])) return BRX_ERR_INVALID_ARGUMENT;
  }
  for (int e = 0; e < 2 * in->n_edges; ++e)
    if (in->edges[e] < 0 || in->edges[e] >= in->n_vertices) return BRX_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return BRX_ERR_CUDA;
  const long long nx = in->n_knots[0] - 1, ny = in->n_knots[1] - 1, nz = in->n_knots[2] - 1;
  const long long n_cells = nx * ny * nz;
  if (n_cells > (1LL << 31) - 1) return BRX_ERR_UNSUPPORTED;
  DevMem m;
  BuildArgs a{};
  for (int d = 0; d < 3; ++d) {
    double* k = nullptr;
    BUILD_CUDA(upload(m, in->knots[d], (size_t)in->n_knots[d], &k));
    a.kn[d] = k;
    a.nk[d] = in->n_knots[d];
  }
  double *verts = nullptr, *planes = nullptr;
  int32_t* edges = nullptr;
  BUILD_CUDA(upload(m, in->vertices, 3 * (size_t)in->n_vertices, &verts));
  BUILD_CUDA(upload(m, in->planes, 4 * (size_t)in->n_planes, &planes));
  BUILD_CUDA(upload(m, in->edges, 2 * (size_t)in->n_edges, &edges));
  a.verts = verts;
  a.planes = planes;
  a.edges = edges;
  a.nv = in->n_vertices;
  a.np = in->n_planes;
  a.ne = in->n_edges;
  a.tol = in->tol;
  a.always_triangulate = in->always_triangulate;
  int32_t *d_type = nullptr, *d_err = nullptr;
  BUILD_CUDA(m.alloc(&d_type, (size_t)n_cells));
  BUILD_CUDA(m.alloc(&d_err, 1));
  BUILD_CUDA(cudaMemset(d_err, 0, sizeof(int32_t)));
  classify_kernel<<<grid_for(n_cells), 128>>>(a, n_cells, d_type);
  BUILD_CUDA(cudaGetLastError());
  out->n_nodes = n_cells;
  out->node_type = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (size_t)n_cells));
  if (!out->node_type) return BRX_ERR_OUT_OF_MEMORY;
  BUILD_CUDA(cudaMemcpy(out->node_type, d_type, sizeof(int32_t) * (size_t)n_cells, cudaMemcpyDeviceToHost));
  std::vector<int64_t> cand;
  for (long long c = 0; c < n_cells; ++c)
    if (out->node_type[c] == 3) cand.push_back(c);
  const long long nc = (long long)cand.size();
  // corners of every cut cell: count, scan, write
  int64_t *d_cand = nullptr, *d_poff = nullptr;
  int32_t* d_cnt = nullptr;
  BUILD_CUDA(upload(m, cand.data(), cand.size(), &d_cand));
  BUILD_CUDA(m.alloc(&d_cnt, (size_t)nc));
  if (nc) cut_cell_kernel<<<grid_for(nc), 128>>>(a, d_cand, nc, 0, d_cnt, nullptr, nullptr, d_err);
  BUILD_CUDA(cudaGetLastError());
  std::vector<int32_t> cnt((size_t)nc);
  BUILD_CUDA(cudaMemcpy(cnt.data(), d_cnt, sizeof(int32_t) * cnt.size(), cudaMemcpyDeviceToHost));
  int32_t err = 0;
  BUILD_CUDA(cudaMemcpy(&err, d_err, sizeof err, cudaMemcpyDeviceToHost));
  if (err) {
    brx_trellis_cells_free(out);
    return BRX_ERR_UNSUPPORTED;
  }
  std::vector<int64_t> poff((size_t)nc + 1, 0);
  for (long long i = 0; i < nc; ++i) poff[i + 1] = poff[i] + cnt[i];
  double* d_pts = nullptr;
  BUILD_CUDA(upload(m, poff.data(), poff.size(), &d_poff));
  BUILD_CUDA(m.alloc(&d_pts, 3 * (size_t)poff[nc]));
  if (nc) cut_cell_kernel<<<grid_for(nc), 128>>>(a, d_cand, nc, 1, d_cnt, d_poff, d_pts, d_err);
  BUILD_CUDA(cudaGetLastError());
  BUILD_CUDA(cudaMemcpy(&err, d_err, sizeof err, cudaMemcpyDeviceToHost));
  if (err) {
    brx_trellis_cells_free(out);
    return BRX_ERR_IMPOSSIBLE;
  }
  // tetrahedra of the cells with corners
  std::vector<int64_t> cells, coff(1, 0);
  std::vector<int64_t> remap;  // index into cand of each kept cell
  for (long long i = 0; i < nc; ++i)
    if (cnt[i] > 0) {
      cells.push_back(cand[i]);
      coff.push_back(coff.back() + cnt[i]);
      remap.push_back(i);
    }
  const long long nk = (long long)cells.size();
  std::vector<double> pts(3 * (size_t)poff[nc]);
  BUILD_CUDA(cudaMemcpy(pts.data(), d_pts, sizeof(double) * pts.size(), cudaMemcpyDeviceToHost));
  std::vector<double> kpts(3 * (size_t)coff.back());
  for (long long i = 0; i < nk; ++i)
    std::memcpy(&kpts[3 * coff[i]], &pts[3 * poff[remap[i]]], sizeof(double) * 3 * (size_t)(coff[i + 1] - coff[i]));
  int64_t *d_cells = nullptr, *d_coff = nullptr, *d_toff = nullptr;
  double* d_kpts = nullptr;
  int32_t *d_tcnt = nullptr, *d_tets = nullptr;
  BUILD_CUDA(upload(m, cells.data(), cells.size(), &d_cells));
  BUILD_CUDA(upload(m, coff.data(), coff.size(), &d_coff));
  BUILD_CUDA(upload(m, kpts.data(), kpts.size(), &d_kpts));
  BUILD_CUDA(m.alloc(&d_tcnt, (size_t)nk));
  if (nk) fan_kernel<<<grid_for(nk), 128>>>(a, d_cells, d_coff, d_kpts, nk, 0, d_tcnt, nullptr, nullptr, d_err);
  BUILD_CUDA(cudaGetLastError());
  std::vector<int32_t> tcnt((size_t)nk);
  BUILD_CUDA(cudaMemcpy(tcnt.data(), d_tcnt, sizeof(int32_t) * tcnt.size(), cudaMemcpyDeviceToHost));
  BUILD_CUDA(cudaMemcpy(&err, d_err, sizeof err, cudaMemcpyDeviceToHost));
  if (err) {
    brx_trellis_cells_free(out);
    return BRX_ERR_UNSUPPORTED;
  }
  std::vector<int64_t> toff((size_t)nk + 1, 0);
  for (long long i = 0; i < nk; ++i) toff[i + 1] = toff[i] + tcnt[i];
  BUILD_CUDA(upload(m, toff.data(), toff.size(), &d_toff));
  BUILD_CUDA(m.alloc(&d_tets, 4 * (size_t)toff[nk]));
  if (nk) fan_kernel<<<grid_for(nk), 128>>>(a, d_cells, d_coff, d_kpts, nk, 1, d_tcnt, d_toff, d_tets, d_err);
  BUILD_CUDA(cudaGetLastError());
  std::vector<int32_t> tets(4 * (size_t)toff[nk]);
  BUILD_CUDA(cudaMemcpy(tets.data(), d_tets, sizeof(int32_t) * tets.size(), cudaMemcpyDeviceToHost));
  BUILD_CUDA(cudaMemcpy(&err, d_err, sizeof err, cudaMemcpyDeviceToHost));
  if (err) {
    brx_trellis_cells_free(out);
    return BRX_ERR_IMPOSSIBLE;
  }
  // POLY nodes: cells whose polytope has tetrahedra; every other cut cell is null
  long long n_poly = 0;
  for (long long i = 0; i < nk; ++i) n_poly += tcnt[i] > 0;
  for (long long c = 0; c < n_cells; ++c)
    if (out->node_type[c] == 3) out->node_type[c] = BRX_NODE_NULL;
  out->n_poly = n_poly;
  out->poly_node = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (size_t)(n_poly ? n_poly : 1)));
  out->point_offset = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * (size_t)(n_poly + 1)));
  out->tet_offset = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * (size_t)(n_poly + 1)));
  long long np_total = 0, nt_total = 0;
  for (long long i = 0; i < nk; ++i)
    if (tcnt[i] > 0) {
      np_total += coff[i + 1] - coff[i];
      nt_total += tcnt[i];
    }
  out->points = static_cast<double*>(std::malloc(sizeof(double) * 3 * (size_t)(np_total ? np_total : 1)));
  out->tets = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * 4 * (size_t)(nt_total ? nt_total : 1)));
  if (!out->poly_node || !out->point_offset || !out->tet_offset || !out->points || !out->tets) {
    brx_trellis_cells_free(out);
    return BRX_ERR_OUT_OF_MEMORY;
  }
  long long k = 0;
  out->point_offset[0] = 0;
  out->tet_offset[0] = 0;
  for (long long i = 0; i < nk; ++i) {
    if (tcnt[i] == 0) continue;
    out->poly_node[k] = (int32_t)cells[i];
    out->node_type[cells[i]] = BRX_NODE_POLY;
    const long long pc = coff[i + 1] - coff[i];
    std::memcpy(out->points + 3 * out->point_offset[k], &kpts[3 * coff[i]], sizeof(double) * 3 * (size_t)pc);
    std::memcpy(out->tets + 4 * out->tet_offset[k], &tets[4 * toff[i]], sizeof(int32_t) * 4 * (size_t)tcnt[i]);
    out->point_offset[k + 1] = out->point_offset[k] + pc;
    out->tet_offset[k + 1] = out->tet_offset[k] + tcnt[i];
    ++k;
  }
  return BRX_OK;
}

}  // extern "C"
