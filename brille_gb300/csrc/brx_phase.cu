// Antiphase table of FP64 complex eigenvectors.
//
// The gather multiplies every vertex row of a group by its antiphase against
// the group's pivot vertex before weighting it (Interpolator::
// interpolate_at_mix, src/interpolator_at.tpp:92-127, with utils::antiphase,
// src/utilities.tpp:567-578).  The factor depends on the ordered vertex pair
// and the mode only, not on q.  For FP64 vertex data it is therefore formed
// once here, whenever the data or the permutation table change, for every
// ordered pair of distinct vertices that share a cube node or a tetrahedron
// (the pairs a group can hold), one complex factor per mode, with the
// arithmetic of the gather's own loop.  GB300 issues FP64 at 1/64 of its
// FP32 rate; per group the table saves 8 FP64 operations per staged element,
// which dominated the FP64 gather when few q share a group (queries that
// stage host outputs in small chunks).
//
// Layout: sorted keys i·N + j (N vertices), and factors [key][mode] as
// (re, im) doubles: 16 bytes per key and mode (3.7 GB for 4.8M keys of 48
// modes).  A table that cannot be allocated is simply not built: the gather
// then forms the factors per group, as it does for FP32 and BF16 storage.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include "brx_handle.h"

using namespace brx_detail;

namespace {

// every ordered pair (a, b), a ≠ b, of the 8 corners of each cube node and
// the 4 corners of each tetrahedron, as the key v_a·N + v_b
__global__ void pair_keys_kernel(const int32_t* cube_vertices, long long n_cube, const int32_t* tet_vertices,
                                 long long n_tets, long long nv, long long* out) {
  const long long total = 56 * n_cube + 12 * n_tets;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    long long vi, vj;
    if (t < 56 * n_cube) {
      const long long c = t / 56;
      const int r = (int)(t - c * 56), a = r / 7, bb = r % 7, b = bb + (bb >= a ? 1 : 0);
      vi = cube_vertices[8 * c + a];
      vj = cube_vertices[8 * c + b];
    } else {
      const long long u = t - 56 * n_cube, c = u / 12;
      const int r = (int)(u - c * 12), a = r / 3, bb = r % 3, b = bb + (bb >= a ? 1 : 0);
      vi = tet_vertices[4 * c + a];
      vj = tet_vertices[4 * c + b];
    }
    out[t] = vi * nv + vj;
  }
}

}  // namespace

namespace brx_detail {

brx_status build_phase_table(brx_handle* h) {
  h->ph_valid = false;
  h->n_ph_keys = 0;
  const Interp& d = h->vecs;
  if (!h->filled || !d.present || !d.cplx || d.store != ST_F64 || (d.el[1] < 3 && d.el[2] < 9)) return BRX_OK;
  const long long nc = 56LL * h->g.n_cube + 12LL * h->g.n_tets;
  const long long nv = h->host_geom.n_vertices;
  if (nc == 0 || nv < 2) return BRX_OK;
  BRX_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t cs = h->sc[0].stream;
  struct Transient {
    DevBuf a, b, tmp, num;
    ~Transient() {
      a.release();
      b.release();
      tmp.release();
      num.release();
    }
  } tr;
  // no room for the table is not an error: the gather forms factors per group
  auto skip = [&]() {
    cudaGetLastError();
    h->ph_keys.release();
    h->ph_table.release();
    return BRX_OK;
  };
  if (tr.a.ensure(sizeof(long long) * nc) != cudaSuccess || tr.b.ensure(sizeof(long long) * nc) != cudaSuccess ||
      tr.num.ensure(sizeof(long long)) != cudaSuccess)
    return skip();
  long long* cand = static_cast<long long*>(tr.a.p);
  long long* sorted = static_cast<long long*>(tr.b.p);
  long long* num = static_cast<long long*>(tr.num.p);
  {
    long long blocks = (nc + 255) / 256;
    if (blocks > 65536) blocks = 65536;
    pair_keys_kernel<<<(unsigned)blocks, 256, 0, cs>>>(h->g.cube_vertices, h->g.n_cube, h->g.tet_vertices,
                                                       h->g.n_tets, nv, cand);
    BRX_CUDA(h, cudaGetLastError());
  }
  int end_bit = 1;
  while (end_bit < 63 && ((long long)1 << end_bit) <= nv * nv) ++end_bit;
  size_t tb_sort = 0, tb_uniq = 0;
  BRX_CUDA(h, cub::DeviceRadixSort::SortKeys(nullptr, tb_sort, cand, sorted, (int64_t)nc, 0, end_bit, cs));
  BRX_CUDA(h, cub::DeviceSelect::Unique(nullptr, tb_uniq, sorted, cand, num, (int64_t)nc, cs));
  if (tr.tmp.ensure(std::max<size_t>(std::max(tb_sort, tb_uniq), 16)) != cudaSuccess) return skip();
  BRX_CUDA(h, cub::DeviceRadixSort::SortKeys(tr.tmp.p, tb_sort, cand, sorted, (int64_t)nc, 0, end_bit, cs));
  BRX_CUDA(h, cub::DeviceSelect::Unique(tr.tmp.p, tb_uniq, sorted, cand, num, (int64_t)nc, cs));
  long long nk = 0;
  BRX_CUDA(h, cudaMemcpyAsync(&nk, num, sizeof nk, cudaMemcpyDeviceToHost, cs));
  BRX_CUDA(h, cudaStreamSynchronize(cs));
  if (nk <= 0) return BRX_OK;
  if (h->ph_keys.ensure(sizeof(long long) * nk) != cudaSuccess ||
      h->ph_table.ensure(sizeof(double2) * (size_t)nk * d.B) != cudaSuccess)
    return skip();
  BRX_CUDA(h, cudaMemcpyAsync(h->ph_keys.p, cand, sizeof(long long) * nk, cudaMemcpyDeviceToDevice, cs));
  brx::GatherParams p{};
  p.data = d.data.p;
  p.B = d.B;
  p.s = span(d);
  p.n_keys = h->n_keys;
  p.keys = static_cast<const long long*>(h->perm_keys.p);
  p.perm_ids = static_cast<const int32_t*>(h->perm_ids.p);
  p.n_perms = h->n_perms;
  p.perms = static_cast<const int32_t*>(h->perms.p);
  p.n_vertices = nv;
  brx::launch_phase_table(p, static_cast<const long long*>(h->ph_keys.p), nk,
                          static_cast<double2*>(h->ph_table.p), cs);
  h->launches += 3;
  BRX_CUDA(h, cudaGetLastError());
  BRX_CUDA(h, cudaStreamSynchronize(cs));
  h->n_ph_keys = nk;
  h->ph_valid = true;
  return BRX_OK;
}

}  // namespace brx_detail
