// C ABI of the GB300 query path (include/brx.h).
//
// A brx_handle owns the device copy of one trellis geometry, its vertex data
// and the per-chunk scratch of the query pipeline:
//
//   locate (FP64 move + wedge + node/tetrahedron search, one thread per q)
//   -> counting sort of q by trellis node
//   -> gather + rotate for the values, then for the vectors
//
// Large queries run in chunks.  With host buffers, chunks alternate between
// two streams and two scratch sets so that copies overlap compute.  Errors
// are collected per q on the device and turned into the reference's
// messages on the host; no exception crosses the ABI.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/brx.h"
#include "brx_kernels.h"
#include "brx_handle.h"

using namespace brx_detail;

namespace brx_detail {

brx_status fail(brx_handle* h, brx_status st, const std::string& msg) {
  if (h) h->message = msg;
  return st;
}

brx_status cuda_fail(brx_handle* h, cudaError_t e, const char* where) {
  std::string m = std::string("CUDA error in ") + where + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return fail(h, BRX_ERR_OUT_OF_MEMORY, m);
  return fail(h, BRX_ERR_CUDA, m);
}


template <typename T>
brx_status upload(brx_handle* h, const T* src, size_t count, const T** dst) {
  h->tables.emplace_back();
  DevBuf& b = h->tables.back();
  size_t bytes = sizeof(T) * (count ? count : 1);
  BRX_CUDA(h, b.ensure(bytes));
  if (count) BRX_CUDA(h, cudaMemcpy(b.p, src, sizeof(T) * count, cudaMemcpyHostToDevice));
  *dst = static_cast<const T*>(b.p);
  return BRX_OK;
}

// C = A·B for 3×3, accumulated from zero in k order (src/utilities.tpp:48-55)
void mm3(double* C, const double* A, const double* B) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += A[3 * i + k] * B[3 * k + j];
      C[3 * i + j] = s;
    }
}

bool host_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged;
}

// Device address of page-locked host memory, else null.
void* mapped_ptr(void* p) {
  cudaPointerAttributes a{};
  if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int span(const Interp& d) { return d.el[0] + d.el[1] + d.el[2]; }

// whether the gather of d takes the group-ordered kernel (launch_t in
// brx_gather.cu): anything but scalars without a phase factor
bool uses_groups(const Interp& d, bool phase) { return d.el[1] / 3 != 0 || d.el[2] / 9 != 0 || phase; }

// rotation support, mirroring Interpolator::rotate_in_place (src/interpolator.hpp:387-428)
brx_status rotation_mode(const Interp& d, int* mode, std::string* msg) {
  *mode = ROT_NONE;
  const int nvec = d.el[1] / 3, nmat = d.el[2] / 9;
  const char* combo = "LengthUnit, RotatesLike combination not implemented";
  switch (d.length_unit) {
    case BRX_LU_REAL_LATTICE:
      if (d.rotates_like == BRX_ROT_VECTOR) *mode = ROT_REAL;
      else if (d.rotates_like == BRX_ROT_PSEUDOVECTOR) *mode = ROT_AXIAL;
      else if (d.rotates_like == BRX_ROT_GAMMA) *mode = ROT_GAMMA;
      else { *msg = "Impossible RotatesLike value!"; return BRX_ERR_UNSUPPORTED; }
      break;
    case BRX_LU_RECIPROCAL_LATTICE:
      if (d.rotates_like != BRX_ROT_VECTOR) { *msg = combo; return BRX_ERR_UNSUPPORTED; }
      *mode = ROT_RECIP;
      break;
    case BRX_LU_ANGSTROM:
      if (d.rotates_like != BRX_ROT_GAMMA) { *msg = combo; return BRX_ERR_UNSUPPORTED; }
      *mode = ROT_GAMMA;
      break;
    default:
      *msg = combo;
      return BRX_ERR_UNSUPPORTED;
  }
  if (*mode == ROT_GAMMA) {
    if (!d.cplx) { *msg = "RotatesLike == Gamma requires complex valued data!"; return BRX_ERR_UNSUPPORTED; }
    const int Nmat = (int)std::sqrt((double)nmat) / 3;
    if (nmat > 0) {
      if (nmat == 9 * Nmat * Nmat) {
        *msg = "Gamma rotation of 3x3 tensors is not defined for this element count";
        return BRX_ERR_UNSUPPORTED;
      }
      *mode = ROT_NONE;  // the reference rotates nothing in this case
    }
  }
  if (nvec == 0 && nmat == 0) *mode = ROT_NONE;
  return BRX_OK;
}

brx_status ensure_scratch(brx_handle* h, long long chunk) {
  if (chunk <= h->scratch_q) return BRX_OK;
  const size_t n = (size_t)chunk;
  const size_t parts[11] = {24 * n, 64 * n, 32 * n, 12 * n, 8 * n, 8 * n, 4 * n, 32 * n, 4 * n, 4 * n, 4 * n};
  size_t rec = 0;
  for (size_t b : parts) rec += (b + 255) & ~size_t(255);
  for (auto& s : h->sc) {
    BRX_CUDA(h, s.rec.ensure(rec));
    char* p = static_cast<char*>(s.rec.p);
    auto take = [&](size_t bytes) {
      char* at = p;
      p += (bytes + 255) & ~size_t(255);
      return at;
    };
    s.r.q_ir = reinterpret_cast<double*>(take(24 * n));
    s.r.w = reinterpret_cast<double*>(take(64 * n));
    s.r.w32 = reinterpret_cast<float*>(take(32 * n));
    s.r.tau = reinterpret_cast<int32_t*>(take(12 * n));
    s.r.rot = reinterpret_cast<int32_t*>(take(8 * n));
    s.r.node = reinterpret_cast<int32_t*>(take(8 * n));
    s.r.nw = reinterpret_cast<int32_t*>(take(4 * n));
    s.r.vidx = reinterpret_cast<int32_t*>(take(32 * n));
    s.r.status = reinterpret_cast<int32_t*>(take(4 * n));
    s.order = reinterpret_cast<int32_t*>(take(4 * n));
    s.r.key = reinterpret_cast<int32_t*>(take(4 * n));
    BRX_CUDA(h, s.sortbuf.ensure(sizeof(int32_t) * group_scratch_ints(n_group_keys(h->g.n_cube, h->g.n_tets))));
    s.sort_scratch = static_cast<int32_t*>(s.sortbuf.p);
    BRX_CUDA(h, s.groupbuf.ensure(sizeof(GroupDesc) * n + 256));
    s.groups = static_cast<GroupDesc*>(s.groupbuf.p);
    s.n_groups = reinterpret_cast<int32_t*>(static_cast<char*>(s.groupbuf.p) + sizeof(GroupDesc) * n + 64);
    s.counters = s.n_groups + 16;
  }
  h->scratch_q = chunk;
  return BRX_OK;
}

GatherParams gather_params(brx_handle* h, const Interp& d, const Scratch& s, long long n, int rot_mode, bool phase,
                           int which) {
  GatherParams p{};
  p.nw = s.r.nw;
  p.vidx = s.r.vidx;
  p.w = s.r.w;
  p.w32 = s.r.w32;
  p.rot = s.r.rot;
  p.q_ir = s.r.q_ir;
  p.status = s.r.status;
  p.order = s.order;
  p.groups = s.groups;
  p.n_groups = s.n_groups;
  p.counter = s.counters + which;
  p.n = n;
  p.n_cube = h->g.n_cube;
  p.cube_vertices = h->g.cube_vertices;
  p.rank_cube = h->rank_cube;
  p.tet_vertices = h->g.tet_vertices;
  p.data = d.data.p;
  p.B = d.B;
  p.s = span(d);
  p.nsc = d.el[0];
  p.nvec = d.el[1] / 3;
  p.nmat = d.el[2] / 9;
  p.rot_mode = rot_mode;
  p.gamma_cart = d.length_unit == BRX_LU_ANGSTROM;
  p.phase_allowed = phase ? 1 : 0;
  p.n_keys = h->n_keys;
  p.keys = static_cast<const long long*>(h->perm_keys.p);
  p.perm_ids = static_cast<const int32_t*>(h->perm_ids.p);
  p.n_perms = h->n_perms;
  p.perms = static_cast<const int32_t*>(h->perms.p);
  p.n_vertices = h->host_geom.n_vertices;
  // the antiphase table holds the eigenvectors' factors (FP64 complex data)
  if (phase && which == 1 && h->ph_valid && d.store == ST_F64 && d.cplx) {
    p.n_ph_keys = h->n_ph_keys;
    p.ph_keys = static_cast<const long long*>(h->ph_keys.p);
    p.ph_table = static_cast<const double2*>(h->ph_table.p);
  }
  p.ops = h->g.ops;
  p.rot_cart = h->g.rot_cart;
  p.n_ops = h->g.n_ops;
  p.gamma_F0 = h->g.gamma_F0;
  p.gamma_vidx = h->g.gamma_vidx;
  p.gamma_vectors = h->g.gamma_vectors;
  p.qmax = h->group_q;
  p.qsplit = h->qsplit;
  p.err = h->err;
  p.variant = h->gather_variant;
  p.stall = h->test_stall ? 1 : 0;
  return p;
}

size_t smem_budget(brx_handle* h, int which) {
  size_t b = h->gather_budget[which];
  if (h->smem_optin && b > h->smem_optin) b = h->smem_optin;
  return b;
}

size_t out_elem_bytes(const Interp& d, bool f32) {
  size_t e = f32 ? 4 : 8;
  return e * (d.cplx ? 2 : 1);
}

// Read the device error word and build the reference's message.
brx_status collect_errors(brx_handle* h, int ir, const double* Q, long long n, bool q_host) {
  ErrorWord ew = *h->err_host;
  if (!ew.flags) return BRX_OK;
  auto has = [&](int st) { return (ew.flags >> st) & 1; };
  double qv[3] = {0, 0, 0};
  long long i = ew.first_bad;
  if (i >= 0 && i < n) {
    if (q_host) std::memcpy(qv, Q + 3 * i, sizeof qv);
    else cudaMemcpy(qv, Q + 3 * i, sizeof qv, cudaMemcpyDeviceToHost);
  }
  char buf[512];
  if (has(BRX_ERR_MOVE_FAILED)) {
    std::snprintf(buf, sizeof buf, "Not all points inside Brillouin zone (%d of %lld still outside; first Q = [%.17g %.17g %.17g])",
                  ew.count, n, qv[0], qv[1], qv[2]);
    return fail(h, BRX_ERR_MOVE_FAILED, buf);
  }
  if (has(BRX_ERR_OUTSIDE_IR)) {
    std::snprintf(buf, sizeof buf, "Q = [%.17g %.17g %.17g] is outside of the irreducible BrillouinZone", qv[0], qv[1], qv[2]);
    return fail(h, BRX_ERR_OUTSIDE_IR, buf);
  }
  if (has(BRX_ERR_IMPOSSIBLE)) return fail(h, BRX_ERR_IMPOSSIBLE, "This shouldn't be possible");
  if (has(BRX_ERR_NULL_NODE)) {
    std::snprintf(buf, sizeof buf, "Attempting to access null node for point Q = [%.17g %.17g %.17g]", qv[0], qv[1], qv[2]);
    return fail(h, BRX_ERR_NULL_NODE, buf);
  }
  if (has(BRX_ERR_TIMEOUT))
    return fail(h, BRX_ERR_TIMEOUT, "a bounded device-side wait ran out; results are incomplete");
  if (has(BRX_ERR_NOT_FOUND)) {
    std::snprintf(buf, sizeof buf, "interpolate_at failed to find %d point%s", ew.count, ew.count > 1 ? "s." : ".");
    return fail(h, BRX_ERR_NOT_FOUND, buf);
  }
  (void)ir;
  return fail(h, BRX_ERR_CUDA, "unknown device error");
}

cudaEvent_t next_event(brx_handle* h) {
  if (h->ev_used == h->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    h->ev_pool.push_back(e);
  }
  return h->ev_pool[h->ev_used++];
}

int32_t* next_group_slot(brx_handle* h) {
  if (h->group_used == h->group_counts.size()) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, sizeof(int32_t), cudaHostAllocDefault) != cudaSuccess) return nullptr;
    h->group_counts.push_back(static_cast<int32_t*>(p));
  }
  return h->group_counts[h->group_used++];
}

// accumulate stage durations from the events recorded since the last call
void harvest_events(brx_handle* h) {
  for (size_t i = 0; i < h->group_used; ++i) h->stage_groups += *h->group_counts[i];
  h->group_used = 0;
  for (size_t i = 0; i + 5 < h->ev_used + 1 && i + 4 < h->ev_used; i += 5) {
    for (int k = 0; k < 4; ++k) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, h->ev_pool[i + k], h->ev_pool[i + k + 1]) == cudaSuccess) h->stage_ms[k] += ms;
    }
  }
  h->ev_used = 0;
}

// The device error word is cleared on the device, in stream order: flags and
// count to zero, first_bad to 0x7f7f7f7f7f7f7f7f (above any q index, so the
// locate kernel's atomicMin keeps the smallest failing one).  No host memory
// is written at call time.
brx_status reset_errors(brx_handle* h, cudaStream_t s) {
  static_assert(sizeof(ErrorWord) == 16 && offsetof(ErrorWord, first_bad) == 8, "ErrorWord layout");
  BRX_CUDA(h, cudaMemsetAsync(h->err, 0, 8, s));
  BRX_CUDA(h, cudaMemsetAsync(reinterpret_cast<char*>(h->err) + 8, 0x7f, 8, s));
  return BRX_OK;
}

// The whole query, chunked.  mode: 0 interpolate_at, 1 ir_interpolate_at.
// sf: vecs_out receives the structure factor (float, n × B) instead of the
// vectors (brx_ir_structure_factor).
brx_status run_query(brx_handle* h, int ir, const double* Q, long long n, void* vals_out, void* vecs_out,
                     uint32_t flags, void* user_stream, const brx_locate_out* lout, bool sf = false) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (n < 0 || (n > 0 && !Q)) return fail(h, BRX_ERR_INVALID_ARGUMENT, "Q must be a non-null (n,3) array");
  BRX_CUDA(h, cudaSetDevice(h->device));
  const bool locate_only = lout != nullptr;
  if (!locate_only) {
    if (!h->filled) return fail(h, BRX_ERR_NOT_FILLED, "The interpolation data must be filled before interpolating.");
    if (!vals_out || (h->vecs.present && !vecs_out))
      return fail(h, BRX_ERR_INVALID_ARGUMENT, "output buffers must be provided");
  }
  const bool no_move = flags & BRX_FLAG_NO_MOVE;
  const bool f32 = flags & BRX_FLAG_OUT_F32;
  h->test_stall = (flags & BRX_FLAG_TEST_TIMEOUT) != 0;
  int vmode = ROT_NONE, cmode = ROT_NONE;
  if (ir && !locate_only) {
    std::string msg;
    brx_status st = rotation_mode(h->vals, &vmode, &msg);
    if (st) return fail(h, st, msg);
    if (h->vecs.present) {
      st = rotation_mode(h->vecs, &cmode, &msg);
      if (st) return fail(h, st, msg);
    }
  }
  const int kmode = no_move ? 2 : (ir ? 1 : 0);
  if (sf) {
    const Interp& c = h->vecs;
    if (!c.present || !c.cplx || c.el[0] != 0 || c.el[2] != 0 || c.el[1] / 3 < 1 || c.el[1] / 3 > 32)
      return fail(h, BRX_ERR_UNSUPPORTED, "the structure factor needs complex eigenvectors of 1-32 atoms and no "
                                          "other elements");
    if (c.store == ST_F64) return fail(h, BRX_ERR_UNSUPPORTED, "the structure factor needs FP32 or BF16 storage");
    if (c.length_unit != BRX_LU_ANGSTROM || (ir && cmode != ROT_GAMMA))
      return fail(h, BRX_ERR_UNSUPPORTED, "the structure factor needs Cartesian (Å) Γ-rotating eigenvectors");
    if (h->sf_n != c.el[1] / 3) return fail(h, BRX_ERR_INVALID_ARGUMENT, "brx_set_atoms with one entry per atom first");
  }
  if (n == 0) return BRX_OK;

  const bool q_host = host_ptr(Q);
  bool o_host = locate_only ? host_ptr(lout->status) : host_ptr(vals_out);
  // page-locked host outputs: the kernels may write them directly over the
  // host link (BRX_ZERO_COPY=1) instead of through staged chunks and copies
  if (o_host && !locate_only) {
    const char* zc_env = std::getenv("BRX_ZERO_COPY");
    if (zc_env && zc_env[0] == '1') {
      void* vz = mapped_ptr(vals_out);
      void* cz = h->vecs.present ? mapped_ptr(vecs_out) : nullptr;
      if (vz && (cz || !h->vecs.present)) {
        vals_out = vz;
        vecs_out = cz;
        o_host = false;
      }
    }
  }
  const bool any_host = q_host || o_host;
  // BRX_FLAG_ASYNC with host I/O needs page-locked Q and outputs: their
  // copies then run in stream order like everything else, and the caller
  // reads the outputs after brx_sync (or an event behind the call)
  const bool pinned_io =
      (!q_host || mapped_ptr(const_cast<double*>(Q))) &&
      (!o_host || locate_only || (mapped_ptr(vals_out) && (!h->vecs.present || mapped_ptr(vecs_out))));
  const bool async = (flags & BRX_FLAG_ASYNC) && !locate_only && (!any_host || pinned_io);

  size_t out_q = 0;  // output bytes per q
  if (!locate_only) {
    out_q += (size_t)h->vals.B * span(h->vals) * out_elem_bytes(h->vals, f32);
    if (h->vecs.present) out_q += sf ? (size_t)h->vecs.B * 4 : (size_t)h->vecs.B * span(h->vecs) * out_elem_bytes(h->vecs, f32);
  }
  long long chunk = 1LL << 24;
  // host outputs: chunks of about BRX_HOST_CHUNK_MB (default 512) MB of
  // outputs, alternating between two streams and staging buffers
  const char* chunk_env = std::getenv("BRX_HOST_CHUNK_MB");
  const long long chunk_mb = chunk_env ? std::atoll(chunk_env) : 0;
  const long long host_chunk = (chunk_mb > 0 && chunk_mb <= 65536 ? chunk_mb : 512) << 20;
  if (o_host && out_q) chunk = std::max<long long>(1024, std::min<long long>(chunk, host_chunk / (long long)out_q));
  if (chunk > n) chunk = n;
  const size_t vrow = (size_t)h->vals.B * span(h->vals) * out_elem_bytes(h->vals, f32);
  const size_t crow = !h->vecs.present ? 0
                      : sf ? (size_t)h->vecs.B * 4 : (size_t)h->vecs.B * span(h->vecs) * out_elem_bytes(h->vecs, f32);
  // buffers that must grow are freed and allocated anew: queued work that
  // may still use them finishes first
  if (h->async_pending) {
    bool grow = chunk > h->scratch_q;
    for (int k = 0; k < 2; ++k) {
      if (!locate_only && o_host && (h->sc[k].vbuf.bytes < vrow * (size_t)chunk + 16 ||
                                     (crow && h->sc[k].cbuf.bytes < crow * (size_t)chunk + 16)))
        grow = true;
      if (q_host && h->sc[k].qbuf.bytes < 24 * (size_t)chunk + 16) grow = true;
    }
    if (grow) BRX_CUDA(h, cudaStreamSynchronize(h->async_stream));
  }
  brx_status st = ensure_scratch(h, chunk);
  if (st) return st;

  cudaStream_t us = static_cast<cudaStream_t>(user_stream);
  // host I/O: chunks alternate between the handle's two streams (copies of
  // one chunk overlap the kernels of the next), joined to the caller's
  // stream at both ends
  const int nstreams = any_host ? 2 : 1;
  cudaStream_t main_s = us ? us : h->sc[0].stream;
  if (h->async_pending && !async)
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "asynchronous queries must be synchronised with brx_sync first");
  if (!h->async_pending) {
    // queued asynchronous queries on one stream share one error word until brx_sync
    st = reset_errors(h, main_s);
    if (st) return st;
  }
  if (nstreams == 2) {
    BRX_CUDA(h, cudaEventRecord(h->sc[0].done, main_s));
    for (int k = 0; k < 2; ++k)
      if (h->sc[k].stream != main_s) BRX_CUDA(h, cudaStreamWaitEvent(h->sc[k].stream, h->sc[0].done, 0));
  }
  if (!locate_only && o_host) {
    for (int k = 0; k < nstreams; ++k) {
      BRX_CUDA(h, h->sc[k].vbuf.ensure(vrow * (size_t)chunk + 16));
      if (crow) BRX_CUDA(h, h->sc[k].cbuf.ensure(crow * (size_t)chunk + 16));
    }
  }
  if (q_host)
    for (int k = 0; k < nstreams; ++k) BRX_CUDA(h, h->sc[k].qbuf.ensure(24 * (size_t)chunk + 16));

  long long ci = 0;
  for (long long base = 0; base < n; base += chunk, ++ci) {
    const long long m = std::min(chunk, n - base);
    // host I/O: consecutive chunks, of this call and of the next, take turns
    // on the two streams, so a queued call computes while this one copies.
    // A chunk's kernels start after the previous chunk's kernels (on the
    // other stream) have finished, not beside them: two chunks computing at
    // once finish together, leave the host link idle meanwhile and then
    // copy together, and the steps fall into compute-then-copy lock step.
    const int slot = nstreams == 2 ? (int)((h->chunk_seq + ci) & 1) : 0;
    Scratch& s = h->sc[slot];
    cudaStream_t cs = nstreams == 2 ? s.stream : main_s;
    const double* Qd = Q + 3 * base;
    if (q_host) {
      BRX_CUDA(h, cudaMemcpyAsync(s.qbuf.p, Q + 3 * base, 24 * (size_t)m, cudaMemcpyHostToDevice, cs));
      Qd = static_cast<const double*>(s.qbuf.p);
    }
    if (nstreams == 2) BRX_CUDA(h, cudaStreamWaitEvent(cs, h->sc[slot ^ 1].computed, 0));
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    if (h->profile && !locate_only) {
      for (auto& e : ev) e = next_event(h);
      cudaEventRecord(ev[0], cs);
      h->stage_q += m;
    }
    launch_locate(h->g, Qd, m, base, kmode, s.r, h->err, h->num_sms, cs);
    ++h->launches;
    if (ev[1]) cudaEventRecord(ev[1], cs);
    if (locate_only) {
      if (nstreams == 2) BRX_CUDA(h, cudaEventRecord(s.computed, cs));
      auto cp = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
        if (!dst) return cudaSuccess;
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, cs);
      };
      BRX_CUDA(h, cp(lout->q_ir ? lout->q_ir + 3 * base : nullptr, s.r.q_ir, 24 * (size_t)m));
      BRX_CUDA(h, cp(lout->tau ? lout->tau + 3 * base : nullptr, s.r.tau, 12 * (size_t)m));
      BRX_CUDA(h, cp(lout->rot ? lout->rot + 2 * base : nullptr, s.r.rot, 8 * (size_t)m));
      BRX_CUDA(h, cp(lout->node ? lout->node + 2 * base : nullptr, s.r.node, 8 * (size_t)m));
      BRX_CUDA(h, cp(lout->n_weights ? lout->n_weights + base : nullptr, s.r.nw, 4 * (size_t)m));
      BRX_CUDA(h, cp(lout->vertex ? lout->vertex + 8 * base : nullptr, s.r.vidx, 32 * (size_t)m));
      BRX_CUDA(h, cp(lout->weight ? lout->weight + 8 * base : nullptr, s.r.w, 64 * (size_t)m));
      BRX_CUDA(h, cp(lout->status ? lout->status + base : nullptr, s.r.status, 4 * (size_t)m));
      continue;
    }
    // the group-ordered gather serves vector and matrix data; scalar-only
    // data (eigenvalues) is gathered per q and needs no grouping
    const bool grouped = uses_groups(h->vals, false) || (h->vecs.present && uses_groups(h->vecs, h->vecs.cplx));
    if (grouped)
      h->launches += launch_grouping(s.r.key, m, n_group_keys(h->g.n_cube, h->g.n_tets), h->group_q, s.sort_scratch,
                                     s.order, s.groups, s.n_groups, cs);
    if (ev[2]) cudaEventRecord(ev[2], cs);
    char* vdst = o_host ? static_cast<char*>(s.vbuf.p) : static_cast<char*>(vals_out) + vrow * (size_t)base;
    {
      GatherParams p = gather_params(h, h->vals, s, m, ir ? vmode : ROT_NONE, false, 0);
      p.out = vdst;
      p.MB = gather_pick_modes(p, h->vals.store, h->vals.cplx, smem_budget(h, 0));
      h->launches += launch_gather(p, h->vals.store, h->vals.cplx, f32, h->num_sms, smem_budget(h, 0), cs);
      h->launches += launch_residual(h, s, m, vdst, f32, cs);
    }
    if (ev[3]) cudaEventRecord(ev[3], cs);
    char* cdst = nullptr;
    if (h->vecs.present) {
      cdst = o_host ? static_cast<char*>(s.cbuf.p) : static_cast<char*>(vecs_out) + crow * (size_t)base;
      GatherParams p = gather_params(h, h->vecs, s, m, ir ? cmode : ROT_NONE, h->vecs.cplx, 1);
      p.out = cdst;
      p.MB = gather_pick_modes(p, h->vecs.store, h->vecs.cplx, smem_budget(h, 1));
      if (sf) {
        p.sf_atoms = h->sf_n;
        p.sf_Q = Qd;
        p.sf_atom = static_cast<const double*>(h->sf_atoms.p);
        p.sf_B = static_cast<const double*>(h->sf_B.p);
        const int k = launch_structure_factor(p, h->vecs.store, h->num_sms, smem_budget(h, 1), cs);
        if (k < 0) return fail(h, BRX_ERR_UNSUPPORTED, "the structure-factor gather does not fit this data");
        h->launches += k;
      } else {
        h->launches += launch_gather(p, h->vecs.store, h->vecs.cplx, f32, h->num_sms, smem_budget(h, 1), cs);
      }
    }
    if (ev[4]) {
      cudaEventRecord(ev[4], cs);
      if (!grouped) cudaMemsetAsync(s.n_groups, 0, sizeof(int32_t), cs);
      if (int32_t* slot = next_group_slot(h)) cudaMemcpyAsync(slot, s.n_groups, sizeof(int32_t), cudaMemcpyDeviceToHost, cs);
    }
    BRX_CUDA(h, cudaGetLastError());
    if (nstreams == 2) BRX_CUDA(h, cudaEventRecord(s.computed, cs));
    if (o_host) {
      BRX_CUDA(h, cudaMemcpyAsync(static_cast<char*>(vals_out) + vrow * (size_t)base, vdst, vrow * (size_t)m,
                                  cudaMemcpyDeviceToHost, cs));
      if (cdst)
        BRX_CUDA(h, cudaMemcpyAsync(static_cast<char*>(vecs_out) + crow * (size_t)base, cdst, crow * (size_t)m,
                                    cudaMemcpyDeviceToHost, cs));
    }
  }
  BRX_CUDA(h, cudaGetLastError());
  if (nstreams == 2) h->chunk_seq += ci;
  if (nstreams == 2) {
    for (int k = 0; k < 2; ++k) {
      if (h->sc[k].stream == main_s) continue;
      BRX_CUDA(h, cudaEventRecord(h->sc[k].done, h->sc[k].stream));
      BRX_CUDA(h, cudaStreamWaitEvent(main_s, h->sc[k].done, 0));
    }
  }
  if (async) {
    // the error word is read once, by brx_sync: a small copy queued behind
    // each call would wait in the copy engine behind the next call's output
    // copies, so each call would finish only with the next one
    h->async_pending = true;
    h->async_stream = main_s;
    if (std::find(h->async_streams.begin(), h->async_streams.end(), main_s) == h->async_streams.end())
      h->async_streams.push_back(main_s);
    h->async_ir = ir;
    h->async_Q = Q;
    h->async_n = n;
    h->async_q_host = q_host;
    return BRX_OK;
  }
  BRX_CUDA(h, cudaMemcpyAsync(h->err_host, h->err, sizeof(ErrorWord), cudaMemcpyDeviceToHost, main_s));
  BRX_CUDA(h, cudaStreamSynchronize(main_s));
  if (h->profile) harvest_events(h);
  return collect_errors(h, ir, Q, n, q_host);
}

}  // namespace brx_detail

extern "C" {

int32_t brx_abi_version(void) { return BRX_ABI_VERSION; }

brx_status brx_create(const brx_geometry* gin, int32_t device, brx_handle** out) {
  if (!gin || !out) return BRX_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const brx_geometry& G = *gin;
  if (G.n_faces < 4 || !G.face_abc || !G.face_normal || !G.face_tau || !G.face_tau_len) return BRX_ERR_INVALID_ARGUMENT;
  if (G.n_ops < 1 || !G.ops || !G.op_inverse || G.identity < 0 || G.identity >= G.n_ops) return BRX_ERR_INVALID_ARGUMENT;
  if (G.n_wedge < 0 || (G.n_wedge > 0 && !G.wedge_normal)) return BRX_ERR_INVALID_ARGUMENT;
  for (int d = 0; d < 3; ++d)
    if (G.n_knots[d] < 2 || !G.knots[d]) return BRX_ERR_INVALID_ARGUMENT;
  long long nn = (long long)(G.n_knots[0] - 1) * (G.n_knots[1] - 1) * (G.n_knots[2] - 1);
  if (G.n_nodes != nn || !G.node_type || !G.node_index || G.n_vertices < 1 || !G.vertex_xyz)
    return BRX_ERR_INVALID_ARGUMENT;
  // every index in the tables must stay in bounds: checked here once so the
  // kernels can trust them
  for (long long i = 0; i < G.n_nodes; ++i) {
    int t = G.node_type[i], k = G.node_index[i];
    if (t == BRX_NODE_CUBE && (k < 0 || k >= G.n_cube)) return BRX_ERR_INVALID_ARGUMENT;
    if (t == BRX_NODE_POLY && (k < 0 || k >= G.n_poly)) return BRX_ERR_INVALID_ARGUMENT;
    if (t != BRX_NODE_NULL && t != BRX_NODE_CUBE && t != BRX_NODE_POLY) return BRX_ERR_INVALID_ARGUMENT;
  }
  for (long long i = 0; i < 8LL * G.n_cube; ++i)
    if (G.cube_vertices[i] < 0 || G.cube_vertices[i] >= G.n_vertices) return BRX_ERR_INVALID_ARGUMENT;
  if (G.n_poly > 0) {
    if (!G.poly_tet_offset || G.poly_tet_offset[0] != 0 || G.poly_tet_offset[G.n_poly] != G.n_tets)
      return BRX_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < G.n_poly; ++i)
      if (G.poly_tet_offset[i + 1] < G.poly_tet_offset[i]) return BRX_ERR_INVALID_ARGUMENT;
  }
  for (long long i = 0; i < 4LL * G.n_tets; ++i)
    if (G.tet_vertices[i] < 0 || G.tet_vertices[i] >= G.n_vertices) return BRX_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < G.n_ops; ++i)
    if (G.op_inverse[i] < 0 || G.op_inverse[i] >= G.n_ops) return BRX_ERR_INVALID_ARGUMENT;
  if (G.n_atoms > 0) {
    for (long long i = 0; i < (long long)G.n_atoms * G.n_ops; ++i)
      if (G.gamma_F0[i] < 0 || G.gamma_F0[i] >= G.n_atoms || G.gamma_vidx[i] < 0 || G.gamma_vidx[i] >= G.n_gamma_vectors)
        return BRX_ERR_INVALID_ARGUMENT;
    // every operation permutes the atoms (GammaTable::F0 of the reference);
    // the gathers rely on it
    std::vector<char> seen((size_t)G.n_atoms);
    for (int r = 0; r < G.n_ops; ++r) {
      std::fill(seen.begin(), seen.end(), 0);
      for (int k = 0; k < G.n_atoms; ++k) {
        const int f = G.gamma_F0[(long long)k * G.n_ops + r];
        if (seen[(size_t)f]) return BRX_ERR_INVALID_ARGUMENT;
        seen[(size_t)f] = 1;
      }
    }
  }

  brx_handle* h = new (std::nothrow) brx_handle();
  if (!h) return BRX_ERR_OUT_OF_MEMORY;
  h->device = device;
  h->host_geom = G;
  auto bail = [&](brx_status st) {
    brx_destroy(h);
    return st;
  };
  if (cudaSetDevice(device) != cudaSuccess) return bail(BRX_ERR_CUDA);
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return bail(BRX_ERR_CUDA);
  h->num_sms = prop.multiProcessorCount;
  h->smem_optin = prop.sharedMemPerBlockOptin;
  h->tables.reserve(64);
  DevGeom& g = h->g;
  std::memcpy(g.outer_B, G.outer_B, sizeof g.outer_B);
  std::memcpy(g.prim_B, G.prim_B, sizeof g.prim_B);
  std::memcpy(g.to_prim_6Pt, G.to_prim_6Pt, sizeof g.to_prim_6Pt);
  std::memcpy(g.from_prim_invPt, G.from_prim_invPt, sizeof g.from_prim_invPt);
  g.is_primitive = G.is_primitive;
  g.n_faces = G.n_faces;
  g.n_wedge = G.n_wedge;
  g.wedge_le_ge = G.wedge_le_ge;
  g.n_ops = G.n_ops;
  g.identity = G.identity;
  g.n_nodes = G.n_nodes;
  g.n_cube = G.n_cube;
  g.n_tets = G.n_tets;
  g.n_atoms = G.n_atoms;
  g.t_main = make_tol(G.float_tolerance, G.digit);
  g.t_def = make_tol(0.0, 1);
  brx_status st = BRX_OK;
#define UP(src, cnt, dst) \
  if ((st = upload(h, src, (size_t)(cnt), &dst)) != BRX_OK) return bail(st)
  UP(G.face_abc, 9 * G.n_faces, g.face_abc);
  UP(G.face_normal, 3 * G.n_faces, g.face_normal);
  UP(G.face_tau, 3 * G.n_faces, g.face_tau);
  UP(G.face_tau_len, G.n_faces, g.face_tau_len);
  UP(G.wedge_normal, 3 * G.n_wedge, g.wedge_normal);
  UP(G.ops, 9 * G.n_ops, g.ops);
  UP(G.op_inverse, G.n_ops, g.op_inverse);
  for (int d = 0; d < 3; ++d) {
    g.n_knots[d] = G.n_knots[d];
    UP(G.knots[d], G.n_knots[d], g.knots[d]);
  }
  UP(G.node_type, G.n_nodes, g.node_type);
  UP(G.node_index, G.n_nodes, g.node_index);
  UP(G.cube_vertices, 8LL * G.n_cube, g.cube_vertices);
  // cube corners on the two corner planes of every axis (cube_canon)
  {
    g.cube_canon = 0;
    g.cube_pattern = 0;
    bool canon = G.n_cube > 0;
    int pattern = 0;
    for (long long c = 0; c < G.n_cube && canon; ++c) {
      const int32_t* cv = G.cube_vertices + 8 * c;
      const double* a3 = G.vertex_xyz + 3 * (long long)cv[0];
      const double* b3 = G.vertex_xyz + 3 * (long long)cv[7];
      int pat = 0;
      for (int i = 0; i < 8 && canon; ++i) {
        const double* v = G.vertex_xyz + 3 * (long long)cv[i];
        for (int d = 0; d < 3; ++d) {
          if (a3[d] == b3[d]) { canon = false; break; }
          if (v[d] == b3[d]) pat |= 1 << (3 * i + d);
          else if (v[d] != a3[d]) { canon = false; break; }
        }
      }
      if (c == 0) pattern = pat;
      else if (pat != pattern) canon = false;
    }
    // BRX_EXACT_PREDICATES=1 (every predicate in FP64, no screens) also
    // keeps the per-corner cube weights, for comparison
    const char* exact_env = std::getenv("BRX_EXACT_PREDICATES");
    if (canon && !(exact_env && exact_env[0] == '1')) {
      g.cube_canon = 1;
      g.cube_pattern = pattern;
    }
  }
  // Morton order of the cube nodes' (i, j, k) for the group keys
  {
    const long long nx = G.n_knots[0] - 1, ny = G.n_knots[1] - 1;
    std::vector<std::pair<unsigned long long, int32_t>> code;
    code.reserve((size_t)G.n_cube);
    for (long long node = 0; node < G.n_nodes; ++node) {
      if (G.node_type[node] != BRX_NODE_CUBE) continue;
      const unsigned long long c[3] = {(unsigned long long)(node % nx), (unsigned long long)((node / nx) % ny),
                                       (unsigned long long)(node / (nx * ny))};
      unsigned long long m = 0;
      for (int bit = 0; bit < 21; ++bit)
        for (int d = 0; d < 3; ++d) m |= ((c[d] >> bit) & 1ULL) << (3 * bit + d);
      code.emplace_back(m, G.node_index[node]);
    }
    if ((long long)code.size() != G.n_cube) return bail(BRX_ERR_INVALID_ARGUMENT);
    std::sort(code.begin(), code.end());
    std::vector<int32_t> rank((size_t)G.n_cube), inv((size_t)G.n_cube);
    for (size_t r = 0; r < code.size(); ++r) {
      const int32_t ni = code[r].second;
      if (ni < 0 || ni >= G.n_cube) return bail(BRX_ERR_INVALID_ARGUMENT);
      rank[(size_t)ni] = (int32_t)r;
      inv[r] = ni;
    }
    UP(rank.data(), rank.size(), g.cube_rank);
    UP(inv.data(), inv.size(), h->rank_cube);
  }
  UP(G.poly_tet_offset, G.n_poly + 1, g.poly_tet_offset);
  UP(G.tet_vertices, 4LL * G.n_tets, g.tet_vertices);
  UP(G.tet_sphere, 4LL * G.n_tets, g.tet_sphere);
  UP(G.tet_volume, G.n_tets, g.tet_volume);
  UP(G.vertex_xyz, 3LL * G.n_vertices, g.vertex_xyz);
  UP(G.gamma_F0, (long long)G.n_atoms * G.n_ops, g.gamma_F0);
  UP(G.gamma_vidx, (long long)G.n_atoms * G.n_ops, g.gamma_vidx);
  UP(G.gamma_vectors, 3LL * G.n_gamma_vectors, g.gamma_vectors);
  // Cartesian rotations L·W·L⁻¹ (src/interpolator.hpp:413-419)
  h->rot_cart.resize(9 * (size_t)G.n_ops);
  for (int j = 0; j < G.n_ops; ++j) {
    double W[9], t[9];
    for (int e = 0; e < 9; ++e) W[e] = (double)G.ops[9 * j + e];
    mm3(t, G.lattice_to_xyz, W);
    mm3(&h->rot_cart[9 * (size_t)j], t, G.lattice_from_xyz);
  }
  UP(h->rot_cart.data(), h->rot_cart.size(), g.rot_cart);
  // FP32 screens of the locate stage (brx_locate.cu): face planes through
  // (a, b, c) with orient3d = k·(h − n̂·x), and the wedge normals carried back
  // through each operation, m = B⁻¹ W B n (FP64 here, rounded once to FP32)
  {
    std::vector<float> plane(4 * (size_t)G.n_faces), band(G.n_faces);
    bool ok = g.t_main.rel < 0.5;
    for (int f = 0; f < G.n_faces; ++f) {
      const double* a3 = G.face_abc + 9 * f;
      double u[3], v[3], n[3];
      for (int i = 0; i < 3; ++i) { u[i] = a3[3 + i] - a3[i]; v[i] = a3[6 + i] - a3[i]; }
      n[0] = u[1] * v[2] - u[2] * v[1];
      n[1] = u[2] * v[0] - u[0] * v[2];
      n[2] = u[0] * v[1] - u[1] * v[0];
      const double k = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      if (!(k > 0)) ok = false;
      double h = 0;
      for (int i = 0; i < 3; ++i) { n[i] /= k; h += n[i] * a3[i]; }
      for (int i = 0; i < 3; ++i) plane[4 * f + i] = (float)n[i];
      plane[4 * f + 3] = (float)h;
      // |orient3d| ≤ abs/(1−rel) is the tolerance band; as a distance, /k
      band[f] = (float)(2.0 * g.t_main.abs_ / (1.0 - g.t_main.rel) / k);
    }
    const int nw = G.n_wedge;
    std::vector<float> wm(3 * (size_t)nw * (G.n_ops + 1));
    double Bm[9], Bi[9];
    std::memcpy(Bm, G.outer_B, sizeof Bm);
    // inverse of B (rows b1, b2, b3)
    const double det = Bm[0] * (Bm[4] * Bm[8] - Bm[5] * Bm[7]) - Bm[1] * (Bm[3] * Bm[8] - Bm[5] * Bm[6]) +
                       Bm[2] * (Bm[3] * Bm[7] - Bm[4] * Bm[6]);
    Bi[0] = (Bm[4] * Bm[8] - Bm[5] * Bm[7]) / det;
    Bi[1] = (Bm[2] * Bm[7] - Bm[1] * Bm[8]) / det;
    Bi[2] = (Bm[1] * Bm[5] - Bm[2] * Bm[4]) / det;
    Bi[3] = (Bm[5] * Bm[6] - Bm[3] * Bm[8]) / det;
    Bi[4] = (Bm[0] * Bm[8] - Bm[2] * Bm[6]) / det;
    Bi[5] = (Bm[2] * Bm[3] - Bm[0] * Bm[5]) / det;
    Bi[6] = (Bm[3] * Bm[7] - Bm[4] * Bm[6]) / det;
    Bi[7] = (Bm[1] * Bm[6] - Bm[0] * Bm[7]) / det;
    Bi[8] = (Bm[0] * Bm[4] - Bm[1] * Bm[3]) / det;
    for (int j = 0; j <= G.n_ops; ++j) {
      double W[9];
      for (int e = 0; e < 9; ++e) W[e] = j < G.n_ops ? (double)G.ops[9 * j + e] : (e % 4 == 0 ? 1.0 : 0.0);
      for (int i = 0; i < nw; ++i) {
        const double* n = G.wedge_normal + 3 * i;
        double t1[3], t2[3], t3[3];
        for (int r = 0; r < 3; ++r) t1[r] = Bm[3 * r] * n[0] + Bm[3 * r + 1] * n[1] + Bm[3 * r + 2] * n[2];
        for (int r = 0; r < 3; ++r) t2[r] = W[3 * r] * t1[0] + W[3 * r + 1] * t1[1] + W[3 * r + 2] * t1[2];
        for (int r = 0; r < 3; ++r) t3[r] = Bi[3 * r] * t2[0] + Bi[3 * r + 1] * t2[1] + Bi[3 * r + 2] * t2[2];
        for (int r = 0; r < 3; ++r) wm[3 * ((size_t)j * nw + i) + r] = (float)t3[r];
        // the margin assumes orthogonal operations: |m| = |n|
        const double mn = std::sqrt(t3[0] * t3[0] + t3[1] * t3[1] + t3[2] * t3[2]);
        const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (std::fabs(mn - nn) > 1e-6 * (nn > 1 ? nn : 1)) ok = false;
      }
    }
    double nmax = 0;
    for (int i = 0; i < nw; ++i) {
      const double* n = G.wedge_normal + 3 * i;
      nmax = std::max(nmax, std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]));
    }
    if (nw > 0 && std::fabs(nmax - 1.0) > 1e-6) ok = false;  // the margin assumes unit normals
    g.wedge_band32 = (float)(2.0 * g.t_main.abs_ / (1.0 - g.t_main.rel));
    // BRX_EXACT_PREDICATES=1 turns the screens off (every predicate in FP64)
    const char* env = std::getenv("BRX_EXACT_PREDICATES");
    if (env && env[0] == '1') ok = false;
    // the zero comparisons' screens assume the default tolerance's values
    if (!(g.t_def.rel <= 1e-11 && g.t_def.abs_ == 5e-15)) ok = false;
    g.screen = ok ? 1 : 0;
    UP(plane.data(), plane.size(), g.face_plane32);
    UP(band.data(), band.size(), g.face_band32);
    UP(wm.data(), wm.size(), g.wedge_m32);
    // Barycentric planes of every tetrahedron, w_j(x) = a_j·x + c_j with
    // w_j = orient3d(…x…)/(6V) as tet_contains forms them: (x−d)·n_j/(6V) for
    // j < 3 and (x−a)·n_3/(6V).  A tetrahedron whose planes do not reproduce
    // w_j(v_k) = δ_jk gets NaN offsets and is never screened out.
    std::vector<float> tp(16 * (size_t)G.n_tets);
    for (long long t = 0; t < G.n_tets; ++t) {
      const double* P[4];
      for (int k = 0; k < 4; ++k) P[k] = G.vertex_xyz + 3 * (long long)G.tet_vertices[4 * t + k];
      const double* A = P[0];
      const double* Bv = P[1];
      const double* Cv = P[2];
      const double* D = P[3];
      auto cross = [](const double* u0, const double* u1, const double* v0, const double* v1, double* o) {
        const double u[3] = {u1[0] - u0[0], u1[1] - u0[1], u1[2] - u0[2]};
        const double v[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
        o[0] = u[1] * v[2] - u[2] * v[1];
        o[1] = u[2] * v[0] - u[0] * v[2];
        o[2] = u[0] * v[1] - u[1] * v[0];
      };
      double n[4][3], c[4];
      cross(D, Bv, D, Cv, n[0]);   // (b−d)×(c−d)
      cross(D, Cv, D, A, n[1]);    // (c−d)×(a−d)
      cross(D, A, D, Bv, n[2]);    // (a−d)×(b−d)
      cross(A, Bv, A, Cv, n[3]);   // (b−a)×(c−a), negated below
      for (int i = 0; i < 3; ++i) n[3][i] = -n[3][i];
      const double vol6 = G.tet_volume[t] * 6.0;
      for (int j = 0; j < 4; ++j) {
        const double* o = j < 3 ? D : A;
        for (int i = 0; i < 3; ++i) n[j][i] /= vol6;
        c[j] = -(o[0] * n[j][0] + o[1] * n[j][1] + o[2] * n[j][2]);
      }
      bool good = std::isfinite(vol6) && vol6 != 0.0;
      for (int j = 0; j < 4 && good; ++j)
        for (int k = 0; k < 4; ++k) {
          const double wv = n[j][0] * P[k][0] + n[j][1] * P[k][1] + n[j][2] * P[k][2] + c[j];
          const double scale = std::fabs(n[j][0] * P[k][0]) + std::fabs(n[j][1] * P[k][1]) +
                               std::fabs(n[j][2] * P[k][2]) + std::fabs(c[j]) + 1.0;
          if (!(std::fabs(wv - (j == k ? 1.0 : 0.0)) <= 1e-9 * scale)) good = false;
        }
      for (int j = 0; j < 4; ++j) {
        for (int i = 0; i < 3; ++i) tp[16 * t + 4 * j + i] = good ? (float)n[j][i] : 0.f;
        tp[16 * t + 4 * j + 3] = good ? (float)c[j] : std::numeric_limits<float>::quiet_NaN();
      }
    }
    UP(tp.data(), tp.size(), g.tet_plane32);
  }
#undef UP
  // the host copy keeps only counts: no pointer into caller memory survives
  h->host_geom.face_abc = h->host_geom.face_normal = h->host_geom.face_tau_len = nullptr;
  h->host_geom.face_tau = nullptr;
  h->host_geom.wedge_normal = h->host_geom.tet_sphere = h->host_geom.tet_volume = nullptr;
  h->host_geom.vertex_xyz = h->host_geom.gamma_vectors = nullptr;
  h->host_geom.ops = h->host_geom.op_inverse = h->host_geom.node_type = h->host_geom.node_index = nullptr;
  h->host_geom.cube_vertices = h->host_geom.poly_tet_offset = h->host_geom.tet_vertices = nullptr;
  h->host_geom.gamma_F0 = h->host_geom.gamma_vidx = nullptr;
  for (int d = 0; d < 3; ++d) h->host_geom.knots[d] = nullptr;
  for (auto& s : h->sc) {
    if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess) return bail(BRX_ERR_CUDA);
    if (cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) != cudaSuccess) return bail(BRX_ERR_CUDA);
    if (cudaEventCreateWithFlags(&s.computed, cudaEventDisableTiming) != cudaSuccess) return bail(BRX_ERR_CUDA);
  }
  if (cudaMalloc(&h->err, sizeof(ErrorWord)) != cudaSuccess) return bail(BRX_ERR_OUT_OF_MEMORY);
  if (cudaHostAlloc(&h->err_host, sizeof(ErrorWord), cudaHostAllocDefault) != cudaSuccess) return bail(BRX_ERR_OUT_OF_MEMORY);
  *out = h;
  return BRX_OK;
}

void brx_destroy(brx_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  for (auto& s : h->sc) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    s.rec.release();
    s.sortbuf.release();
    s.groupbuf.release();
    s.qbuf.release();
    s.vbuf.release();
    s.cbuf.release();
    if (s.done) cudaEventDestroy(s.done);
    if (s.computed) cudaEventDestroy(s.computed);
    if (s.stream) cudaStreamDestroy(s.stream);
  }
  for (auto& b : h->tables) b.release();
  for (auto e : h->ev_pool) cudaEventDestroy(e);
  for (auto p : h->group_counts) cudaFreeHost(p);
  h->vals.data.release();
  h->vecs.data.release();
  h->ph_keys.release();
  h->ph_table.release();
  h->perm_keys.release();
  h->perm_ids.release();
  h->perms.release();
  h->mlp_w.release();
  h->mlp_b.release();
  h->mlp_x.release();
  h->mlp_wt.release();
  h->sf_atoms.release();
  h->sf_B.release();
  h->mlp_bt.release();
  if (h->err) cudaFree(h->err);
  if (h->err_host) cudaFreeHost(h->err_host);
  delete h;
}

}  // extern "C"

template <typename In, typename Out>
__global__ void convert_kernel(const In* __restrict__ src, Out* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if constexpr (std::is_same<Out, __nv_bfloat16>::value) dst[i] = __float2bfloat16_rn((float)src[i]);
    else dst[i] = (Out)src[i];
  }
}

template <typename In, typename Out>
static void convert(const In* src, Out* dst, size_t n, cudaStream_t s) {
  if (!n) return;
  size_t blocks = (n + 255) / 256;
  if (blocks > 65536) blocks = 65536;
  convert_kernel<In, Out><<<(unsigned)blocks, 256, 0, s>>>(src, dst, n);
}

extern "C" {

// Vertex data to the device in the storage precision.  Sources are float64
// / complex128 or float32 / complex64, in host or device memory; the
// conversion runs on the device (host sources are staged in chunks).
static brx_status fill_one(brx_handle* h, const brx_data* d, Interp& dst, int storage) {
  if (!d) { dst.present = false; return BRX_OK; }
  if (!d->data || d->n_branches < 1) return fail(h, BRX_ERR_INVALID_ARGUMENT, "data must be non-empty");
  if (d->dtype != BRX_F64 && d->dtype != BRX_C128 && d->dtype != BRX_F32 && d->dtype != BRX_C64)
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "data must be float64, complex128, float32 or complex64");
  for (int i = 0; i < 3; ++i)
    if (d->elements[i] < 0) return fail(h, BRX_ERR_INVALID_ARGUMENT, "negative element count");
  if (d->elements[1] % 3 || d->elements[2] % 9)
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "vector elements must be a multiple of 3 and matrix elements of 9");
  const int s = d->elements[0] + d->elements[1] + d->elements[2];
  if (s < 1) return fail(h, BRX_ERR_INVALID_ARGUMENT, "each branch needs at least one element");
  if (s > 32 * 24) return fail(h, BRX_ERR_INVALID_ARGUMENT, "more than 768 elements per branch are not supported");
  const bool in64 = d->dtype == BRX_F64 || d->dtype == BRX_C128;
  dst.present = true;
  dst.cplx = d->dtype == BRX_C128 || d->dtype == BRX_C64;
  dst.B = d->n_branches;
  dst.s = s;
  for (int i = 0; i < 3; ++i) dst.el[i] = d->elements[i];
  dst.rotates_like = d->rotates_like;
  dst.length_unit = d->length_unit;
  const size_t count = (size_t)h->host_geom.n_vertices * dst.B * s * (dst.cplx ? 2 : 1);  // reals
  const size_t in_size = in64 ? 8 : 4;
  dst.store = storage == BRX_STORE_F64 ? ST_F64 : (storage == BRX_STORE_F32 ? ST_F32 : ST_BF16);
  const size_t out_size = dst.store == ST_F64 ? 8 : (dst.store == ST_F32 ? 4 : 2);
  // 16 bytes of slack: the FP32 gather copies rows in whole 16-byte units
  BRX_CUDA(h, dst.data.ensure(out_size * count + 16));
  cudaStream_t cs = h->sc[0].stream;
  auto conv = [&](const void* src, size_t off, size_t n) {
    char* out = static_cast<char*>(dst.data.p) + out_size * off;
    if (in64) {
      const double* in = static_cast<const double*>(src);
      if (dst.store == ST_F64) convert(in, reinterpret_cast<double*>(out), n, cs);
      else if (dst.store == ST_F32) convert(in, reinterpret_cast<float*>(out), n, cs);
      else convert(in, reinterpret_cast<__nv_bfloat16*>(out), n, cs);
    } else {
      const float* in = static_cast<const float*>(src);
      if (dst.store == ST_F64) convert(in, reinterpret_cast<double*>(out), n, cs);
      else if (dst.store == ST_F32) convert(in, reinterpret_cast<float*>(out), n, cs);
      else convert(in, reinterpret_cast<__nv_bfloat16*>(out), n, cs);
    }
  };
  if (!host_ptr(d->data)) {
    conv(d->data, 0, count);
  } else {
    // chunks of at most 64 Mi reals through one device staging buffer
    const size_t chunk = std::min<size_t>(count, (size_t)64 << 20);
    DevBuf stage;
    if (stage.ensure(in_size * chunk) != cudaSuccess) return fail(h, BRX_ERR_OUT_OF_MEMORY, "fill staging buffer");
    for (size_t off = 0; off < count; off += chunk) {
      const size_t n = std::min(chunk, count - off);
      cudaError_t e = cudaMemcpyAsync(stage.p, static_cast<const char*>(d->data) + in_size * off, in_size * n,
                                      cudaMemcpyHostToDevice, cs);
      if (e == cudaSuccess) {
        conv(stage.p, off, n);
        e = cudaStreamSynchronize(cs);  // the staging buffer is reused
      }
      if (e != cudaSuccess) {
        stage.release();
        return cuda_fail(h, e, "fill");
      }
    }
    stage.release();
  }
  BRX_CUDA(h, cudaGetLastError());
  BRX_CUDA(h, cudaStreamSynchronize(cs));
  return BRX_OK;
}

brx_status brx_fill(brx_handle* h, const brx_data* values, const brx_data* vectors, int32_t storage) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (!values) return fail(h, BRX_ERR_INVALID_ARGUMENT, "values must be provided");
  if (storage < BRX_STORE_F64 || storage > BRX_STORE_BF16) return fail(h, BRX_ERR_INVALID_ARGUMENT, "unknown storage");
  if (vectors && vectors->n_branches != values->n_branches)
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "The values and vectors must have matching number of points and branches");
  BRX_CUDA(h, cudaSetDevice(h->device));
  h->filled = false;
  h->ph_valid = false;
  h->mlp_on = false;  // a residual model belongs to the data it was trained on
  // bfloat16 storage applies to the eigenvectors; eigenvalues keep float32
  brx_status st = fill_one(h, values, h->vals, storage == BRX_STORE_BF16 ? BRX_STORE_F32 : storage);
  if (st) return st;
  st = fill_one(h, vectors, h->vecs, storage);
  if (st) return st;
  h->storage = storage;
  h->filled = true;
  // new data invalidates any permutation table (DualInterpolator::replace_data)
  h->n_keys = 0;
  h->n_perms = 0;
  return build_phase_table(h);
}

brx_status brx_set_permutations(brx_handle* h, int64_t n_keys, const int64_t* keys, const int32_t* perm_ids,
                                int32_t n_perms, const int32_t* perms) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (!h->filled) return fail(h, BRX_ERR_NOT_FILLED, "The interpolation data must be filled before setting permutations.");
  if (n_keys < 0 || n_perms < 0 || (n_keys > 0 && (!keys || !perm_ids || !perms || n_perms < 1)))
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "invalid permutation table");
  const int B = h->vals.B;
  for (long long i = 0; i < n_keys; ++i) {
    if (i && keys[i] <= keys[i - 1]) return fail(h, BRX_ERR_INVALID_ARGUMENT, "permutation keys must be strictly increasing");
    if (perm_ids[i] < 0 || perm_ids[i] >= n_perms) return fail(h, BRX_ERR_INVALID_ARGUMENT, "permutation id out of range");
  }
  for (long long i = 0; i < (long long)n_perms * B; ++i)
    if (perms[i] < 0 || perms[i] >= B) return fail(h, BRX_ERR_INVALID_ARGUMENT, "permutation entry out of range");
  BRX_CUDA(h, cudaSetDevice(h->device));
  h->n_keys = 0;
  h->n_perms = 0;
  h->ph_valid = false;
  if (n_keys == 0) return build_phase_table(h);
  BRX_CUDA(h, h->perm_keys.ensure(sizeof(int64_t) * n_keys));
  BRX_CUDA(h, h->perm_ids.ensure(sizeof(int32_t) * n_keys));
  BRX_CUDA(h, h->perms.ensure(sizeof(int32_t) * (size_t)n_perms * B));
  BRX_CUDA(h, cudaMemcpy(h->perm_keys.p, keys, sizeof(int64_t) * n_keys, cudaMemcpyHostToDevice));
  BRX_CUDA(h, cudaMemcpy(h->perm_ids.p, perm_ids, sizeof(int32_t) * n_keys, cudaMemcpyHostToDevice));
  BRX_CUDA(h, cudaMemcpy(h->perms.p, perms, sizeof(int32_t) * (size_t)n_perms * B, cudaMemcpyHostToDevice));
  h->n_keys = n_keys;
  h->n_perms = n_perms;
  return build_phase_table(h);
}

brx_status brx_ir_interpolate_at(brx_handle* h, const double* Q, int64_t n, void* values_out, void* vectors_out,
                                 uint32_t flags, void* stream) {
  return run_query(h, 1, Q, n, values_out, vectors_out, flags, stream, nullptr);
}

brx_status brx_interpolate_at(brx_handle* h, const double* Q, int64_t n, void* values_out, void* vectors_out,
                              uint32_t flags, void* stream) {
  return run_query(h, 0, Q, n, values_out, vectors_out, flags, stream, nullptr);
}

brx_status brx_set_atoms(brx_handle* h, const brx_atoms* atoms) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (!atoms || atoms->n_atoms < 1 || atoms->n_atoms > 32 || !atoms->weight || !atoms->position)
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "1-32 atoms with weights and positions are needed");
  BRX_CUDA(h, cudaSetDevice(h->device));
  std::vector<double> a(4 * (size_t)atoms->n_atoms);
  for (int k = 0; k < atoms->n_atoms; ++k) {
    a[4 * k] = atoms->weight[k];
    for (int i = 0; i < 3; ++i) a[4 * k + 1 + i] = atoms->position[3 * k + i];
  }
  BRX_CUDA(h, h->sf_atoms.ensure(sizeof(double) * a.size()));
  BRX_CUDA(h, cudaMemcpy(h->sf_atoms.p, a.data(), sizeof(double) * a.size(), cudaMemcpyHostToDevice));
  BRX_CUDA(h, h->sf_B.ensure(sizeof(double) * 9));
  BRX_CUDA(h, cudaMemcpy(h->sf_B.p, h->g.outer_B, sizeof(double) * 9, cudaMemcpyHostToDevice));
  h->sf_n = atoms->n_atoms;
  return BRX_OK;
}

brx_status brx_ir_structure_factor(brx_handle* h, const double* Q, int64_t n, void* values_out, float* sf_out,
                                   uint32_t flags, void* stream) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (!sf_out && n > 0) return fail(h, BRX_ERR_INVALID_ARGUMENT, "output buffers must be provided");
  return run_query(h, 1, Q, n, values_out, sf_out, flags, stream, nullptr, true);
}

brx_status brx_locate(brx_handle* h, const double* Q, int64_t n, int32_t ir, uint32_t flags,
                      const brx_locate_out* out, void* stream) {
  if (!h || !out) return BRX_ERR_INVALID_ARGUMENT;
  if (!out->status) return fail(h, BRX_ERR_INVALID_ARGUMENT, "brx_locate needs a status array");
  brx_status st = run_query(h, ir ? 1 : 0, Q, n, nullptr, nullptr, flags & ~BRX_FLAG_ASYNC, stream, out);
  // per-q status is returned in out->status; the call itself succeeds
  if (st == BRX_ERR_MOVE_FAILED || st == BRX_ERR_OUTSIDE_IR || st == BRX_ERR_NOT_FOUND || st == BRX_ERR_NULL_NODE ||
      st == BRX_ERR_IMPOSSIBLE)
    return BRX_OK;
  return st;
}

brx_status brx_sync(brx_handle* h, void* stream) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (!h->async_pending) return BRX_OK;
  // every stream with queued calls: they share the handle's error word
  if (stream) BRX_CUDA(h, cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  for (cudaStream_t s : h->async_streams) BRX_CUDA(h, cudaStreamSynchronize(s));
  h->async_streams.clear();
  h->async_pending = false;
  BRX_CUDA(h, cudaMemcpyAsync(h->err_host, h->err, sizeof(ErrorWord), cudaMemcpyDeviceToHost, h->sc[0].stream));
  BRX_CUDA(h, cudaStreamSynchronize(h->sc[0].stream));
  if (h->profile) harvest_events(h);
  return collect_errors(h, h->async_ir, h->async_Q, h->async_n, h->async_q_host);
}

const char* brx_last_error(const brx_handle* h) { return h ? h->message.c_str() : "null handle"; }

int64_t brx_launch_count(const brx_handle* h) { return h ? h->launches : 0; }

brx_status brx_profile(brx_handle* h, int32_t enable) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  h->profile = enable != 0;
  h->ev_used = 0;
  for (double& x : h->stage_ms) x = 0;
  h->stage_q = 0;
  h->stage_groups = 0;
  h->group_used = 0;
  return BRX_OK;
}

// Times the gathers under each candidate shared-memory budget on a sample
// query (stage events, best of reps) and keeps the fastest per data kind.
brx_status brx_tune(brx_handle* h, const double* Q, int64_t n, void* values_out, void* vectors_out, uint32_t flags,
                    void* stream, int32_t reps) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (!h->filled) return fail(h, BRX_ERR_NOT_FILLED, "The interpolation data must be filled before interpolating.");
  if (!Q || n < 1) return fail(h, BRX_ERR_INVALID_ARGUMENT, "a non-empty sample is needed");
  if (reps < 1) reps = 1;
  flags &= ~BRX_FLAG_ASYNC;
  const bool f32 = flags & BRX_FLAG_OUT_F32;
  BRX_CUDA(h, cudaSetDevice(h->device));
  // the caller's output buffers, or temporary ones
  DevBuf vo, co;
  const size_t vrow = (size_t)h->vals.B * span(h->vals) * out_elem_bytes(h->vals, f32);
  const size_t crow = h->vecs.present ? (size_t)h->vecs.B * span(h->vecs) * out_elem_bytes(h->vecs, f32) : 0;
  void* vp = values_out;
  void* cp = vectors_out;
  if (!vp) {
    BRX_CUDA(h, vo.ensure(vrow * (size_t)n));
    vp = vo.p;
  }
  if (crow && !cp) {
    cudaError_t e = co.ensure(crow * (size_t)n);
    if (e != cudaSuccess) { vo.release(); return cuda_fail(h, e, "tune buffers"); }
    cp = co.p;
  }
  const size_t cands[] = {24 * 1024, 32 * 1024, 40 * 1024, 56 * 1024, 72 * 1024, 96 * 1024, 128 * 1024, 160 * 1024};
  brx_status st = BRX_OK;
  // time of the gather stage `which` (2 values, 3 vectors), best of reps
  auto timed = [&](int which) -> double {
    double t = 1e300;
    for (int r = 0; r < reps && !st; ++r) {
      brx_profile(h, 1);
      st = run_query(h, 1, Q, n, vp, crow ? cp : nullptr, flags, stream, nullptr);
      if (!st) t = std::min(t, h->stage_ms[which]);
    }
    return t;
  };
  // the heavier gather decides the group size and the work split
  const int lead = (h->vecs.present && uses_groups(h->vecs, h->vecs.cplx)) ? 1 : 0;
  for (int which = 0; which < 2 && !st; ++which) {
    const Interp& d = which ? h->vecs : h->vals;
    if (!d.present || !uses_groups(d, which ? d.cplx : false)) continue;
    size_t best_b = h->gather_budget[which];
    double best = 1e300;
    if (which != lead) {
      for (size_t c : cands) {
        if (c > h->smem_optin || st) continue;
        h->gather_budget[which] = c;
        const double t = timed(2 + which);
        if (st) break;
        if (t < best) { best = t; best_b = c; }
      }
      h->gather_budget[which] = best_b;
      continue;
    }
    // the heavier gather: kernel (FP32 data: warp-independent or
    // CTA-synchronous) × q per descriptor × shared-memory budget, timing
    // each distinct launch shape once
    int rot = ROT_NONE;
    {
      std::string msg;
      if (rotation_mode(d, &rot, &msg)) rot = ROT_NONE;
    }
    const bool fp32 = d.store != ST_F64;
    int best_v = h->gather_variant, best_g = h->group_q;
    std::vector<long long> seen;
    for (int v : {0, 1}) {
      if (!fp32 && v == 0) continue;
      for (int gq : {16, 32, 64, 128}) {
        for (size_t c : cands) {
          if (c > h->smem_optin || st) continue;
          h->gather_variant = v;
          h->group_q = gq;
          h->gather_budget[which] = c;
          GatherParams p = gather_params(h, d, h->sc[0], n, rot, which ? d.cplx : false, which);
          const long long key = gather_shape_key(p, d.store, d.cplx, f32, c);
          if (std::find(seen.begin(), seen.end(), key) != seen.end()) continue;
          seen.push_back(key);
          const double t = timed(2 + which);
          if (st) break;
          if (t < best) { best = t; best_b = c; best_v = v; best_g = gq; }
        }
      }
    }
    h->gather_budget[which] = best_b;
    h->gather_variant = best_v;
    h->group_q = best_g;
    // work units per thread: the CTA-synchronous kernel only
    if (best_v == 1 && !st) {
      int best_s = h->qsplit;
      for (int qs : {1, 2, 4}) {
        h->qsplit = qs;
        const double t = timed(2 + which);
        if (st) break;
        if (t < best) { best = t; best_s = qs; }
      }
      h->qsplit = best_s;
    }
  }
  brx_profile(h, 0);
  h->profile = false;
  vo.release();
  co.release();
  return st;
}

brx_status brx_tuning(const brx_handle* h, int32_t* out, int32_t n) {
  if (!h || !out || n < 1) return BRX_ERR_INVALID_ARGUMENT;
  const int32_t v[5] = {(int32_t)(h->gather_budget[0] / 1024), (int32_t)(h->gather_budget[1] / 1024), h->group_q,
                        h->qsplit, h->gather_variant};
  for (int i = 0; i < n && i < 5; ++i) out[i] = v[i];
  return BRX_OK;
}

brx_status brx_set_tuning(brx_handle* h, const int32_t* v, int32_t n) {
  if (!h || !v || n < 5) return BRX_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < 2; ++i)
    if (v[i] < 8 || (size_t)v[i] * 1024 > h->smem_optin)
      return fail(h, BRX_ERR_INVALID_ARGUMENT, "gather budget out of range");
  if (v[2] < 8 || v[2] > 128) return fail(h, BRX_ERR_INVALID_ARGUMENT, "q per descriptor must be in [8, 128]");
  if (v[3] != 1 && v[3] != 2 && v[3] != 4) return fail(h, BRX_ERR_INVALID_ARGUMENT, "units per thread: 1, 2 or 4");
  if (v[4] != 0 && v[4] != 1) return fail(h, BRX_ERR_INVALID_ARGUMENT, "gather kernel: 0 or 1");
  h->gather_budget[0] = (size_t)v[0] * 1024;
  h->gather_budget[1] = (size_t)v[1] * 1024;
  h->group_q = v[2];
  h->qsplit = v[3];
  h->gather_variant = v[4];
  return BRX_OK;
}

brx_status brx_stage_times(const brx_handle* h, double* ms, int32_t n, int64_t* q_count, int64_t* groups) {
  if (!h || !ms || n < 0) return BRX_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < n && i < 4; ++i) ms[i] = h->stage_ms[i];
  if (q_count) *q_count = h->stage_q;
  if (groups) *groups = h->stage_groups;
  return BRX_OK;
}

}  // extern "C"
