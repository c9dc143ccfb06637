// Batched queries: many interpolators (different trellises, space groups,
// mode counts and ragged q counts) answered by one persistent launch per
// stage — locate, the counting sort of every item's q by group key, the
// values gather and the vectors gather — so that a whole batch is a fixed
// sequence of launches that a CUDA graph can capture and replay.
//
// The item tables (zone geometry, gather parameters with their output
// pointers, Q pointers, error words) live in one device block that every
// run refreshes from pinned host memory with one copy; a replayed graph
// therefore sees the I/O pointers last given to brx_batch_set_io.
//
// An autotuner (brx_batch_tune) times the launch shapes of locate (block
// size, CTAs per SM, q per tile) and the shared-memory budget of the
// gathers (which sets the modes staged per block and the CTAs per SM) on
// the batch itself with CUDA events, and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/brx.h"
#include "brx_handle.h"
#include "brx_kernels.h"

using namespace brx_detail;

namespace brx_detail {
bool uses_groups(const Interp& d, bool phase);
}

struct brx_batch {
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  int n = 0;
  int mode = 1;  // 0 interpolate_at, 1 ir_interpolate_at, 2 no move
  bool out_f32 = false;
  std::vector<brx_handle*> h;
  std::vector<long long> nq, q_off;
  std::vector<int32_t> key_off;
  long long total_q = 0, total_keys = 0;
  bool vals_grouped = false, has_vecs = false, vecs_grouped = false;
  int vals_store = 0, vecs_store = 0;
  bool vals_cplx = false, vecs_cplx = false;
  std::vector<int> vals_rot, vecs_rot;
  // tuned launch shapes
  int loc_threads = 128, loc_ctas = 4, tile_q = 2048;
  size_t budget_vals = 56 * 1024, budget_vecs = 56 * 1024;
  // gather kernels: with warp on (FP32 data), items of at least warp_min_g
  // element groups per mode take the warp-independent gather (kGroupQ q per
  // descriptor) and the others the CTA-synchronous one with qmax_small q
  // per descriptor (a second descriptor list); with warp off every item
  // takes the CTA-synchronous gather
  bool warp = true;
  int warp_min_g = 8, qmax_small = 64;
  std::vector<int32_t> item_class;  // 1: CTA-synchronous gather with qmax_small
  int n_class[2] = {0, 0};
  bool scalar_vec = false;  // FP32 scalar values by chunks of 4 branches
  // planned from the above
  std::vector<int4> tiles;
  size_t loc_smem = 0;
  // one launch per item class (part) and gather
  struct GatherPlan {
    brx::GatherBatch gb[2];
    size_t smem[2] = {0, 0};
    int ctas[2] = {0, 0};
    bool on[2] = {false, false};
  } gp_vals, gp_vecs;
  std::vector<brx::GatherParams> pv, pc;
  std::vector<long long> qb_off;  // first (q, branch) pair, or chunk of 4 branches, of each item
  // device memory
  DevBuf tables;   // geoms | q_off | key_off | tiles | qb_off
  DevBuf io;       // Qptr | vals params | vecs params | error words
  DevBuf rec, sortbuf, groupbuf;
  brx::Records r{};
  int32_t* order = nullptr;
  int32_t* sort_scratch = nullptr;
  brx::GroupDesc* groups = nullptr;
  int32_t* n_groups = nullptr;
  int32_t* counters = nullptr;
  // device views into the blocks
  const brx::DevGeom* d_geoms = nullptr;
  const long long* d_q_off = nullptr;
  const int32_t* d_key_off = nullptr;
  const int4* d_tiles = nullptr;
  const long long* d_qb_off = nullptr;
  const int32_t* d_class = nullptr;
  long long group_cap = 0;  // descriptors the list holds
  const double* const* d_Q = nullptr;
  brx::GatherParams* d_pv = nullptr;
  brx::GatherParams* d_pc = nullptr;
  brx::ErrorWord* d_err = nullptr;
  // pinned mirror of the io block, and the error words read back
  unsigned char* io_host = nullptr;
  brx::ErrorWord* err_host = nullptr;
  size_t io_bytes = 0, off_pv = 0, off_pc = 0, off_err = 0;
  bool io_set = false;
  std::vector<const double*> Q;
  std::vector<void*> vout, cout;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long graph_launches = 0;  // kernels in the captured graph
  long long launches = 0;
  std::string message = "no error";
};

namespace {

brx_status bfail(brx_batch* b, brx_status st, const std::string& m) {
  if (b) b->message = m;
  return st;
}

#define BB_CUDA(b, call)                                                                       \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return bfail(b, e_ == cudaErrorMemoryAllocation ? BRX_ERR_OUT_OF_MEMORY : BRX_ERR_CUDA,  \
                   std::string("CUDA error in ") + #call + ": " + cudaGetErrorString(e_));     \
  } while (0)

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

brx::GatherParams item_params(brx_batch* b, int i, const Interp& d, int rot_mode, bool phase, int which) {
  brx_handle* h = b->h[i];
  brx::GatherParams p{};
  p.nw = b->r.nw;
  p.vidx = b->r.vidx;
  p.w = b->r.w;
  p.w32 = b->r.w32;
  p.rot = b->r.rot;
  p.q_ir = b->r.q_ir;
  p.status = b->r.status;
  p.order = b->order;
  p.groups = b->groups;
  p.n_groups = b->n_groups;
  p.counter = b->counters + which;
  p.n = b->nq[i];
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
  p.ops = h->g.ops;
  p.rot_cart = h->g.rot_cart;
  p.n_ops = h->g.n_ops;
  p.gamma_F0 = h->g.gamma_F0;
  p.gamma_vidx = h->g.gamma_vidx;
  p.gamma_vectors = h->g.gamma_vectors;
  p.qmax = brx::kGroupQ;
  p.q_base = b->q_off[i];
  p.err = b->d_err + i;
  p.variant = 0;  // the batch chooses its gather kernel for all items at once
  p.key_base = b->key_off[i];
  return p;
}

// Modes per block for every item under a shared-memory budget, and the
// batch launch dimensions (the largest item's) that fit the device.
brx_status plan_gather(brx_batch* b, std::vector<brx::GatherParams>& P, int store, bool cplx, size_t budget, int qmax,
                       brx::GatherBatch* gb, size_t* smem, int* ctas) {
  for (auto& p : P) p.MB = brx::gather_pick_modes(p, store, cplx, budget);
  for (int round = 0; round < 64; ++round) {
    int e = 1, na = 0;
    long long yb = 1;
    for (const auto& p : P) {
      e = std::max(e, p.MB);
      na = std::max(na, p.rot_mode == brx::ROT_GAMMA ? p.nvec : 0);
      yb = std::max(yb, brx::gather_ybuf(store, cplx, p.MB, p.s));
    }
    const size_t need = brx::gather_batch_smem(store, cplx, qmax, e, na, yb);
    bool reducible = false;
    for (const auto& p : P) reducible = reducible || p.MB > 1;
    if (need <= budget || (!reducible && need <= b->smem_optin)) {
      gb->qmax = qmax;
      gb->e_modes = e;
      gb->ph_atoms = na;
      gb->ybuf = yb;
      *smem = need;
      *ctas = brx::gather_max_ctas(store, cplx, b->out_f32, need);
      if (*ctas < 1) return bfail(b, BRX_ERR_INVALID_ARGUMENT, "batch gather does not fit in shared memory");
      return BRX_OK;
    }
    // the largest staging buffer gives up half its modes
    int worst = 0;
    long long wy = -1;
    for (int i = 0; i < (int)P.size(); ++i) {
      const long long y = brx::gather_ybuf(store, cplx, P[i].MB, P[i].s);
      if (y > wy) { wy = y; worst = i; }
    }
    if (P[worst].MB <= 1) {
      // the largest buffer cannot shrink: accept what the device holds
      if (need > b->smem_optin) break;
      gb->qmax = qmax;
      gb->e_modes = e;
      gb->ph_atoms = na;
      gb->ybuf = yb;
      *smem = need;
      *ctas = brx::gather_max_ctas(store, cplx, b->out_f32, need);
      if (*ctas < 1) break;
      return BRX_OK;
    }
    P[worst].MB = (P[worst].MB + 1) / 2;
  }
  return bfail(b, BRX_ERR_INVALID_ARGUMENT, "batch gather does not fit in shared memory");
}

// Tiles, gather parameters, device tables and launch shapes from the tuned
// choices; invalidates a captured graph.
brx_status plan(brx_batch* b) {
  if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  b->tiles.clear();
  for (int i = 0; i < b->n; ++i)
    for (long long s0 = 0; s0 < b->nq[i]; s0 += b->tile_q)
      b->tiles.push_back(make_int4(i, (int)s0, (int)std::min<long long>(b->tile_q, b->nq[i] - s0), 0));
  b->loc_smem = 0;
  for (auto* h : b->h) b->loc_smem = std::max(b->loc_smem, brx::locate_smem_bytes(h->g));
  // gather parameters
  b->pv.clear();
  b->pc.clear();
  b->qb_off.assign(b->n + 1, 0);
  b->scalar_vec = !b->vals_grouped && b->vals_store == brx::ST_F32 && !b->vals_cplx && b->out_f32;
  for (int i = 0; i < b->n; ++i) {
    brx_handle* h = b->h[i];
    b->pv.push_back(item_params(b, i, h->vals, b->vals_rot[i], false, 0));
    if (b->has_vecs) b->pc.push_back(item_params(b, i, h->vecs, b->vecs_rot[i], h->vecs.cplx, 1));
    const long long chunks = b->nq[i] * (long long)((h->vals.B + 3) / 4);
    if (h->n_keys != 0 || chunks >= (1LL << 31)) b->scalar_vec = false;
  }
  for (int i = 0; i < b->n; ++i) {
    const int B = b->h[i]->vals.B;
    b->qb_off[i + 1] = b->qb_off[i] + b->nq[i] * (long long)(b->scalar_vec ? (B + 3) / 4 : B);
  }
  // item classes: the element groups per mode of the grouped data decide
  const std::vector<brx::GatherParams>& lead = b->has_vecs ? b->pc : b->pv;
  const int lead_store = b->has_vecs ? b->vecs_store : b->vals_store;
  const bool split = b->warp && lead_store != brx::ST_F64;
  b->item_class.assign(b->n, 0);
  b->n_class[0] = b->n_class[1] = 0;
  for (int i = 0; i < b->n; ++i) {
    const int G = lead[i].nsc + lead[i].nvec;
    if (split && G < b->warp_min_g) b->item_class[i] = 1;
    ++b->n_class[b->item_class[i]];
  }
  // the gathers, one launch per non-empty class: class 0 the warp-independent
  // kernel if on and its items fit it, else (and class 1) the classic kernel
  // under the shared-memory budget
  auto plan_one = [&](std::vector<brx::GatherParams>& P, int store, bool cplx, size_t budget,
                      brx_batch::GatherPlan* gp) -> brx_status {
    *gp = brx_batch::GatherPlan{};
    for (int c = 0; c < 2; ++c) {
      std::vector<brx::GatherParams> Pc;
      for (int i = 0; i < b->n; ++i)
        if (b->item_class[i] == c) Pc.push_back(P[i]);
      if (Pc.empty()) continue;
      const int qmax = c == 1 ? b->qmax_small : brx::kGroupQ;
      for (auto& p : Pc) p.qmax = qmax;
      gp->on[c] = true;
      if (c == 0 && b->warp &&
          brx::gather_warp_plan(store, cplx, b->out_f32, Pc.data(), (int)Pc.size(), qmax, budget, &gp->gb[c],
                                &gp->smem[c], &gp->ctas[c]))
        continue;
      gp->gb[c] = brx::GatherBatch{};
      brx_status st = plan_gather(b, Pc, store, cplx, budget, qmax, &gp->gb[c], &gp->smem[c], &gp->ctas[c]);
      if (st) return st;
      // the modes per block chosen for the class's items
      for (int i = 0, k = 0; i < b->n; ++i)
        if (b->item_class[i] == c) P[i].MB = Pc[k++].MB;
    }
    return BRX_OK;
  };
  if (b->vals_grouped) {
    brx_status st = plan_one(b->pv, b->vals_store, b->vals_cplx, b->budget_vals, &b->gp_vals);
    if (st) return st;
  }
  if (b->has_vecs) {
    brx_status st = plan_one(b->pc, b->vecs_store, b->vecs_cplx, b->budget_vecs, &b->gp_vecs);
    if (st) return st;
  }
  for (int i = 0; i < b->n; ++i) {
    const int qmax = b->item_class[i] == 1 ? b->qmax_small : brx::kGroupQ;
    b->pv[i].qmax = qmax;
    if (b->has_vecs) b->pc[i].qmax = qmax;
  }
  // device tables: geoms | q_off | key_off | tiles | qb_off | item classes
  const size_t o_geom = 0;
  const size_t o_qoff = align256(o_geom + sizeof(brx::DevGeom) * b->n);
  const size_t o_koff = align256(o_qoff + sizeof(long long) * (b->n + 1));
  const size_t o_tile = align256(o_koff + sizeof(int32_t) * b->n);
  const size_t o_qb = align256(o_tile + sizeof(int4) * std::max<size_t>(1, b->tiles.size()));
  const size_t o_cls = align256(o_qb + sizeof(long long) * (b->n + 1));
  const size_t total = align256(o_cls + sizeof(int32_t) * b->n);
  BB_CUDA(b, b->tables.ensure(total));
  std::vector<unsigned char> host(total, 0);
  for (int i = 0; i < b->n; ++i) std::memcpy(host.data() + o_geom + sizeof(brx::DevGeom) * i, &b->h[i]->g, sizeof(brx::DevGeom));
  std::memcpy(host.data() + o_qoff, b->q_off.data(), sizeof(long long) * (b->n + 1));
  std::memcpy(host.data() + o_koff, b->key_off.data(), sizeof(int32_t) * b->n);
  if (!b->tiles.empty()) std::memcpy(host.data() + o_tile, b->tiles.data(), sizeof(int4) * b->tiles.size());
  std::memcpy(host.data() + o_qb, b->qb_off.data(), sizeof(long long) * (b->n + 1));
  std::memcpy(host.data() + o_cls, b->item_class.data(), sizeof(int32_t) * b->n);
  BB_CUDA(b, cudaMemcpy(b->tables.p, host.data(), total, cudaMemcpyHostToDevice));
  unsigned char* base = static_cast<unsigned char*>(b->tables.p);
  b->d_geoms = reinterpret_cast<const brx::DevGeom*>(base + o_geom);
  b->d_q_off = reinterpret_cast<const long long*>(base + o_qoff);
  b->d_key_off = reinterpret_cast<const int32_t*>(base + o_koff);
  b->d_tiles = reinterpret_cast<const int4*>(base + o_tile);
  b->d_qb_off = reinterpret_cast<const long long*>(base + o_qb);
  b->d_class = reinterpret_cast<const int32_t*>(base + o_cls);
  // class 0 descriptors upwards from the start of the list, class 1
  // downwards from its end
  auto fill_gb = [&](brx_batch::GatherPlan& gp, brx::GatherParams* items, int which) {
    for (int c = 0; c < 2; ++c) {
      brx::GatherBatch& gb = gp.gb[c];
      gb.items = items;
      gb.key_off = b->d_key_off;
      gb.n_items = b->n;
      gb.groups = c == 0 ? b->groups : b->groups + b->group_cap;
      gb.reverse = c;
      gb.n_groups = b->n_groups + c;
      gb.counter = b->counters + 2 * which + c;
    }
  };
  fill_gb(b->gp_vals, b->d_pv, 0);
  fill_gb(b->gp_vecs, b->d_pc, 1);
  return BRX_OK;
}

// Host mirror of the io block: Q pointers, gather parameters (with the
// output pointers) and cleared error words.
void stage_io(brx_batch* b) {
  for (int i = 0; i < b->n; ++i) {
    b->pv[i].out = b->vout[i];
    if (b->has_vecs) b->pc[i].out = b->cout[i];
  }
  std::memcpy(b->io_host, b->Q.data(), sizeof(double*) * b->n);
  std::memcpy(b->io_host + b->off_pv, b->pv.data(), sizeof(brx::GatherParams) * b->n);
  if (b->has_vecs) std::memcpy(b->io_host + b->off_pc, b->pc.data(), sizeof(brx::GatherParams) * b->n);
  brx::ErrorWord z{0, 0, (long long)0x7fffffffffffffffLL};
  for (int i = 0; i < b->n; ++i) std::memcpy(b->io_host + b->off_err + sizeof(brx::ErrorWord) * i, &z, sizeof z);
}

// The run proper: launches and copies only (capturable).  Returns the
// number of kernels launched.
long long enqueue(brx_batch* b, cudaStream_t s, cudaEvent_t* stage_ev) {
  long long k = 0;
  auto mark = [&](int i) {
    if (stage_ev) cudaEventRecord(stage_ev[i], s);
  };
  cudaMemcpyAsync(b->io.p, b->io_host, b->io_bytes, cudaMemcpyHostToDevice, s);
  mark(0);
  if (b->total_q == 0) {  // nothing to locate; the gathers would read no work count
    for (int i = 1; i < 5; ++i) mark(i);
    cudaMemcpyAsync(b->err_host, b->d_err, sizeof(brx::ErrorWord) * b->n, cudaMemcpyDeviceToHost, s);
    return k;
  }
  brx::launch_locate_batch(b->d_geoms, b->d_q_off, b->d_key_off, (int)b->total_keys, b->d_tiles,
                           (int)b->tiles.size(), b->d_Q, b->mode, b->r, b->d_err, b->loc_smem, b->loc_threads,
                           b->num_sms * b->loc_ctas, s);
  ++k;
  mark(1);
  if (b->vals_grouped || b->vecs_grouped) {
    brx::GroupSplit split;
    if (b->n_class[1] > 0) {
      split.key_off = b->d_key_off;
      split.item_class = b->d_class;
      split.n_items = b->n;
      split.qmax = b->qmax_small;
      split.groups_end = b->groups + b->group_cap;
      split.n_groups = b->n_groups + 1;
    }
    k += brx::launch_grouping(b->r.key, b->total_q, b->total_keys, brx::kGroupQ, b->sort_scratch, b->order,
                              b->groups, b->n_groups, s, split);
  }
  mark(2);
  auto gathers = [&](const brx_batch::GatherPlan& gp, int store, bool cplx) {
    for (int c = 0; c < 2; ++c)
      if (gp.on[c]) {
        brx::launch_gather_batch(gp.gb[c], store, cplx, b->out_f32, b->num_sms, gp.smem[c], gp.ctas[c], s);
        ++k;
      }
  };
  if (b->vals_grouped) {
    gathers(b->gp_vals, b->vals_store, b->vals_cplx);
  } else if (b->scalar_vec) {
    brx::launch_scalar_batch_vec(b->d_pv, b->d_qb_off, b->n, b->qb_off[b->n], b->num_sms, s);
  } else {
    brx::launch_scalar_batch(b->d_pv, b->d_qb_off, b->n, b->qb_off[b->n], b->vals_store, b->vals_cplx, b->out_f32,
                             b->num_sms, s);
  }
  if (!b->vals_grouped) ++k;
  mark(3);
  if (b->has_vecs) gathers(b->gp_vecs, b->vecs_store, b->vecs_cplx);
  mark(4);
  cudaMemcpyAsync(b->err_host, b->d_err, sizeof(brx::ErrorWord) * b->n, cudaMemcpyDeviceToHost, s);
  return k;
}

// the io block: layout, device and pinned buffers, sized for n items
brx_status alloc_io(brx_batch* b) {
  b->off_pv = align256(sizeof(double*) * b->n);
  b->off_pc = align256(b->off_pv + sizeof(brx::GatherParams) * b->n);
  b->off_err = align256(b->off_pc + sizeof(brx::GatherParams) * b->n);
  b->io_bytes = align256(b->off_err + sizeof(brx::ErrorWord) * b->n);
  BB_CUDA(b, b->io.ensure(b->io_bytes));
  BB_CUDA(b, cudaMallocHost(&b->io_host, b->io_bytes));
  std::memset(b->io_host, 0, b->io_bytes);
  BB_CUDA(b, cudaMallocHost(&b->err_host, sizeof(brx::ErrorWord) * b->n));
  std::memset(b->err_host, 0, sizeof(brx::ErrorWord) * b->n);
  unsigned char* base = static_cast<unsigned char*>(b->io.p);
  b->d_Q = reinterpret_cast<const double* const*>(base);
  b->d_pv = reinterpret_cast<brx::GatherParams*>(base + b->off_pv);
  b->d_pc = reinterpret_cast<brx::GatherParams*>(base + b->off_pc);
  b->d_err = reinterpret_cast<brx::ErrorWord*>(base + b->off_err);
  return BRX_OK;
}

}  // namespace

extern "C" {

brx_status brx_batch_create(brx_handle* const* handles, int32_t n, const int64_t* n_q, int32_t ir, uint32_t flags,
                            brx_batch** out) {
  if (!out) return BRX_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!handles || n < 1 || !n_q) return BRX_ERR_INVALID_ARGUMENT;
  brx_batch* b = new (std::nothrow) brx_batch;
  if (!b) return BRX_ERR_OUT_OF_MEMORY;
  auto bail = [&](brx_status st) {
    brx_batch_destroy(b);
    return st;
  };
  b->n = n;
  b->out_f32 = flags & BRX_FLAG_OUT_F32;
  b->mode = (flags & BRX_FLAG_NO_MOVE) ? 2 : (ir ? 1 : 0);
  b->h.assign(handles, handles + n);
  b->nq.assign(n_q, n_q + n);
  b->q_off.assign(n + 1, 0);
  b->key_off.assign(n, 0);
  brx_handle* h0 = handles[0];
  if (!h0 || !h0->filled) return bail(BRX_ERR_NOT_FILLED);
  b->device = h0->device;
  b->num_sms = h0->num_sms;
  b->smem_optin = h0->smem_optin;
  b->vals_store = h0->vals.store;
  b->vals_cplx = h0->vals.cplx;
  b->has_vecs = h0->vecs.present;
  b->vecs_store = h0->vecs.store;
  b->vecs_cplx = h0->vecs.cplx;
  b->vals_grouped = uses_groups(h0->vals, false);
  b->vecs_grouped = b->has_vecs;
  long long keys = 0;
  for (int i = 0; i < n; ++i) {
    brx_handle* h = handles[i];
    if (!h || !h->filled || n_q[i] < 0 || n_q[i] > (1LL << 30)) return bail(BRX_ERR_INVALID_ARGUMENT);
    if (h->device != b->device || h->vals.store != b->vals_store || h->vals.cplx != b->vals_cplx ||
        uses_groups(h->vals, false) != b->vals_grouped || h->vecs.present != b->has_vecs ||
        (b->has_vecs && (h->vecs.store != b->vecs_store || h->vecs.cplx != b->vecs_cplx)))
      return bail(BRX_ERR_INVALID_ARGUMENT);
    int vm = brx::ROT_NONE, cm = brx::ROT_NONE;
    if (b->mode == 1) {
      std::string msg;
      if (rotation_mode(h->vals, &vm, &msg)) return bail(BRX_ERR_UNSUPPORTED);
      if (b->has_vecs && rotation_mode(h->vecs, &cm, &msg)) return bail(BRX_ERR_UNSUPPORTED);
    }
    b->vals_rot.push_back(vm);
    b->vecs_rot.push_back(cm);
    b->q_off[i + 1] = b->q_off[i] + n_q[i];
    b->key_off[i] = (int32_t)keys;
    keys += brx::n_group_keys(h->g.n_cube, h->g.n_tets);
  }
  if (keys >= (1LL << 31) - 1 || b->q_off[n] >= (1LL << 31) - 1) return bail(BRX_ERR_INVALID_ARGUMENT);
  b->total_keys = keys;
  b->total_q = b->q_off[n];
  if (cudaSetDevice(b->device) != cudaSuccess) return bail(BRX_ERR_CUDA);
  // records, sort scratch and work descriptors for every q of the batch
  const size_t m = (size_t)std::max<long long>(1, b->total_q);
  const size_t parts[11] = {24 * m, 64 * m, 32 * m, 12 * m, 8 * m, 8 * m, 4 * m, 32 * m, 4 * m, 4 * m, 4 * m};
  size_t rec = 0;
  for (size_t x : parts) rec += align256(x);
  if (b->rec.ensure(rec) != cudaSuccess) return bail(BRX_ERR_OUT_OF_MEMORY);
  char* p = static_cast<char*>(b->rec.p);
  auto take = [&](size_t bytes) {
    char* at = p;
    p += align256(bytes);
    return at;
  };
  b->r.q_ir = reinterpret_cast<double*>(take(24 * m));
  b->r.w = reinterpret_cast<double*>(take(64 * m));
  b->r.w32 = reinterpret_cast<float*>(take(32 * m));
  b->r.tau = reinterpret_cast<int32_t*>(take(12 * m));
  b->r.rot = reinterpret_cast<int32_t*>(take(8 * m));
  b->r.node = reinterpret_cast<int32_t*>(take(8 * m));
  b->r.nw = reinterpret_cast<int32_t*>(take(4 * m));
  b->r.vidx = reinterpret_cast<int32_t*>(take(32 * m));
  b->r.status = reinterpret_cast<int32_t*>(take(4 * m));
  b->order = reinterpret_cast<int32_t*>(take(4 * m));
  b->r.key = reinterpret_cast<int32_t*>(take(4 * m));
  if (b->sortbuf.ensure(sizeof(int32_t) * brx::group_scratch_ints(b->total_keys)) != cudaSuccess)
    return bail(BRX_ERR_OUT_OF_MEMORY);
  b->sort_scratch = static_cast<int32_t*>(b->sortbuf.p);
  if (b->groupbuf.ensure(sizeof(brx::GroupDesc) * m + 256) != cudaSuccess) return bail(BRX_ERR_OUT_OF_MEMORY);
  b->groups = static_cast<brx::GroupDesc*>(b->groupbuf.p);
  b->group_cap = (long long)m;  // both descriptor lists together hold at most one per q
  b->n_groups = reinterpret_cast<int32_t*>(static_cast<char*>(b->groupbuf.p) + sizeof(brx::GroupDesc) * m + 64);
  b->counters = b->n_groups + 16;
  brx_status st = alloc_io(b);
  if (st) return bail(st);
  b->Q.assign(n, nullptr);
  b->vout.assign(n, nullptr);
  b->cout.assign(n, nullptr);
  st = plan(b);
  if (st) return bail(st);
  *out = b;
  return BRX_OK;
}

void brx_batch_destroy(brx_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->io_host) cudaFreeHost(b->io_host);
  if (b->err_host) cudaFreeHost(b->err_host);
  b->tables.release();
  b->io.release();
  b->rec.release();
  b->sortbuf.release();
  b->groupbuf.release();
  delete b;
}

brx_status brx_batch_set_io(brx_batch* b, const double* const* Q, void* const* values, void* const* vectors) {
  if (!b) return BRX_ERR_INVALID_ARGUMENT;
  if (!Q || !values || (b->has_vecs && !vectors)) return bfail(b, BRX_ERR_INVALID_ARGUMENT, "Q and outputs are needed");
  for (int i = 0; i < b->n; ++i) {
    if (b->nq[i] > 0 && (!Q[i] || !values[i] || (b->has_vecs && !vectors[i])))
      return bfail(b, BRX_ERR_INVALID_ARGUMENT, "item " + std::to_string(i) + ": null Q or output");
    for (const void* ptr : {static_cast<const void*>(Q[i]), static_cast<const void*>(values[i]),
                            b->has_vecs ? static_cast<const void*>(vectors[i]) : nullptr}) {
      if (!ptr || b->nq[i] == 0) continue;
      cudaPointerAttributes a{};
      if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess || (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)) {
        cudaGetLastError();
        return bfail(b, BRX_ERR_INVALID_ARGUMENT, "batched queries take device buffers only");
      }
    }
    b->Q[i] = Q[i];
    b->vout[i] = values[i];
    if (b->has_vecs) b->cout[i] = vectors[i];
  }
  b->io_set = true;
  stage_io(b);
  return BRX_OK;
}

brx_status brx_batch_run(brx_batch* b, void* stream) {
  if (!b) return BRX_ERR_INVALID_ARGUMENT;
  if (!b->io_set) return bfail(b, BRX_ERR_INVALID_ARGUMENT, "brx_batch_set_io first");
  BB_CUDA(b, cudaSetDevice(b->device));
  b->launches += enqueue(b, static_cast<cudaStream_t>(stream), nullptr);
  BB_CUDA(b, cudaGetLastError());
  return BRX_OK;
}

brx_status brx_batch_capture(brx_batch* b, void* stream) {
  if (!b) return BRX_ERR_INVALID_ARGUMENT;
  if (!b->io_set) return bfail(b, BRX_ERR_INVALID_ARGUMENT, "brx_batch_set_io first");
  BB_CUDA(b, cudaSetDevice(b->device));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaStream_t cap = s;
  bool own = false;
  if (!s) {  // the legacy stream cannot be captured
    BB_CUDA(b, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    own = true;
  }
  if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    b->graph_launches = enqueue(b, cap, nullptr);
    e = cudaStreamEndCapture(cap, &b->graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (own) cudaStreamDestroy(cap);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return bfail(b, BRX_ERR_CUDA, std::string("graph capture failed: ") + cudaGetErrorString(e));
  }
  return BRX_OK;
}

brx_status brx_batch_launch(brx_batch* b, void* stream) {
  if (!b) return BRX_ERR_INVALID_ARGUMENT;
  if (!b->exec) return brx_batch_run(b, stream);
  BB_CUDA(b, cudaSetDevice(b->device));
  BB_CUDA(b, cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)));
  b->launches += b->graph_launches;
  return BRX_OK;
}

brx_status brx_batch_sync(brx_batch* b, void* stream, int32_t* failed_item) {
  if (!b) return BRX_ERR_INVALID_ARGUMENT;
  if (failed_item) *failed_item = -1;
  BB_CUDA(b, cudaSetDevice(b->device));
  BB_CUDA(b, cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  BB_CUDA(b, cudaGetLastError());
  for (int i = 0; i < b->n; ++i) {
    const brx::ErrorWord ew = b->err_host[i];
    if (!ew.flags) continue;
    brx_handle* h = b->h[i];
    *h->err_host = ew;
    brx_status st = collect_errors(h, b->mode == 1, b->Q[i], b->nq[i], false);
    if (failed_item) *failed_item = i;
    return bfail(b, st, "item " + std::to_string(i) + ": " + h->message);
  }
  return BRX_OK;
}

// Times candidates stage by stage on the batch's current I/O: locate launch
// shapes first, then the gathers' shared-memory budgets (given the tuned
// locate records); keeps the fastest of each and re-plans.
brx_status brx_batch_tune(brx_batch* b, void* stream, int32_t reps) {
  if (!b) return BRX_ERR_INVALID_ARGUMENT;
  if (!b->io_set) return bfail(b, BRX_ERR_INVALID_ARGUMENT, "brx_batch_set_io first");
  if (reps < 1) reps = 1;
  BB_CUDA(b, cudaSetDevice(b->device));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t ev[5];
  for (auto& e : ev) BB_CUDA(b, cudaEventCreate(&e));
  auto time_run = [&](int from, int to) -> float {
    float best = 1e30f;
    for (int r = 0; r < reps; ++r) {
      enqueue(b, s, ev);
      cudaStreamSynchronize(s);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[from], ev[to]);
      best = std::min(best, ms);
    }
    return best;
  };
  brx_status st = BRX_OK;
  // locate: block size, CTAs per SM, q per tile
  {
    int bt = b->loc_threads, bc = b->loc_ctas, bq = b->tile_q;
    float best = 1e30f;
    for (int threads : {64, 128, 256})
      for (int per_sm : {2, 4, 8})
        for (int tq : {1024, 4096}) {
          if (threads * per_sm > 1024) continue;
          b->loc_threads = threads;
          b->loc_ctas = per_sm;
          b->tile_q = tq;
          if (plan(b)) continue;
          stage_io(b);
          const float t = time_run(0, 1);
          if (t < best) { best = t; bt = threads; bc = per_sm; bq = tq; }
        }
    b->loc_threads = bt;
    b->loc_ctas = bc;
    b->tile_q = bq;
  }
  // gathers (the grouped one: vectors, else values), coordinate descent:
  // budget per kernel choice (warp off; warp on for every item), then the
  // class split, then the q per descriptor of the small class
  const size_t budgets[] = {24 * 1024, 40 * 1024, 56 * 1024, 80 * 1024, 112 * 1024};
  const bool vecs = b->has_vecs;
  if (!st && (vecs || b->vals_grouped)) {
    size_t* budget = vecs ? &b->budget_vecs : &b->budget_vals;
    const int from = vecs ? 3 : 2, to = vecs ? 4 : 3;
    const int lead_store = vecs ? b->vecs_store : b->vals_store;
    bool bw = b->warp;
    size_t bb = *budget;
    int bg = b->warp_min_g, bq = b->qmax_small;
    float best = 1e30f;
    auto trial = [&]() -> float {
      if (plan(b)) return 1e30f;
      stage_io(b);
      return time_run(from, to);
    };
    for (int w = 0; w < (lead_store != brx::ST_F64 ? 2 : 1); ++w)
      for (size_t bud : budgets) {
        if (bud > b->smem_optin) continue;
        b->warp = w == 1;
        b->warp_min_g = 0;
        *budget = bud;
        const float t = trial();
        if (t < best) { best = t; bb = bud; bw = b->warp; bg = 0; }
      }
    b->warp = bw;
    *budget = bb;
    b->warp_min_g = bg;
    if (bw) {
      for (int g : {4, 8, 16}) {
        b->warp_min_g = g;
        const float t = trial();
        if (t < best) { best = t; bg = g; }
      }
      b->warp_min_g = bg;
      if (bg > 0)
        for (int q : {32, 64, 128}) {
          b->qmax_small = q;
          const float t = trial();
          if (t < best) { best = t; bq = q; }
        }
      b->qmax_small = bq;
    }
  }
  if (!st && vecs && b->vals_grouped) {
    size_t bb = b->budget_vals;
    float best = 1e30f;
    for (size_t bud : budgets) {
      if (bud > b->smem_optin) continue;
      b->budget_vals = bud;
      if (plan(b)) continue;
      stage_io(b);
      const float t = time_run(2, 3);
      if (t < best) { best = t; bb = bud; }
    }
    b->budget_vals = bb;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (st) return st;
  st = plan(b);
  if (st) return st;
  stage_io(b);
  return BRX_OK;
}

brx_status brx_batch_config(const brx_batch* b, int32_t* cfg, int32_t n) {
  if (!b || !cfg || n < 1) return BRX_ERR_INVALID_ARGUMENT;
  auto ctas = [](const brx_batch::GatherPlan& gp) { return gp.on[0] ? gp.ctas[0] : gp.ctas[1]; };
  auto warps = [](const brx_batch::GatherPlan& gp) { return gp.on[0] ? gp.gb[0].warps : 0; };
  const int32_t v[12] = {b->loc_threads, b->loc_ctas, b->tile_q, (int32_t)(b->budget_vals / 1024),
                         (int32_t)(b->budget_vecs / 1024), ctas(b->gp_vals), ctas(b->gp_vecs),
                         (int32_t)b->tiles.size(), warps(b->gp_vals), warps(b->gp_vecs),
                         b->warp ? b->warp_min_g : -1, b->n_class[1] > 0 ? b->qmax_small : 0};
  for (int i = 0; i < n && i < 12; ++i) cfg[i] = v[i];
  return BRX_OK;
}

brx_status brx_batch_set_config(brx_batch* b, const int32_t* cfg, int32_t n) {
  if (!b || !cfg || n < 5) return BRX_ERR_INVALID_ARGUMENT;
  if (cfg[0] != 64 && cfg[0] != 128 && cfg[0] != 256)
    return bfail(b, BRX_ERR_INVALID_ARGUMENT, "locate threads: 64, 128 or 256");
  if (cfg[1] < 1 || cfg[0] * cfg[1] > 2048) return bfail(b, BRX_ERR_INVALID_ARGUMENT, "locate CTAs per SM out of range");
  if (cfg[2] < 64 || cfg[2] > (1 << 20)) return bfail(b, BRX_ERR_INVALID_ARGUMENT, "q per tile must be in [64, 2^20]");
  for (int i = 3; i < 5; ++i)
    if (cfg[i] < 8 || (size_t)cfg[i] * 1024 > b->smem_optin)
      return bfail(b, BRX_ERR_INVALID_ARGUMENT, "gather budget out of range");
  b->loc_threads = cfg[0];
  b->loc_ctas = cfg[1];
  b->tile_q = cfg[2];
  b->budget_vals = (size_t)cfg[3] * 1024;
  b->budget_vecs = (size_t)cfg[4] * 1024;
  if (n > 10) {
    if (cfg[10] > 64) return bfail(b, BRX_ERR_INVALID_ARGUMENT, "warp gather minimum element groups out of range");
    b->warp = cfg[10] >= 0;
    if (b->warp) b->warp_min_g = cfg[10];
  }
  if (n > 11 && cfg[11] != 0) {
    if (cfg[11] < 8 || cfg[11] > 128) return bfail(b, BRX_ERR_INVALID_ARGUMENT, "q per descriptor must be in [8, 128]");
    b->qmax_small = cfg[11];
  }
  brx_status st = plan(b);
  if (st) return st;
  if (b->io_set) stage_io(b);
  return BRX_OK;
}

int64_t brx_batch_launch_count(const brx_batch* b) { return b ? b->launches : 0; }

const char* brx_batch_last_error(const brx_batch* b) { return b ? b->message.c_str() : "null batch"; }

}  // extern "C"
