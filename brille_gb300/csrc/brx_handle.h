// Internals of brx_handle shared by the C-ABI translation units.
// Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/brx.h"
#include "brx_kernels.h"

namespace brx_detail {

using namespace brx;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

struct Interp {
  bool present = false;
  bool cplx = false;
  int store = ST_F64;  // StoreKind of the device copy
  int B = 0, s = 0;
  int el[3] = {0, 0, 0};
  int rotates_like = 0, length_unit = 0;
  DevBuf data;
};

struct Scratch {
  DevBuf rec;     // records
  DevBuf sortbuf; // counts, offsets, cursors, block sums
  DevBuf groupbuf;  // work descriptors + their count + queue cursors
  DevBuf qbuf;    // staged Q
  DevBuf vbuf, cbuf;  // staged outputs (host I/O)
  Records r{};
  int32_t* order = nullptr;
  int32_t* sort_scratch = nullptr;
  GroupDesc* groups = nullptr;
  int32_t* n_groups = nullptr;
  int32_t* counters = nullptr;  // one work-queue cursor per interpolator
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  cudaEvent_t computed = nullptr;  // after this slot's latest chunk's kernels, before its copies
};

}  // namespace brx_detail

struct brx_handle {
  using DevGeom = brx::DevGeom;
  using ErrorWord = brx::ErrorWord;
  using DevBuf = brx_detail::DevBuf;
  using Interp = brx_detail::Interp;
  using Scratch = brx_detail::Scratch;
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  DevGeom g{};
  const int32_t* rank_cube = nullptr;  // device, inverse of g.cube_rank
  std::vector<DevBuf> tables;
  brx_geometry host_geom{};
  std::vector<double> rot_cart;
  Interp vals, vecs;
  int storage = BRX_STORE_F64;
  bool filled = false;
  // permutation table
  DevBuf perm_keys, perm_ids, perms;
  long long n_keys = 0;
  int n_perms = 0;
  // antiphase table of FP64 complex eigenvectors (brx_phase.cu): keys of
  // the vertex pairs that share a node, one factor per key and mode
  DevBuf ph_keys, ph_table;
  long long n_ph_keys = 0;
  bool ph_valid = false;
  Scratch sc[2];
  long long scratch_q = 0;
  ErrorWord* err = nullptr;       // device
  ErrorWord* err_host = nullptr;  // pinned
  std::string message = "no error";
  long long launches = 0;
  // stage timing (brx_profile): events per chunk, accumulated after sync
  bool profile = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  double stage_ms[5] = {0, 0, 0, 0, 0};
  long long stage_q = 0;
  long long stage_groups = 0;
  std::vector<int32_t*> group_counts;  // pinned, one per profiled chunk
  size_t group_used = 0;
  // learned eigenvalue residual (brx_set_residual_model)
  bool mlp_on = false;
  brx_mlp_dims mlp_dims{};
  float mlp_omega_scale = 1.f, mlp_res_scale = 1.f, mlp_clip = 0.f;
  int mlp_groups = 1;  // warp groups per CTA of the inference kernel
  // shared-memory budget per CTA of the values (0) and vectors (1) gathers
  // (modes staged per block, hence CTAs per SM); brx_tune picks them
  size_t gather_budget[2] = {56 * 1024, 56 * 1024};
  int group_q = brx::kGroupQ;  // q per gather work descriptor
  int qsplit = 2;         // FP32 gather work units per thread and block
  int gather_variant = 0; // FP32 gather: 0 warp-independent where it applies, 1 classic
  DevBuf mlp_w, mlp_b, mlp_x;  // bf16 weights, biases, one sub-chunk of feature rows
  bool mlp_tc = false;         // dense layers on tcgen05 (else mma.sync)
  DevBuf mlp_wt, mlp_bt;       // the tcgen05 kernel's weights (core-matrix order) and padded biases
  // structure factor (brx_set_atoms): c_k and fractional x_k per atom, and
  // the reciprocal basis rows, on the device
  int sf_n = 0;
  DevBuf sf_atoms, sf_B;
  bool test_stall = false;  // this call carries BRX_FLAG_TEST_TIMEOUT
  bool async_pending = false;
  cudaStream_t async_stream = nullptr;           // stream of the last queued call
  std::vector<cudaStream_t> async_streams;       // every stream with queued calls
  long long chunk_seq = 0;  // host-I/O chunks so far: chunks alternate streams across calls too
  int async_ir = 0;
  const double* async_Q = nullptr;
  long long async_n = 0;
  bool async_q_host = false;
};

namespace brx_detail {

brx_status fail(brx_handle* h, brx_status st, const std::string& msg);
brx_status cuda_fail(brx_handle* h, cudaError_t e, const char* where);
int span(const Interp& d);
brx_status rotation_mode(const Interp& d, int* mode, std::string* msg);
brx::GatherParams gather_params(brx_handle* h, const Interp& d, const Scratch& s, long long n, int rot_mode,
                                bool phase, int which);
size_t smem_budget(brx_handle* h, int which);
size_t out_elem_bytes(const Interp& d, bool f32);
brx_status collect_errors(brx_handle* h, int ir, const double* Q, long long n, bool q_host);
brx_status reset_errors(brx_handle* h, cudaStream_t s);
// (Re)builds the antiphase table after the vertex data or the permutation
// table changed (no-op unless the eigenvectors are complex FP64 data).
brx_status build_phase_table(brx_handle* h);
// Adds the learned residual to the eigenvalues just gathered for a chunk;
// returns the number of kernels launched (0 without a model).
int launch_residual(brx_handle* h, const Scratch& s, long long n, void* values_out, bool out_f32, cudaStream_t cs);

}  // namespace brx_detail

#define BRX_CUDA(h, call)                                                   \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) return brx_detail::cuda_fail(h, e_, #call);      \
  } while (0)
