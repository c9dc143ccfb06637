// brx_ir_interpolate_at_noalloc: ir_interpolate_at without any allocation.
//
// Who needs it: callers that must not allocate device memory while they run.
// A serving loop with a per-request latency budget cannot take the implicit
// device-wide synchronisation that cudaMalloc and cudaFree bring; a host
// framework that hands all device memory to its own caching pool (PyTorch's
// or JAX's allocator, say) may have nothing left for an outside cudaMalloc,
// and a plugin inside such a host is often not allowed to allocate at all.
// The regular entry point grows its scratch on demand, so any call may
// allocate; this one never does.
//
// How: the per-q scratch of the pipeline (locate records, gather work
// descriptors, work-queue counters) lives in one file-scope __device__ array
// of fixed size, enough for BRX_NOALLOC_MAX_Q q per call (about 14 MB, held by
// every GPU that loads this library until the process exits).  Host code
// cannot use the array's name as a device address, so the first call on each
// device, with that device current, looks the address up with
// cudaGetSymbolAddress and also loads every kernel the call launches; that
// first call should come before any stream capture.  Later calls allocate
// nothing: no cudaMalloc, cudaFree, pinned-host or library allocation.
//
// Every call shares the array and it keeps the last call's contents; the
// counters that must start at zero, and the handle's error word, are cleared
// on the device at the start of each call.  Calls that overlap on the GPU
// (two streams, two handles on one device, or two threads) race on the
// array: serialise them.
//
// Semantics differ from brx_ir_interpolate_at in three ways: Q and the
// outputs must be device memory on the handle's device, n is at most
// BRX_NOALLOC_MAX_Q, and q are gathered one per work group instead of grouped
// by shared vertices.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/brx.h"
#include "brx_handle.h"
#include "brx_kernels.h"

using namespace brx_detail;

namespace {

// per-q bytes: q_ir 24, weights 64, τ 12, R/R⁻¹ 8, node 8, count 4, vertex ids 32, status 4, key 4,
// order 4, work descriptor 12; each array is padded to 256 bytes
constexpr size_t kPerQ = 24 + 64 + 32 + 12 + 8 + 8 + 4 + 32 + 4 + 4 + 4 + 12;
constexpr size_t kScratchBytes = kPerQ * BRX_NOALLOC_MAX_Q + 16 * 256;

static __device__ __align__(256) unsigned char brx_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch[kMaxDevices] = {};

__global__ void one_q_per_group_kernel(const int32_t* status, const int32_t* key, long long n, int32_t* order,
                                       brx::GroupDesc* groups, int32_t* n_groups) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    order[i] = (int32_t)i;
    if (status[i]) continue;
    const int slot = atomicAdd(n_groups, 1);
    brx::GroupDesc g;
    g.key = key[i];
    g.start = (int32_t)i;
    g.count = 1;
    groups[slot] = g;
  }
}

// the array's device address on `device`, looked up once with that device
// current; the kernels are loaded at the same time
brx_status scratch_address(brx_handle* h, void** out) {
  int device = 0;
  BRX_CUDA(h, cudaGetDevice(&device));
  if (device < 0 || device >= kMaxDevices) return fail(h, BRX_ERR_INVALID_ARGUMENT, "device index out of range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, brx_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGetSymbolAddress(brx_noalloc_scratch)");
    e = brx::preload_query_kernels();
    if (e != cudaSuccess) return cuda_fail(h, e, "loading the query kernels");
    cudaFuncAttributes a;
    e = cudaFuncGetAttributes(&a, one_q_per_group_kernel);
    if (e != cudaSuccess) return cuda_fail(h, e, "loading one_q_per_group_kernel");
    g_scratch[device] = p;
  }
  *out = g_scratch[device];
  return BRX_OK;
}

// device (or managed) memory that the handle's device reaches directly;
// device memory of another GPU is refused rather than read as peer memory
bool is_device_ptr(const void* p, int device) {
  if (!p) return false;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == device;
}

}  // namespace

extern "C" brx_status brx_ir_interpolate_at_noalloc(brx_handle* h, const double* Q, int64_t n, void* values_out,
                                                    void* vectors_out, uint32_t flags, void* stream) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (n < 0 || n > BRX_NOALLOC_MAX_Q)
    return fail(h, BRX_ERR_INVALID_ARGUMENT,
                "brx_ir_interpolate_at_noalloc takes at most " + std::to_string(BRX_NOALLOC_MAX_Q) +
                    " q per call; split the batch or use brx_ir_interpolate_at");
  if (!h->filled) return fail(h, BRX_ERR_NOT_FILLED, "The interpolation data must be filled before interpolating.");
  if (h->async_pending) return fail(h, BRX_ERR_INVALID_ARGUMENT, "asynchronous queries must be synchronised with brx_sync first");
  BRX_CUDA(h, cudaSetDevice(h->device));
  void* base = nullptr;
  brx_status st = scratch_address(h, &base);
  if (st) return st;
  if (n == 0) return BRX_OK;
  if (!is_device_ptr(Q, h->device) || !is_device_ptr(values_out, h->device) ||
      (h->vecs.present && !is_device_ptr(vectors_out, h->device)))
    return fail(h, BRX_ERR_INVALID_ARGUMENT,
                "brx_ir_interpolate_at_noalloc needs Q and outputs in device memory of the handle's device");
  std::string msg;
  int vmode = brx::ROT_NONE, cmode = brx::ROT_NONE;
  st = rotation_mode(h->vals, &vmode, &msg);
  if (st) return fail(h, st, msg);
  if (h->vecs.present) {
    st = rotation_mode(h->vecs, &cmode, &msg);
    if (st) return fail(h, st, msg);
  }
  const bool f32 = flags & BRX_FLAG_OUT_F32;
  const int kmode = (flags & BRX_FLAG_NO_MOVE) ? 2 : 1;
  cudaStream_t cs = stream ? static_cast<cudaStream_t>(stream) : h->sc[0].stream;

  // carve the array: one region per per-q field, each 256-byte aligned
  const size_t m = (size_t)BRX_NOALLOC_MAX_Q;
  char* p = static_cast<char*>(base);
  auto take = [&](size_t bytes) {
    char* at = p;
    p += (bytes + 255) & ~size_t(255);
    return at;
  };
  Scratch s;
  s.r.q_ir = reinterpret_cast<double*>(take(24 * m));
  s.r.w = reinterpret_cast<double*>(take(64 * m));
  s.r.w32 = reinterpret_cast<float*>(take(32 * m));
  s.r.tau = reinterpret_cast<int32_t*>(take(12 * m));
  s.r.rot = reinterpret_cast<int32_t*>(take(8 * m));
  s.r.node = reinterpret_cast<int32_t*>(take(8 * m));
  s.r.nw = reinterpret_cast<int32_t*>(take(4 * m));
  s.r.vidx = reinterpret_cast<int32_t*>(take(32 * m));
  s.r.status = reinterpret_cast<int32_t*>(take(4 * m));
  s.r.key = reinterpret_cast<int32_t*>(take(4 * m));
  s.order = reinterpret_cast<int32_t*>(take(4 * m));
  s.groups = reinterpret_cast<brx::GroupDesc*>(take(12 * m));
  s.n_groups = reinterpret_cast<int32_t*>(take(64));
  s.counters = s.n_groups + 4;

  // the counters must start at zero; everything else is overwritten
  BRX_CUDA(h, cudaMemsetAsync(s.n_groups, 0, 64, cs));
  st = reset_errors(h, cs);
  if (st) return st;
  brx::launch_locate(h->g, Q, n, 0, kmode, s.r, h->err, h->num_sms, cs);
  long long blocks = (n + 255) / 256;
  one_q_per_group_kernel<<<(unsigned)blocks, 256, 0, cs>>>(s.r.status, s.r.key, n, s.order, s.groups, s.n_groups);
  h->launches += 2;
  {
    brx::GatherParams gp = gather_params(h, h->vals, s, n, vmode, false, 0);
    gp.out = values_out;
    gp.MB = brx::gather_pick_modes(gp, h->vals.store, h->vals.cplx, smem_budget(h, 0));
    h->launches += brx::launch_gather(gp, h->vals.store, h->vals.cplx, f32, h->num_sms, smem_budget(h, 0), cs);
  }
  if (h->vecs.present) {
    brx::GatherParams gp = gather_params(h, h->vecs, s, n, cmode, h->vecs.cplx, 1);
    gp.out = vectors_out;
    gp.MB = brx::gather_pick_modes(gp, h->vecs.store, h->vecs.cplx, smem_budget(h, 1));
    h->launches += brx::launch_gather(gp, h->vecs.store, h->vecs.cplx, f32, h->num_sms, smem_budget(h, 1), cs);
  }
  BRX_CUDA(h, cudaGetLastError());
  BRX_CUDA(h, cudaMemcpyAsync(h->err_host, h->err, sizeof(brx::ErrorWord), cudaMemcpyDeviceToHost, cs));
  if (flags & BRX_FLAG_ASYNC) {
    h->async_pending = true;
    h->async_stream = cs;
    h->async_streams.assign(1, cs);
    h->async_ir = 1;
    h->async_Q = Q;
    h->async_n = n;
    return BRX_OK;
  }
  BRX_CUDA(h, cudaStreamSynchronize(cs));
  return collect_errors(h, 1, Q, n, false);
}
