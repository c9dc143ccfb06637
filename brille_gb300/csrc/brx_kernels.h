// Kernel launch interfaces shared by the C-ABI layer.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "brx_device.cuh"

namespace brx {

constexpr int kLocateThreads = 128;
constexpr int kGatherThreads = 128;

enum RotMode { ROT_NONE = 0, ROT_REAL = 1, ROT_RECIP = 2, ROT_AXIAL = 3, ROT_GAMMA = 4 };
enum StoreKind { ST_F64 = 0, ST_F32 = 1, ST_BF16 = 2 };

struct GroupDesc {
  int32_t key;    // group key (cube node / tetrahedron and pivot slot)
  int32_t start;  // first entry in the key-sorted order
  int32_t count;  // number of q (≤ the query's group size)
};

constexpr int kGroupQ = 32;  // default q per work descriptor

struct GatherParams {
  // locate records (chunk-local)
  const int32_t* nw;
  const int32_t* vidx;
  const double* w;
  const float* w32;          // the weights in FP32 (read by the FP32 gathers)
  const int32_t* rot;
  const double* q_ir;
  const int32_t* status;     // per-q status (scalar path)
  const int32_t* order;      // key-sorted q indices
  const GroupDesc* groups;   // work descriptors
  const int32_t* n_groups;   // device count of descriptors
  int32_t* counter;          // work-queue cursor
  long long n;
  // trellis (group key decoding)
  int n_cube;
  const int32_t* cube_vertices;
  const int32_t* rank_cube;  // group-key rank → cube index (Morton order of the cube nodes)
  const int32_t* tet_vertices;
  // vertex data
  const void* data;          // n_vertices × B × s (complex: interleaved pairs)
  int B, s;
  int nsc, nvec, nmat;       // scalars, 3-vectors, 3×3 matrices per branch
  int rot_mode;              // RotMode
  int gamma_cart;            // Γ data in Cartesian (Å) components: use L·W·L⁻¹
  int phase_allowed;         // antiphase alignment (complex vectors)
  // permutation table (sorted keys i*n_vertices+j)
  long long n_keys;
  const long long* keys;
  const int32_t* perm_ids;
  int n_perms;
  const int32_t* perms;
  long long n_vertices;
  // antiphase table of FP64 complex data (null: formed per group): one
  // factor per mode for every sorted key i*n_vertices+j of an ordered pair
  // of vertices sharing a node, against the pivot i
  long long n_ph_keys;
  const long long* ph_keys;
  const double2* ph_table;
  // rotation tables
  const int32_t* ops;
  const double* rot_cart;
  int n_ops;
  const int32_t* gamma_F0;
  const int32_t* gamma_vidx;
  const double* gamma_vectors;
  // output
  void* out;                 // n × B × s, double or float (complex: pairs)
  int MB;                    // modes staged per block
  int qmax;                  // q per work descriptor
  int qsplit;                // FP32 gather: about qsplit work units per thread and block (0: 2)
  ErrorWord* err;            // bounded waits that run out report here
  int variant;               // FP32 gather: 0 warp-independent kernel where it applies, 1 classic
  int stall;                 // BRX_FLAG_TEST_TIMEOUT: the first bounded wait of each warp never completes
  // batches: records are indexed by batch-wide q, the output by q − q_base;
  // group keys are batch-wide, the trellis's own by key − key_base
  long long q_base;
  int key_base;
  // structure factor instead of the vectors (sf_atoms > 0, FP32 warp gather
  // only): per q and mode |Σ_k c_k e^{2πi Q·x_k} (Q_c·e_k)|² into out
  // (float, n × B), Q_c = Q·B
  int sf_atoms;
  const double* sf_Q;     // the caller's Q (r.l.u.), chunk-local, n × 3
  const double* sf_atom;  // sf_atoms × 4: c_k, then x_k (fractional)
  const double* sf_B;     // 9: rows of the reciprocal basis (Å⁻¹)
};

// One persistent gather launch over the groups of many interpolators that
// share storage, complex-ness and output type.  Shared memory is laid out
// for the largest item: e_modes entries of antiphase per slot, ph_atoms Γ
// phases per q, and two staging buffers of ybuf elements.
struct GatherBatch {
  const GatherParams* items;  // n_items, device
  const int32_t* key_off;     // n_items: first batch-wide group key of each item
  int n_items;
  const GroupDesc* groups;
  const int32_t* n_groups;
  int32_t* counter;
  int qmax;
  int e_modes;
  int ph_atoms;
  long long ybuf;
  int warps;  // 0: the classic CTA-synchronous kernel; else the warp-independent one with this many warps
  int reverse;  // descriptor g at groups[-1 - g] (a list written downwards from its end)
  int sf_atoms;  // structure-factor atoms (single interpolator only; 0: vectors)
};

// Second descriptor list of a batch's grouping: keys of class-1 items
// (item_class[i] == 1; key_off ascending over the items) take qmax q per
// descriptor and are written downwards from groups_end.  item_class null:
// one list.
struct GroupSplit {
  const int32_t* key_off = nullptr;
  const int32_t* item_class = nullptr;
  int n_items = 0;
  int qmax = 0;
  GroupDesc* groups_end = nullptr;
  int32_t* n_groups = nullptr;
};

size_t locate_smem_bytes(const DevGeom& g);
void launch_locate(const DevGeom& g, const double* Q, long long n, long long base, int mode, const Records& r,
                   ErrorWord* err, int num_sms, cudaStream_t s);
size_t locate_smem_bytes(const DevGeom& g);
// Locate for many trellises in one launch: tiles (item, first q, count),
// block size 64, 128 or 256.
void launch_locate_batch(const DevGeom* geoms, const long long* q_off, const int32_t* key_off, int key_fail,
                         const int4* tiles, int n_tiles, const double* const* Qptr, int mode, const Records& r,
                         ErrorWord* err, size_t smem, int threads, int grid, cudaStream_t s);

// Counting sort of q by group key and the work descriptors of the groups.
// Returns the number of kernel launches.
int launch_grouping(const int32_t* key, long long n, long long n_keys, int qmax, int32_t* scratch, int32_t* order,
                    GroupDesc* groups, int32_t* n_groups, cudaStream_t s, const GroupSplit& split = GroupSplit{});
size_t group_scratch_ints(long long n_keys);

// Gather + rotate for one interpolator.  Returns the number of launches.
// The vectors gather in structure-factor form (p.sf_atoms > 0, FP32 / BF16
// storage): 1 on launch, -1 when the data do not fit it.
int launch_structure_factor(const GatherParams& p, int store_kind, int num_sms, size_t budget, cudaStream_t s);
int launch_gather(const GatherParams& p, int store_kind, bool cplx, bool out_f32, int num_sms,
                  size_t smem_budget, cudaStream_t s);
size_t gather_smem_bytes(const GatherParams& p, int store_kind, bool cplx, int MB);

// Batched gather: group-ordered items (vector/matrix data) in one persistent
// launch; scalar-only items in one launch over all (q, branch) pairs with
// qb_off[i] = Σ_{k<i} n_k·B_k.  grid 0: one CTA per SM times occupancy.
void launch_gather_batch(const GatherBatch& gb, int store_kind, bool cplx, bool out_f32, int num_sms, size_t smem,
                         int ctas_per_sm, cudaStream_t s);
void launch_scalar_batch(const GatherParams* items, const long long* qb_off, int n_items, long long total,
                         int store_kind, bool cplx, bool out_f32, int num_sms, cudaStream_t s);
// FP32 scalar values with FP32 outputs and no permutation tables: one
// thread per (q, 4 branches); qc_off[i] = Σ_{k<i} n_k·⌈B_k/4⌉.
void launch_scalar_batch_vec(const GatherParams* items, const long long* qc_off, int n_items, long long total,
                             int num_sms, cudaStream_t s);
// shared memory of a batch launch from its largest item dimensions
size_t gather_batch_smem(int store_kind, bool cplx, int qmax, int e_modes, int ph_atoms, long long ybuf);
// staging elements of one block of MB modes of an item with s elements per mode
long long gather_ybuf(int store_kind, bool cplx, int MB, int s);
int gather_max_ctas(int store_kind, bool cplx, bool out_f32, size_t smem);
// The warp-independent FP32 gather for a batch (host copies of the items)
// within a shared-memory budget per CTA: fills gb's layout and warps, the
// launch's shared memory and CTAs per SM; false when an item does not fit
// it (FP64 data, matrices, unaligned data).
bool gather_warp_plan(int store_kind, bool cplx, bool out_f32, const GatherParams* items, int n, int qmax,
                      size_t budget, GatherBatch* gb, size_t* smem, int* ctas_per_sm);

// Antiphase table of FP64 complex data p.data (p.B, p.s, permutation table
// and n_vertices as the gather reads them): out[k·B + b] for every key k.
void launch_phase_table(const GatherParams& p, const long long* keys, long long n_keys, double2* out,
                        cudaStream_t s);

// Load every query kernel of this library on the current device (module
// loading is otherwise deferred to the first launch).
cudaError_t preload_query_kernels();
int gather_pick_modes(const GatherParams& p, int store_kind, bool cplx, size_t smem_budget);
// Launch shape launch_gather takes for p under a budget (kernel, q per
// descriptor, warps and modes per block or modes per block, CTAs per SM)
// as one key: equal keys run alike.
long long gather_shape_key(const GatherParams& p, int store_kind, bool cplx, bool out_f32, size_t budget);

}  // namespace brx
