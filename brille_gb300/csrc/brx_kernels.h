// Kernel launch interfaces shared by the C-ABI layer.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "brx_device.cuh"

namespace brx {

constexpr int kLocateThreads = 128;
constexpr int kGatherThreads = 256;

enum RotMode { ROT_NONE = 0, ROT_REAL = 1, ROT_RECIP = 2, ROT_AXIAL = 3, ROT_GAMMA = 4 };
enum StoreKind { ST_F64 = 0, ST_F32 = 1, ST_BF16 = 2 };

struct GatherParams {
  // locate records (chunk-local)
  const int32_t* nw;
  const int32_t* vidx;
  const double* w;
  const int32_t* rot;
  const double* q_ir;
  const int32_t* status;
  const int32_t* order;      // processing order (node-sorted) or nullptr
  long long n;
  // vertex data
  const void* data;          // n_vertices × B × s (complex: interleaved pairs)
  int B, s;
  int nsc, nvec, nmat;       // scalars, 3-vectors, 3×3 matrices per branch
  int rot_mode;              // RotMode
  int gamma_cart;            // Γ data in Cartesian (Å) components: use L·W·L⁻¹
  int phase_allowed;         // antiphase alignment (complex vectors)
  int Nmat;                  // Γ matrix block size (atoms)
  // permutation table (sorted keys i*n_vertices+j)
  long long n_keys;
  const long long* keys;
  const int32_t* perm_ids;
  int n_perms;
  const int32_t* perms;
  long long n_vertices;
  // rotation tables
  const int32_t* ops;
  const double* rot_cart;
  int n_ops;
  const int32_t* gamma_F0;
  const int32_t* gamma_vidx;
  const double* gamma_vectors;
  // output
  void* out;                 // n × B × s, double or float (complex: pairs)
  int q_tile;                // q per CTA
  int n_chunks;              // threads per (q, branch), power of two ≤ 32
  int chunk_len;             // elements per thread
};

size_t locate_smem_bytes(const DevGeom& g);
void launch_locate(const DevGeom& g, const double* Q, long long n, long long base, int mode, const Records& r,
                   ErrorWord* err, int num_sms, cudaStream_t s);

// Node-ordered processing: counting sort of q by trellis node.
void launch_node_sort(const int32_t* node, const int32_t* status, long long n, long long n_nodes,
                      int32_t* counts, int32_t* order, cudaStream_t s);
size_t node_sort_scratch_ints(long long n_nodes);

// Gather + rotate for one interpolator.  Returns the number of launches.
int launch_gather(const GatherParams& p, int store_kind, bool cplx, bool out_f32, int num_sms,
                  size_t smem_budget, cudaStream_t s);
size_t gather_smem_bytes(const GatherParams& p, int store_kind, bool cplx, int q_tile);
int gather_pick_tile(const GatherParams& p, int store_kind, bool cplx, size_t smem_budget);

}  // namespace brx
