// Learned residual correction of interpolated eigenvalues.
//
// A small MLP (d_in → 128 → 128 → 128 → n_out, tanh-form GELU) predicts, per mode, the
// difference between the exact eigenvalue and the trellis interpolation at
// q.  Its input row is built on the GPU from the locate record of q:
//
//   col 0-2    position of q in its node cell, (x − knot_lo)/(knot_hi − knot_lo)
//   col 3-10   weights of the (up to) 8 vertex slots, 0 for unused slots
//   col 11     1 for a tetrahedron, 0 for a cube node
//   col 12 …   vertex eigenvalues, slot-major: 12 + slot·B + mode
//   then       interpolated eigenvalues, B columns
//   then       position of q in the trellis box, (x − knot_first)/(knot_last − knot_first), 3 columns
//   then       zero padding up to d_in
//
// eigenvalues divided by omega_scale.  Training runs on the FP32 CUDA-core
// kernels of this file (a tiled GEMM with optional transposes, bias + GELU,
// GELU derivative, bias sums, Adam).  Weights, biases and activations are
// rounded to bfloat16 wherever inference rounds them, so training sees the
// inference arithmetic; gradients pass straight through the rounding onto
// FP32 master weights.  Inference is one fused kernel on the tensor cores
// (mma m16n8k16, bf16 operands, FP32 accumulate): feature rows into a
// shared-memory tile, four dense layers, and the residual added to the
// eigenvalues the gather wrote, 128 q per tile.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/brx.h"
#include "brx_handle.h"
#include "brx_kernels.h"

namespace brx {

constexpr int kWidth = 128;

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
// GELU in its tanh form, 0.5·x·(1 + tanh(√(2/π)·(x + 0.044715·x³))).
// Training evaluates tanh accurately; inference uses the special-function
// unit's tanh.approx (relative error about 2⁻¹¹, below the bf16 rounding of
// the activations), one instruction where an erf costs a dozen.
constexpr float kGeluC = 0.7978845608028654f, kGeluA = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
  const float u = kGeluC * fmaf(kGeluA * x * x, x, x);
  return 0.5f * x * (1.f + tanhf(u));
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float x2 = x * x;
  const float t = tanhf(kGeluC * fmaf(kGeluA * x2, x, x));
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * kGeluC * fmaf(3.f * kGeluA, x2, 1.f);
}
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;\n" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu_fast(float x) {
  const float h = 0.5f * x;
  return fmaf(h, tanh_approx(kGeluC * fmaf(kGeluA * x * x, x, x)), h);
}

// Offsets of the parameter blocks in the flat FP32 parameter vector:
// W0 (128 × d_in), b0, W1 (128 × 128), b1, W2, b2, W3 (n_out × 128), b3;
// every W row-major [out][in].
struct MlpLayout {
  long long W[4], b[4], total;
  int in[4], out[4];
};

__host__ __device__ inline MlpLayout mlp_layout(int d_in, int n_out) {
  MlpLayout L;
  L.in[0] = d_in;   L.out[0] = kWidth;
  L.in[1] = kWidth; L.out[1] = kWidth;
  L.in[2] = kWidth; L.out[2] = kWidth;
  L.in[3] = kWidth; L.out[3] = n_out;
  long long o = 0;
  for (int l = 0; l < 4; ++l) {
    L.W[l] = o; o += (long long)L.out[l] * L.in[l];
    L.b[l] = o; o += L.out[l];
  }
  L.total = o;
  return L;
}

// ---------------------------------------------------------------------------
// feature rows
// ---------------------------------------------------------------------------
struct FeatureArgs {
  const double* q_ir;
  const int32_t* node;     // n × 2
  const int32_t* nw;
  const int32_t* vidx;     // n × 8
  const double* w;         // n × 8
  const float* w32;        // n × 8 FP32 copies, or null
  const int32_t* status;
  long long n;
  const void* values;      // n_vertices × B, float or double
  int values_f64;
  int B;
  int d_in;
  float inv_omega;         // 1 / omega_scale
};


// Feature arithmetic is FP32 with explicit rounding (no contraction), so
// that the oracle repeats it bit for bit; the rows are rounded to bf16 for
// the network anyway.
//
// The whole row of q i through put(col, value) (the caller zeroes the row
// first and has checked status[i] == 0): position in the node cell (0-2),
// slot weights (3-10), tetrahedron flag (11), vertex eigenvalues
// (12 + slot·B + mode), interpolated eigenvalues Σ w·v in slot order
// (12 + 8B + mode, also returned through base unscaled; the FP32 gather
// forms the same sum, possibly with fused multiply-adds), position in the
// trellis box (12 + 9B + 0..2), and the distance |q_ir| to Γ over the
// longest side of that box (15 + 9B): acoustic branches rise as a cone
// from Γ, where linear interpolation errs most.
// The record's vertex ids and weights are read once, as vectors.
template <typename VT, class Put>
__device__ __forceinline__ void feature_all(const DevGeom& g, const FeatureArgs& a, long long i, Put put,
                                            float* base) {
  const int node = a.node[2 * i], tet = a.node[2 * i + 1];
  const int nx = g.n_knots[0] - 1, ny = g.n_knots[1] - 1;
  const int rest = node / nx;
  const int sub[3] = {node - rest * nx, rest % ny, rest / ny};
  const float q0 = (float)a.q_ir[3 * i], q1 = (float)a.q_ir[3 * i + 1], q2 = (float)a.q_ir[3 * i + 2];
  float x[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
    x[d] = __fadd_rn(__fadd_rn(__fmul_rn((float)g.outer_B[d], q0), __fmul_rn((float)g.outer_B[3 + d], q1)),
                     __fmul_rn((float)g.outer_B[6 + d], q2));
  const int B = a.B;
  float span = 0.f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double* kn = g.knots[d];
    const float lo = (float)kn[sub[d]], hi = (float)kn[sub[d] + 1];
    put(d, __fdiv_rn(__fsub_rn(x[d], lo), __fsub_rn(hi, lo)));
    const float lo0 = (float)kn[0], hi0 = (float)kn[g.n_knots[d] - 1];
    put(12 + 9 * B + d, __fdiv_rn(__fsub_rn(x[d], lo0), __fsub_rn(hi0, lo0)));
    span = fmaxf(span, __fsub_rn(hi0, lo0));
  }
  const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(x[0], x[0]), __fmul_rn(x[1], x[1])), __fmul_rn(x[2], x[2]));
  put(15 + 9 * B, __fdiv_rn(__fsqrt_rn(r2), span));
  const int nw = min(a.nw[i], 8);
  const int4 v0 = reinterpret_cast<const int4*>(a.vidx + 8 * i)[0];
  const int4 v1 = reinterpret_cast<const int4*>(a.vidx + 8 * i)[1];
  const int vid[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
  float wf[8];
  if (a.w32) {
    const float4 w0 = reinterpret_cast<const float4*>(a.w32 + 8 * i)[0];
    const float4 w1 = reinterpret_cast<const float4*>(a.w32 + 8 * i)[1];
    wf[0] = w0.x; wf[1] = w0.y; wf[2] = w0.z; wf[3] = w0.w;
    wf[4] = w1.x; wf[5] = w1.y; wf[6] = w1.z; wf[7] = w1.w;
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const double2 w2 = reinterpret_cast<const double2*>(a.w + 8 * i)[k];
      wf[2 * k] = (float)w2.x;
      wf[2 * k + 1] = (float)w2.y;
    }
  }
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if (k < nw) put(3 + k, wf[k]);
  put(11, tet >= 0 ? 1.f : 0.f);
  const VT* vals = static_cast<const VT*>(a.values);
  for (int b = 0; b < B; ++b) {
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k < nw) {
        const float ev = (float)vals[(long long)vid[k] * B + b];
        put(12 + k * B + b, __fmul_rn(ev, a.inv_omega));
        s = __fadd_rn(s, __fmul_rn(wf[k], ev));
      }
    }
    if (base) base[b] = s;
    put(12 + 8 * B + b, __fmul_rn(s, a.inv_omega));
  }
}

// The row through put and the plain values through base (NaN where the
// locate failed); the caller zeroes the row first.
template <class Put>
__device__ void feature_row(const DevGeom& g, const FeatureArgs& a, long long i, Put put, float* base) {
  if (a.status[i]) {
    for (int b = 0; b < a.B; ++b) base[b] = __int_as_float(0x7fc00000);
    return;
  }
  if (a.values_f64) feature_all<double>(g, a, i, put, base);
  else feature_all<float>(g, a, i, put, base);
}

__global__ void mlp_features_kernel(DevGeom g, FeatureArgs a, float* X, float* base) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < a.n; i += (long long)gridDim.x * blockDim.x) {
    float* row = X + i * a.d_in;
    for (int k = 0; k < a.d_in; ++k) row[k] = 0.f;
    feature_row(g, a, i, [row](int k, float v) { row[k] = v; }, base + i * a.B);
  }
}

// ---------------------------------------------------------------------------
// training kernels (FP32 CUDA cores)
// ---------------------------------------------------------------------------
// C[M×N] = Σ_k A(m,k)·B(k,n);
// A(m,k) = A[m·lda+k], or A[k·lda+m] when transA;
// B(k,n) = B[k·ldb+n], or B[n·ldb+k] when transB.
// Operands are rounded to bfloat16 on load when roundA / roundB.
constexpr int kTile = 64, kTK = 16;

__global__ void __launch_bounds__(256)
gemm_f32_kernel(int M, int N, int K, const float* A, int lda, int transA, int roundA, const float* Bm, int ldb,
                int transB, int roundB, float* C, int ldc) {
  __shared__ float As[kTK][kTile + 1];
  __shared__ float Bs[kTK][kTile + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kTK) {
    for (int t = threadIdx.x; t < kTK * kTile; t += 256) {
      // consecutive threads walk the operand's contiguous index
      int kk, mm;
      if (transA) { kk = t / kTile; mm = t % kTile; } else { kk = t % kTK; mm = t / kTK; }
      const int m = m0 + mm, k = k0 + kk;
      float v = 0.f;
      if (m < M && k < K) v = transA ? A[(long long)k * lda + m] : A[(long long)m * lda + k];
      As[kk][mm] = roundA ? bf16_round(v) : v;
      int kb, nn;
      if (transB) { kb = t % kTK; nn = t / kTK; } else { kb = t / kTile; nn = t % kTile; }
      const int n = n0 + nn, kq = k0 + kb;
      float u = 0.f;
      if (n < N && kq < K) u = transB ? Bm[(long long)n * ldb + kq] : Bm[(long long)kq * ldb + n];
      Bs[kb][nn] = roundB ? bf16_round(u) : u;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) { a[i] = As[kk][ty * 4 + i]; b[i] = Bs[kk][tx * 4 + i]; }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
      if (m < M && n < N) C[(long long)m * ldc + n] = acc[i][j];
    }
}

static void gemm(int M, int N, int K, const float* A, int lda, int tA, int rA, const float* B, int ldb, int tB, int rB,
                 float* C, int ldc, cudaStream_t s) {
  dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
  gemm_f32_kernel<<<grid, 256, 0, s>>>(M, N, K, A, lda, tA, rA, B, ldb, tB, rB, C, ldc);
}

static unsigned elem_blocks(long long total, int threads) {
  long long b = (total + threads - 1) / threads;
  return (unsigned)(b > 8192 ? 8192 : (b < 1 ? 1 : b));
}

// Z += bf16(bias); H = bf16(GELU(Z)) for hidden layers, H = Z for the
// output (no bf16 rounding when rnd is 0)
__global__ void bias_act_kernel(float* Z, float* H, const float* bias, long long M, int N, int act, int rnd) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M * N; t += (long long)gridDim.x * blockDim.x) {
    const float b = bias[t % N];
    const float z = Z[t] + (rnd ? bf16_round(b) : b);
    Z[t] = z;
    if (act) {
      const float h = gelu(z);
      H[t] = rnd ? bf16_round(h) : h;
    } else {
      H[t] = z;
    }
  }
}

// Mean squared error over the first B outputs of each row: dY = 2(Y − T)/(M·B)
// (0 on padding columns), loss += Σ(Y − T)²/(M·B).
__global__ void mse_grad_kernel(const float* Y, const float* T, float* dY, long long M, int n_out, int B, float* loss) {
  float part = 0.f;
  const float scale = 1.f / ((float)M * B);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M * n_out; t += (long long)gridDim.x * blockDim.x) {
    const long long m = t / n_out;
    const int b = (int)(t % n_out);
    float d = 0.f;
    if (b < B) {
      const float e = Y[t] - T[m * B + b];
      d = 2.f * e * scale;
      part += e * e * scale;
    }
    dY[t] = d;
  }
  for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, part);
}

__global__ void gelu_backward_kernel(float* dH, const float* Z, long long total) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x)
    dH[t] *= gelu_grad(Z[t]);
}

// db[n] = Σ_m dZ[m][n], one block per column
__global__ void __launch_bounds__(256) colsum_kernel(const float* dZ, long long M, int N, float* db) {
  const int n = blockIdx.x;
  float s = 0.f;
  for (long long m = threadIdx.x; m < M; m += blockDim.x) s += dZ[m * N + n];
  __shared__ float red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int off = 128; off > 0; off >>= 1) {
    if ((int)threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) db[n] = red[0];
}

__global__ void adam_kernel(float* p, const float* g, float* m, float* v, long long n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// Workspace: Z1..Z3 and H1..H3 (M × 128 each), Y and dY (M × n_out), two
// M × 128 gradient buffers.
size_t mlp_workspace_floats(long long M, int n_out) { return (size_t)M * (8 * kWidth + 2 * n_out); }

struct Work {
  float *Z[3], *H[3], *Y, *dY, *dA, *dB;
};

static Work carve(float* ws, long long M, int n_out) {
  Work w;
  for (int l = 0; l < 3; ++l) {
    w.Z[l] = ws + (size_t)M * kWidth * l;
    w.H[l] = ws + (size_t)M * kWidth * (3 + l);
  }
  w.Y = ws + (size_t)M * kWidth * 6;
  w.dY = w.Y + (size_t)M * n_out;
  w.dA = w.dY + (size_t)M * n_out;
  w.dB = w.dA + (size_t)M * kWidth;
  return w;
}

// Forward pass in training arithmetic; outputs land in w.Y.
static void mlp_forward_train(int d_in, int n_out, int rnd, const float* P, const float* X, long long M,
                              const Work& w, cudaStream_t s) {
  const MlpLayout L = mlp_layout(d_in, n_out);
  const float* Hin = X;
  for (int l = 0; l < 4; ++l) {
    float* Zl = l < 3 ? w.Z[l] : w.Y;
    float* Hl = l < 3 ? w.H[l] : w.Y;
    // Z = H_prev · Wᵀ: B(k,n) = W[n·in + k]
    gemm((int)M, L.out[l], L.in[l], Hin, L.in[l], 0, rnd, P + L.W[l], L.in[l], 1, rnd, Zl, L.out[l], s);
    bias_act_kernel<<<elem_blocks(M * L.out[l], 256), 256, 0, s>>>(Zl, Hl, P + L.b[l], M, L.out[l], l < 3, rnd);
    Hin = Hl;
  }
}

// Backward pass from w.dY into the gradient vector G (same layout as P).
static void mlp_backward(int d_in, int n_out, int rnd, const float* P, float* G, const float* X, long long M,
                         const Work& w, cudaStream_t s) {
  const MlpLayout L = mlp_layout(d_in, n_out);
  float* dZ = w.dY;
  for (int l = 3; l >= 0; --l) {
    const float* Hprev = l > 0 ? w.H[l - 1] : X;
    // dW = dZᵀ · H_prev (out × in): A(m,k) = dZ[k·out + m]
    gemm(L.out[l], L.in[l], (int)M, dZ, L.out[l], 1, 0, Hprev, L.in[l], 0, rnd, G + L.W[l], L.in[l], s);
    colsum_kernel<<<L.out[l], 256, 0, s>>>(dZ, M, L.out[l], G + L.b[l]);
    if (l == 0) break;
    // dH_prev = dZ · bf16(W) (M × in), then through the GELU of layer l−1
    float* dH = dZ == w.dA ? w.dB : w.dA;
    gemm((int)M, L.in[l], L.out[l], dZ, L.out[l], 0, 0, P + L.W[l], L.in[l], 0, rnd, dH, L.in[l], s);
    gelu_backward_kernel<<<elem_blocks(M * L.in[l], 256), 256, 0, s>>>(dH, w.Z[l - 1], M * (long long)L.in[l]);
    dZ = dH;
  }
}

// ---------------------------------------------------------------------------
// inference: features + four dense layers on the tensor cores + residual add
// ---------------------------------------------------------------------------
constexpr int kInferRows = 128;        // q per tile, one tile per warp group at a time
constexpr int kGroupThreads = 256;     // a warp group: 8 warps × 16 rows
constexpr int kMaxGroups = 2;          // warp groups per CTA

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void ldsm_x4(uint32_t* r, uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr)
               : "memory");
}

__device__ __forceinline__ void ldsm_x2(uint32_t* r, uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(addr)
               : "memory");
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// named barrier of one warp group (id 1 + group; 0 is __syncthreads)
__device__ __forceinline__ void group_sync(int group) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(1 + group), "n"(kGroupThreads) : "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}


// bf16 elements per shared-memory row of the hidden activations and of the
// staged feature rows: 8 extra spread the rows over the banks (strides of
// 2·cols + 16 bytes put the 8 rows of an ldmatrix phase on disjoint banks)
// and keep every row 16-byte aligned
__host__ __device__ inline int act_stride() { return kWidth + 8; }
__host__ __device__ inline int stage_stride(int d_in) { return d_in + 8; }

__device__ __forceinline__ void cp_async16(uint32_t saddr, const void* gaddr) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(saddr), "l"(gaddr) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// One warp computes its 16 rows × (8·NT) output columns of a layer with
// K = in: A fragments (ldmatrix.x4) from src (row stride ss), B fragments
// (ldmatrix.x4 for two n-tiles, .x2 for one) from the layer's weight rows
// W[n][k].  Hidden layers write bf16(GELU(acc + b)) to the warp's rows of
// dst (row stride ds); the output layer writes acc + b to out.
template <int NT, bool kHidden>
__device__ __forceinline__ void warp_layer(const __nv_bfloat16* Wl, int in, int ws, const float* bl,
                                           const __nv_bfloat16* src, int ss, __nv_bfloat16* dst, int ds, int row0,
                                           int lane, float* out, int out_ld, int n_valid) {
  float acc[NT][4];
#pragma unroll
  for (int t = 0; t < NT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
  const int mat = lane >> 3, r8 = lane & 7;
  // A: matrices (rows 0-7, k 0-7), (rows 8-15, k 0-7), (rows 0-7, k 8-15), (rows 8-15, k 8-15)
  const uint32_t a_addr = smem_u32(src + (size_t)(row0 + r8 + ((mat & 1) << 3)) * ss + ((mat >> 1) << 3));
  // B, two n-tiles: (tile 0, k 0-7), (tile 0, k 8-15), (tile 1, k 0-7), (tile 1, k 8-15)
  const uint32_t b_addr = NT == 1 ? smem_u32(Wl + (size_t)r8 * ws + ((mat & 1) << 3))
                                  : smem_u32(Wl + (size_t)(((mat >> 1) << 3) + r8) * ws + ((mat & 1) << 3));
  for (int k0 = 0; k0 < in; k0 += 16) {
    uint32_t a[4];
    ldsm_x4(a, a_addr + 2 * k0);
    if (NT == 1) {
      uint32_t b[2];
      ldsm_x2(b, b_addr + 2 * k0);
      mma_bf16(acc[0], a, b);
    } else {
#pragma unroll
      for (int p = 0; p < NT / 2; ++p) {
        uint32_t b[4];
        ldsm_x4(b, b_addr + 2 * (p * 16 * ws + k0));
        mma_bf16(acc[2 * p], a, b);
        mma_bf16(acc[2 * p + 1], a, b + 2);
      }
    }
  }
  __syncwarp();
  const int g = lane >> 2, tq = lane & 3;
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    const int c0 = t * 8 + 2 * tq;
    if (kHidden) {
      const float b0 = bl[c0], b1 = bl[c0 + 1];
      *reinterpret_cast<uint32_t*>(dst + (size_t)(row0 + g) * ds + c0) =
          pack_bf16(gelu_fast(acc[t][0] + b0), gelu_fast(acc[t][1] + b1));
      *reinterpret_cast<uint32_t*>(dst + (size_t)(row0 + g + 8) * ds + c0) =
          pack_bf16(gelu_fast(acc[t][2] + b0), gelu_fast(acc[t][3] + b1));
    } else {
      if (c0 < n_valid) {
        out[(row0 + g) * out_ld + c0] = acc[t][0] + bl[c0];
        out[(row0 + g + 8) * out_ld + c0] = acc[t][2] + bl[c0];
      }
      if (c0 + 1 < n_valid) {
        out[(row0 + g) * out_ld + c0 + 1] = acc[t][1] + bl[c0 + 1];
        out[(row0 + g + 8) * out_ld + c0 + 1] = acc[t][3] + bl[c0 + 1];
      }
    }
  }
  __syncwarp();
}

// bf16 feature rows X of one sub-chunk in tiles of 128 rows, each tile in
// the tensor cores' canonical K-major layout without swizzle: 8-row × 16-byte
// core matrices, K-groups adjacent (128 B apart), 8-row groups d_in·16 B
// apart.  Each thread builds one row in shared memory, then the block writes
// its tile as contiguous 16-byte stores.
constexpr int kRowsPerBlock = 128;

__global__ void __launch_bounds__(kRowsPerBlock) mlp_xrows_kernel(DevGeom g, FeatureArgs a, __nv_bfloat16* X) {
  extern __shared__ __align__(16) unsigned char xs[];
  const int d_in = a.d_in, ss = stage_stride(d_in);
  __nv_bfloat16* rows = reinterpret_cast<__nv_bfloat16*>(xs);
  for (long long r0 = (long long)blockIdx.x * kRowsPerBlock; r0 < a.n; r0 += (long long)gridDim.x * kRowsPerBlock) {
    __nv_bfloat16* row = rows + (size_t)threadIdx.x * ss;
    for (int k = 0; k < d_in / 2; ++k) reinterpret_cast<uint32_t*>(row)[k] = 0u;
    const long long i = r0 + threadIdx.x;
    if (i < a.n && !a.status[i]) {
      auto put = [row](int k, float v) { row[k] = __float2bfloat16_rn(v); };
      if (a.values_f64) feature_all<double>(g, a, i, put, nullptr);
      else feature_all<float>(g, a, i, put, nullptr);
    }
    __syncthreads();
    // the whole tile (rows past n are zeros), 16-byte pieces in core-matrix
    // order: piece t = ((row/8)·(d_in/8) + k/8)·8 + row%8
    const int chunks = d_in / 8;
    uint4* dst = reinterpret_cast<uint4*>(X + (size_t)r0 * d_in);
    for (int t = threadIdx.x; t < kRowsPerBlock * chunks; t += kRowsPerBlock) {
      const int r8 = t & 7, gc = t >> 3;
      const int r = (gc / chunks) * 8 + r8, c = gc % chunks;
      dst[t] = reinterpret_cast<const uint4*>(rows + (size_t)r * ss)[c];
    }
    __syncthreads();
  }
}

size_t xrows_smem(int d_in) { return (size_t)kRowsPerBlock * stage_stride(d_in) * 2; }

struct InferArgs {
  const __nv_bfloat16* X;  // feature rows, tiles of 128 rows in core-matrix order
  const int32_t* status;   // n
  long long n;
  int d_in, B;
  const __nv_bfloat16* W;  // layers' [out][in] bf16, one after another
  const float* bias;       // layers' biases (bf16-rounded values), one after another
  int n_out;
  float res_scale;         // network outputs are residuals in units of res_scale
  float clip;              // |residual| above clip is dropped (plain interpolation kept); 0: no clip
  void* values_out;        // n × B, float or double: += residual
  int out_f64;
};

struct InferSmem {
  size_t woff[4];
  int wstride[4];
  size_t bias_off, grp_off, grp_bytes, stage_off, act_off, out_off, total;
};

// weights and biases once per CTA, then per warp group: a staged tile of
// feature rows, the hidden activations and the output tile
__host__ __device__ inline InferSmem infer_smem(int d_in, int n_out, int groups) {
  const MlpLayout L = mlp_layout(d_in, n_out);
  InferSmem s;
  size_t o = 0;
  for (int l = 0; l < 4; ++l) {
    s.wstride[l] = L.in[l] + 8;
    s.woff[l] = o;
    o += (size_t)L.out[l] * s.wstride[l] * 2;
  }
  o = (o + 15) & ~size_t(15);
  s.bias_off = o;
  o += (size_t)(L.out[0] + L.out[1] + L.out[2] + L.out[3]) * 4;
  o = (o + 15) & ~size_t(15);
  s.grp_off = o;
  s.stage_off = 0;
  s.act_off = ((size_t)kInferRows * stage_stride(d_in) * 2 + 15) & ~size_t(15);
  s.out_off = s.act_off + (((size_t)kInferRows * act_stride() * 2 + 15) & ~size_t(15));
  s.grp_bytes = s.out_off + (((size_t)kInferRows * n_out * 4 + 15) & ~size_t(15));
  o += s.grp_bytes * groups;
  s.total = o;
  return s;
}

// One CTA per SM, blockDim = 256 × groups.  Each warp group streams 128-row
// tiles of X: layer 0 reads the staged tile, after which the group's
// cp.async prefetch of its next tile overlaps layers 1-3 and the residual
// add; the other group interleaves on the same SM.
__global__ void __launch_bounds__(kGroupThreads * kMaxGroups, 1)
mlp_infer_kernel(InferArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int d_in = a.d_in, n_out = a.n_out, B = a.B;
  const int groups = blockDim.x / kGroupThreads;
  const MlpLayout L = mlp_layout(d_in, n_out);
  const InferSmem S = infer_smem(d_in, n_out, groups);
  float* sb = reinterpret_cast<float*>(sm + S.bias_off);
  {
    long long src = 0;
    int bo = 0;
    for (int l = 0; l < 4; ++l) {
      __nv_bfloat16* dst = reinterpret_cast<__nv_bfloat16*>(sm + S.woff[l]);
      for (int t = threadIdx.x; t < L.out[l] * L.in[l]; t += blockDim.x)
        dst[(size_t)(t / L.in[l]) * S.wstride[l] + t % L.in[l]] = a.W[src + t];
      for (int t = threadIdx.x; t < L.out[l]; t += blockDim.x) sb[bo + t] = a.bias[bo + t];
      src += (long long)L.out[l] * L.in[l];
      bo += L.out[l];
    }
  }
  const __nv_bfloat16* W0 = reinterpret_cast<const __nv_bfloat16*>(sm + S.woff[0]);
  const __nv_bfloat16* W1 = reinterpret_cast<const __nv_bfloat16*>(sm + S.woff[1]);
  const __nv_bfloat16* W2 = reinterpret_cast<const __nv_bfloat16*>(sm + S.woff[2]);
  const __nv_bfloat16* W3 = reinterpret_cast<const __nv_bfloat16*>(sm + S.woff[3]);
  const float* b1 = sb + L.out[0];
  const float* b2 = b1 + L.out[1];
  const float* b3 = b2 + L.out[2];
  const int grp = threadIdx.x / kGroupThreads, gt = threadIdx.x % kGroupThreads;
  const int lane = gt & 31, row0 = (gt >> 5) * 16;
  unsigned char* gbase = sm + S.grp_off + S.grp_bytes * grp;
  __nv_bfloat16* stage = reinterpret_cast<__nv_bfloat16*>(gbase + S.stage_off);
  __nv_bfloat16* act = reinterpret_cast<__nv_bfloat16*>(gbase + S.act_off);
  float* out_tile = reinterpret_cast<float*>(gbase + S.out_off);
  const int ss = stage_stride(d_in), as = act_stride(), chunks = d_in / 8;
  const long long n_tiles = (a.n + kInferRows - 1) / kInferRows;
  const long long step = (long long)gridDim.x * groups;
  // rows past n are zero-filled with plain stores, the rest copied by cp.async
  auto stage_tile = [&](long long tile) {
    for (int t = gt; t < kInferRows * chunks; t += kGroupThreads) {
      const int r = t / chunks, c = t % chunks;
      __nv_bfloat16* d = stage + (size_t)r * ss + 8 * c;
      cp_async16(smem_u32(d), a.X + (size_t)tile * kInferRows * d_in + (((r >> 3) * chunks + c) << 6) + ((r & 7) << 3));
    }
    cp_async_commit();
  };
  long long tile = (long long)blockIdx.x * groups + grp;
  if (tile < n_tiles) stage_tile(tile);
  __syncthreads();  // weights and biases staged
  for (; tile < n_tiles; tile += step) {
    cp_async_wait_all();
    group_sync(grp);  // the whole staged tile is visible
    warp_layer<16, true>(W0, L.in[0], S.wstride[0], sb, stage, ss, act, as, row0, lane, nullptr, 0, 0);
    group_sync(grp);  // every warp is done with the staged tile
    if (tile + step < n_tiles) stage_tile(tile + step);
    warp_layer<16, true>(W1, L.in[1], S.wstride[1], b1, act, as, act, as, row0, lane, nullptr, 0, 0);
    warp_layer<16, true>(W2, L.in[2], S.wstride[2], b2, act, as, act, as, row0, lane, nullptr, 0, 0);
    for (int c = 0; c < n_out; c += 8)
      warp_layer<1, false>(W3 + (size_t)c * S.wstride[3], L.in[3], S.wstride[3], b3 + c, act, as, nullptr, 0, row0,
                           lane, out_tile + c, n_out, n_out - c);
    // each warp adds the residuals of its own 16 rows
    for (int t = lane; t < 16 * B; t += 32) {
      const int r = row0 + t / B, b = t % B;
      const long long i = tile * kInferRows + r;
      if (i >= a.n || a.status[i]) continue;
      const float res = out_tile[r * n_out + b] * a.res_scale;
      if (a.clip > 0.f && !(fabsf(res) <= a.clip)) continue;
      if (a.out_f64) static_cast<double*>(a.values_out)[i * B + b] += (double)res;
      else static_cast<float*>(a.values_out)[i * B + b] += res;
    }
    __syncwarp();
  }
  cp_async_wait_all();
}

// ---------------------------------------------------------------------------
// inference on tcgen05: accumulators in tensor memory
// ---------------------------------------------------------------------------
// Per CTA four slots of 4 warps, each taking 128-q tiles on its own: the
// tile's feature rows arrive by one bulk copy (cp.async.bulk, completion on
// an mbarrier) already in the canonical K-major core-matrix layout; for
// every layer one elected thread issues K/16 tcgen05.mma (M 128, N 128 or
// 16, bf16 × bf16 → FP32 in tensor memory, 128 columns per slot) and
// commits them to the slot's mbarrier; the slot's 128 threads then read
// their row of the accumulator (tcgen05.ld 32x32b, warp w owns lanes
// 32(w mod 4)…), add the bias, apply GELU and write the bf16 row back into
// the slot's one activation buffer (the MMA has finished reading it), in
// core-matrix order, as the next layer's A operand.  While one slot runs its
// epilogue the other slots' MMAs keep the tensor core busy.  The next tile's
// bulk copy is issued as soon as layer 3 has read the buffer.
// Every wait is bounded (about a second of clock cycles): on expiry the slot
// records BRX_ERR_TIMEOUT, leaves its loop together (barrier with an AND
// reduction), waits for its own copy in flight and the CTA frees its tensor
// memory.
constexpr int kTcSlots = 4;
constexpr int kTcThreads = 128 * kTcSlots;
constexpr int kTcCols = 128 * kTcSlots;        // tensor-memory columns per CTA (all 512)
constexpr long long kSpinCycles = 2000000000LL;

struct TcSmem {
  size_t w_off[4];
  int n_rows[4];   // output rows of each layer (the last padded to 16)
  size_t w_bytes, bias_off, slot_off, buf_bytes, mbar_off, tmem_off, total;
};

__host__ __device__ inline int tc_out_pad(int n_out) { return (n_out + 15) / 16 * 16; }

__host__ __device__ inline TcSmem tc_smem(int d_in, int n_out) {
  TcSmem S;
  const int K[4] = {d_in, kWidth, kWidth, kWidth};
  const int N[4] = {kWidth, kWidth, kWidth, tc_out_pad(n_out)};
  size_t o = 0;
  for (int l = 0; l < 4; ++l) {
    S.w_off[l] = o;
    S.n_rows[l] = N[l];
    o += (size_t)N[l] * K[l] * 2;
  }
  S.w_bytes = o;
  o = (o + 127) & ~size_t(127);
  S.bias_off = o;
  o += (size_t)(3 * kWidth + tc_out_pad(n_out)) * 4;
  o = (o + 127) & ~size_t(127);
  S.slot_off = o;
  S.buf_bytes = (size_t)kInferRows * (d_in > kWidth ? d_in : kWidth) * 2;
  o += S.buf_bytes * kTcSlots;
  S.mbar_off = o;
  o += 8 * 2 * kTcSlots;
  S.tmem_off = o;
  o += 16;
  S.total = o;
  return S;
}

// shared-memory matrix descriptor: K-major, no swizzle; lbo = byte distance
// of core matrices adjacent along K, sbo = along M / N
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}
// instruction descriptor, kind::f16: FP32 accumulator, bf16 A and B, both K-major
__device__ __forceinline__ uint32_t tc_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t phase) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(mbar), "r"(phase)
      : "memory");
  return done != 0;
}
// bounded wait for the completion of phase `phase`
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase, long long limit = kSpinCycles) {
  const long long t0 = clock64();
  while (!mbar_try(mbar, phase))
    if (clock64() - t0 > limit) return false;
  return true;
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(mbar) : "memory");
}
// BRX_FLAG_TEST_TIMEOUT: about a millisecond on a barrier nothing completes
constexpr long long kTcStallCycles = 2000000LL;
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}
// AND of pred over the slot's 128 threads (named barrier 1 + slot)
__device__ __forceinline__ bool slot_all(int slot, bool pred) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.b32 p, %1, 0;\n"
      " barrier.cta.red.and.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)pred), "r"(1 + slot), "n"(128)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

struct TcArgs {
  const __nv_bfloat16* X;   // tiles of 128 feature rows, core-matrix order
  const int32_t* status;
  long long n;
  int d_in, n_out, B;
  const uint4* Wt;          // the four layers' weights, core-matrix order (layer 3 padded to 16 rows)
  const float* bias;        // 3·128 + pad(n_out) biases (bf16-rounded values)
  float res_scale, clip;
  void* values_out;
  int out_f64;
  ErrorWord* err;
  int stall;  // BRX_FLAG_TEST_TIMEOUT: each slot's first wait for its rows never completes
};

__global__ void __launch_bounds__(kTcThreads, 1) mlp_infer_tc_kernel(TcArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  const TcSmem S = tc_smem(a.d_in, a.n_out);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int slot = tid / 128, st = tid % 128, wq = warp & 3;
  float* sb = reinterpret_cast<float*>(sm + S.bias_off);
  for (int i = tid; i < (int)(S.w_bytes / 16); i += kTcThreads) reinterpret_cast<uint4*>(sm)[i] = a.Wt[i];
  for (int i = tid; i < 3 * kWidth + tc_out_pad(a.n_out); i += kTcThreads) sb[i] = a.bias[i];
  const uint32_t mbar_mma = smem_u32(sm + S.mbar_off) + 16 * slot;
  const uint32_t mbar_x = mbar_mma + 8;
  // s_fail[slot]: the slot's issuer gave up waiting for its rows and
  // released the slot's MMA barrier without issuing; s_stall: a barrier
  // nothing completes (BRX_FLAG_TEST_TIMEOUT)
  __shared__ int s_fail[kTcSlots];
  __shared__ __align__(8) unsigned long long s_stall;
  if (tid == 0) {
    for (int s = 0; s < kTcSlots; ++s) {
      mbar_init(smem_u32(sm + S.mbar_off) + 16 * s, 1);
      mbar_init(smem_u32(sm + S.mbar_off) + 16 * s + 8, 1);
      s_fail[s] = 0;
    }
    mbar_init(smem_u32(&s_stall), 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(sm + S.tmem_off)),
                 "n"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  fence_proxy_async();  // weights written by this CTA are read by the tensor core
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *reinterpret_cast<volatile uint32_t*>(sm + S.tmem_off);
  const uint32_t tmem_d = tmem_base + 128 * slot;
  unsigned char* buf = sm + S.slot_off + S.buf_bytes * slot;
  const int B = a.B;
  const long long n_tiles = (a.n + kInferRows - 1) / kInferRows;
  const long long step = (long long)gridDim.x * kTcSlots;
  const uint32_t tile_bytes = (uint32_t)kInferRows * a.d_in * 2;
  const bool issuer = st == 0;
  uint32_t ph_mma = 0, ph_x = 0;
  bool x_pending = false, mma_pending = false, stall = a.stall != 0;
  long long tile = (long long)blockIdx.x * kTcSlots + slot;
  if (issuer && tile < n_tiles) {
    mbar_expect_tx(mbar_x, tile_bytes);
    bulk_load(smem_u32(buf), a.X + (size_t)tile * kInferRows * a.d_in, tile_bytes, mbar_x);
    x_pending = true;
  }
  bool ok = true;
  const int row = wq * 32 + lane;
  const uint32_t taddr = tmem_d + ((uint32_t)(wq * 32) << 16);
  for (; tile < n_tiles && ok; tile += step) {
    for (int l = 0; l < 4 && ok; ++l) {
      const int K = l == 0 ? a.d_in : kWidth, N = S.n_rows[l];
      bool good = true;
      if (issuer) {
        if (l == 0) {
          if (stall) {
            // test of the error path: the tile's rows stay in flight and
            // are drained at exit
            good = mbar_wait(smem_u32(&s_stall), 0, kTcStallCycles);
            stall = false;
          } else {
            good = mbar_wait(mbar_x, ph_x);
          }
          if (good) {
            ph_x ^= 1;
            x_pending = false;
          }
        }
        tc_fence_after();
        if (good) {
          const uint32_t a0 = smem_u32(buf), b0 = smem_u32(sm + S.w_off[l]);
          const uint32_t idesc = tc_idesc(kInferRows, N);
          for (int k = 0; k < K / 16; ++k)
            tc_mma(tmem_d, tc_desc(a0 + 256 * k, 128, 16 * K), tc_desc(b0 + 256 * k, 128, 16 * K), idesc, k > 0);
          tc_commit(mbar_mma);
        } else {
          // nothing to compute: release the slot's threads waiting below
          s_fail[slot] = 1;
          mbar_arrive(mbar_mma);
        }
      }
      const bool done = mbar_wait(mbar_mma, ph_mma);
      if (done) ph_mma ^= 1;
      else mma_pending = true;  // an MMA may still write tensor memory
      good = done && !*reinterpret_cast<volatile int*>(&s_fail[slot]);
      tc_fence_after();
      if (l == 3 && issuer && good && tile + step < n_tiles) {
        // layer 3 has read the buffer: the next tile's rows go there now
        mbar_expect_tx(mbar_x, tile_bytes);
        bulk_load(smem_u32(buf), a.X + (size_t)(tile + step) * kInferRows * a.d_in, tile_bytes, mbar_x);
        x_pending = true;
      }
      if (good) {
        if (l < 3) {
          const float* bl = sb + kWidth * l;
#pragma unroll 1
          for (int c = 0; c < kWidth / 32; ++c) {
            float v[32];
            tmem_ld32(taddr + 32 * c, v);
            uint32_t pk[16];
#pragma unroll
            for (int j = 0; j < 16; ++j)
              pk[j] = pack_bf16(gelu_fast(v[2 * j] + bl[32 * c + 2 * j]),
                                gelu_fast(v[2 * j + 1] + bl[32 * c + 2 * j + 1]));
            // row `row`, K-groups 4c … 4c+3 of a 128-wide K-major operand
            unsigned char* dst = buf + (size_t)(((row >> 3) * (kWidth / 8) + 4 * c) * 128 + (row & 7) * 16);
#pragma unroll
            for (int q = 0; q < 4; ++q)
              *reinterpret_cast<uint4*>(dst + 128 * q) = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
          }
          fence_proxy_async();
        } else {
          float v[16];
          tmem_ld16(taddr, v);
          const long long i = tile * kInferRows + row;
          if (i < a.n && !a.status[i]) {
            const float* bl = sb + 3 * kWidth;
            for (int b = 0; b < B && b < 16; ++b) {
              const float res = (v[b] + bl[b]) * a.res_scale;
              if (a.clip > 0.f && !(fabsf(res) <= a.clip)) continue;
              if (a.out_f64) static_cast<double*>(a.values_out)[i * B + b] += (double)res;
              else static_cast<float*>(a.values_out)[i * B + b] += res;
            }
          }
        }
      }
      tc_fence_before();
      ok = slot_all(slot, good);
    }
  }
  if (!ok && st == 0) {
    atomicOr(&a.err->flags, 1 << BRX_ERR_TIMEOUT);
    atomicAdd(&a.err->count, 1);
  }
  // no copy may land and no MMA may write tensor memory after exit
  if (issuer && x_pending) mbar_wait(mbar_x, ph_x);
  if (issuer && mma_pending) mbar_wait(mbar_mma, ph_mma);
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem_base), "n"(kTcCols) : "memory");
  }
}

}  // namespace brx

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace brx_detail;

namespace {

// q per sub-chunk of the residual: 2^19 feature rows of ≤ 160 bytes stay in
// the 129 MB L2 between the feature and network kernels
constexpr long long kResidualSub = 1LL << 19;

bool mlp_dims_ok(const brx_mlp_dims* d) {
  return d && d->d_in >= 16 && d->d_in % 16 == 0 && d->d_in <= 512 && d->n_out >= 8 && d->n_out % 8 == 0 &&
         d->n_out <= 64 && d->n_modes >= 1 && d->n_modes <= d->n_out && (d->flags & ~BRX_MLP_FP32) == 0;
}

int feature_cols(int B) { return 16 + 9 * B; }

brx::FeatureArgs feature_args(const brx_handle* h, const double* q_ir, const int32_t* node, const int32_t* nw,
                              const int32_t* vidx, const double* w, const int32_t* status, long long n, int d_in,
                              float omega_scale) {
  brx::FeatureArgs a{};
  a.q_ir = q_ir;
  a.node = node;
  a.nw = nw;
  a.vidx = vidx;
  a.w = w;
  a.status = status;
  a.n = n;
  a.values = h->vals.data.p;
  a.values_f64 = h->vals.store == brx::ST_F64;
  a.B = h->vals.B;
  a.d_in = d_in;
  a.inv_omega = 1.f / omega_scale;
  return a;
}

brx_status check_model_fits(brx_handle* h, const brx_mlp_dims* d) {
  if (!mlp_dims_ok(d)) return fail(h, BRX_ERR_INVALID_ARGUMENT, "invalid residual model dimensions");
  if (!h->filled) return fail(h, BRX_ERR_NOT_FILLED, "The interpolation data must be filled before interpolating.");
  if (h->vals.s != 1 || h->vals.cplx || h->vals.B != d->n_modes)
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "the residual model needs one real eigenvalue per mode");
  if (d->d_in < feature_cols(h->vals.B))
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "d_in is too small for the feature row");
  if (brx::infer_smem(d->d_in, d->n_out, 1).total > h->smem_optin)
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "the residual model does not fit in shared memory");
  return BRX_OK;
}

}  // namespace

extern "C" {

int64_t brx_mlp_param_count(const brx_mlp_dims* d) {
  if (!mlp_dims_ok(d)) return -1;
  return brx::mlp_layout(d->d_in, d->n_out).total;
}

int64_t brx_mlp_workspace_floats(const brx_mlp_dims* d, int64_t batch) {
  if (!mlp_dims_ok(d) || batch < 1) return -1;
  return (int64_t)brx::mlp_workspace_floats(batch, d->n_out);
}

brx_status brx_mlp_features(brx_handle* h, const brx_locate_out* records, int64_t n, const brx_mlp_dims* d,
                            float omega_scale, float* X, float* base, void* stream) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (!records || !X || !base || n < 0 || !(omega_scale > 0.f))
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "features need records, X, base and a positive omega_scale");
  if (!records->q_ir || !records->node || !records->n_weights || !records->vertex || !records->weight ||
      !records->status)
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "every locate record array is needed for features");
  brx_status st = check_model_fits(h, d);
  if (st) return st;
  BRX_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : h->sc[0].stream;
  if (n == 0) return BRX_OK;
  brx::FeatureArgs a = feature_args(h, records->q_ir, records->node, records->n_weights, records->vertex,
                                    records->weight, records->status, n, d->d_in, omega_scale);
  long long blocks = (n + 127) / 128;
  if (blocks > (long long)h->num_sms * 16) blocks = (long long)h->num_sms * 16;
  brx::mlp_features_kernel<<<(unsigned)blocks, 128, 0, s>>>(h->g, a, X, base);
  ++h->launches;
  BRX_CUDA(h, cudaGetLastError());
  if (!stream) BRX_CUDA(h, cudaStreamSynchronize(s));
  return BRX_OK;
}

brx_status brx_mlp_train_step(const brx_mlp_dims* d, float* params, float* grads, float* adam_m, float* adam_v,
                              int32_t step, float lr, const float* X, const float* T, int64_t batch, float* workspace,
                              float* loss, void* stream) {
  if (!mlp_dims_ok(d) || !params || !grads || !X || !T || !workspace || !loss || batch < 1 || batch > (1LL << 24))
    return BRX_ERR_INVALID_ARGUMENT;
  if ((adam_m == nullptr) != (adam_v == nullptr) || (adam_m && step < 1)) return BRX_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const brx::Work w = brx::carve(workspace, batch, d->n_out);
  const int rnd = (d->flags & BRX_MLP_FP32) ? 0 : 1;
  brx::mlp_forward_train(d->d_in, d->n_out, rnd, params, X, batch, w, s);
  if (cudaMemsetAsync(loss, 0, sizeof(float), s) != cudaSuccess) return BRX_ERR_CUDA;
  brx::mse_grad_kernel<<<brx::elem_blocks(batch * d->n_out, 256), 256, 0, s>>>(w.Y, T, w.dY, batch, d->n_out,
                                                                              d->n_modes, loss);
  brx::mlp_backward(d->d_in, d->n_out, rnd, params, grads, X, batch, w, s);
  if (adam_m) {
    const long long np = brx::mlp_layout(d->d_in, d->n_out).total;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
    brx::adam_kernel<<<brx::elem_blocks(np, 256), 256, 0, s>>>(params, grads, adam_m, adam_v, np, lr, b1, b2, 1e-8f,
                                                               c1, c2);
  }
  return cudaGetLastError() == cudaSuccess ? BRX_OK : BRX_ERR_CUDA;
}

brx_status brx_mlp_forward(const brx_mlp_dims* d, const float* params, const float* X, int64_t batch, float* Y,
                           float* workspace, void* stream) {
  if (!mlp_dims_ok(d) || !params || !X || !Y || !workspace || batch < 1 || batch > (1LL << 24))
    return BRX_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const brx::Work w = brx::carve(workspace, batch, d->n_out);
  brx::mlp_forward_train(d->d_in, d->n_out, (d->flags & BRX_MLP_FP32) ? 0 : 1, params, X, batch, w, s);
  if (cudaMemcpyAsync(Y, w.Y, sizeof(float) * batch * d->n_out, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return BRX_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? BRX_OK : BRX_ERR_CUDA;
}

brx_status brx_set_residual_model(brx_handle* h, const brx_mlp_dims* d, const float* params, float omega_scale,
                                  float res_scale, float clip) {
  if (!h) return BRX_ERR_INVALID_ARGUMENT;
  if (!params) {
    h->mlp_on = false;
    return BRX_OK;
  }
  if (!(omega_scale > 0.f) || !(res_scale > 0.f) || !(clip >= 0.f))
    return fail(h, BRX_ERR_INVALID_ARGUMENT, "residual model scales must be positive");
  brx_status st = check_model_fits(h, d);
  if (st) return st;
  const brx::MlpLayout L = brx::mlp_layout(d->d_in, d->n_out);
  std::vector<__nv_bfloat16> W;
  std::vector<float> b;
  for (int l = 0; l < 4; ++l) {
    for (long long t = 0; t < (long long)L.out[l] * L.in[l]; ++t) W.push_back(__float2bfloat16_rn(params[L.W[l] + t]));
    for (int t = 0; t < L.out[l]; ++t) b.push_back(__bfloat162float(__float2bfloat16_rn(params[L.b[l] + t])));
  }
  BRX_CUDA(h, cudaSetDevice(h->device));
  BRX_CUDA(h, h->mlp_w.ensure(W.size() * sizeof(__nv_bfloat16)));
  BRX_CUDA(h, h->mlp_b.ensure(b.size() * sizeof(float)));
  BRX_CUDA(h, cudaMemcpy(h->mlp_w.p, W.data(), W.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice));
  BRX_CUDA(h, cudaMemcpy(h->mlp_b.p, b.data(), b.size() * sizeof(float), cudaMemcpyHostToDevice));
  // the tcgen05 kernel's operands: weights in core-matrix order (layer 3
  // padded to 16 rows), biases padded alike
  {
    const brx::TcSmem T = brx::tc_smem(d->d_in, d->n_out);
    const char* env = std::getenv("BRX_MLP_KERNEL");
    h->mlp_tc = T.total <= h->smem_optin && !(env && std::strcmp(env, "mma") == 0);
    if (h->mlp_tc) {
      std::vector<__nv_bfloat16> Wt(T.w_bytes / 2, __float2bfloat16_rn(0.f));
      for (int l = 0; l < 4; ++l) {
        const int K = L.in[l];
        for (int nrow = 0; nrow < L.out[l]; ++nrow)
          for (int k = 0; k < K; ++k)
            Wt[T.w_off[l] / 2 + ((size_t)(nrow >> 3) * (K / 8) + (k >> 3)) * 64 + (nrow & 7) * 8 + (k & 7)] =
                __float2bfloat16_rn(params[L.W[l] + (long long)nrow * K + k]);
      }
      std::vector<float> bt(3 * brx::kWidth + brx::tc_out_pad(d->n_out), 0.f);
      for (int t = 0; t < 3 * brx::kWidth + d->n_out; ++t) bt[t] = b[t];
      BRX_CUDA(h, h->mlp_wt.ensure(T.w_bytes));
      BRX_CUDA(h, h->mlp_bt.ensure(bt.size() * sizeof(float)));
      BRX_CUDA(h, cudaMemcpy(h->mlp_wt.p, Wt.data(), T.w_bytes, cudaMemcpyHostToDevice));
      BRX_CUDA(h, cudaMemcpy(h->mlp_bt.p, bt.data(), bt.size() * sizeof(float), cudaMemcpyHostToDevice));
      BRX_CUDA(h, cudaFuncSetAttribute(brx::mlp_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)T.total));
    }
  }
  const int groups = brx::infer_smem(d->d_in, d->n_out, 2).total <= h->smem_optin ? 2 : 1;
  const size_t smem = brx::infer_smem(d->d_in, d->n_out, groups).total;
  BRX_CUDA(h, cudaFuncSetAttribute(brx::mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  BRX_CUDA(h, cudaFuncSetAttribute(brx::mlp_xrows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)brx::xrows_smem(d->d_in)));
  BRX_CUDA(h, h->mlp_x.ensure((size_t)kResidualSub * d->d_in * sizeof(__nv_bfloat16)));
  h->mlp_groups = groups;
  h->mlp_dims = *d;
  h->mlp_omega_scale = omega_scale;
  h->mlp_res_scale = res_scale;
  h->mlp_clip = clip;
  h->mlp_on = true;
  return BRX_OK;
}

}  // extern "C"

namespace brx_detail {

int launch_residual(brx_handle* h, const Scratch& s, long long n, void* values_out, bool out_f32, cudaStream_t cs) {
  if (!h->mlp_on || n <= 0) return 0;
  const int d_in = h->mlp_dims.d_in, B = h->vals.B, groups = h->mlp_groups;
  const size_t smem = brx::infer_smem(d_in, h->mlp_dims.n_out, groups).total;
  const size_t out_row = (size_t)B * (out_f32 ? 4 : 8);
  __nv_bfloat16* X = static_cast<__nv_bfloat16*>(h->mlp_x.p);
  int launches = 0;
  // sub-chunks whose feature rows stay in L2 between the two kernels
  for (long long off = 0; off < n; off += kResidualSub) {
    const long long m = std::min<long long>(kResidualSub, n - off);
    brx::FeatureArgs f = feature_args(h, s.r.q_ir + 3 * off, s.r.node + 2 * off, s.r.nw + off,
                                      s.r.vidx + 8 * off, s.r.w + 8 * off, s.r.status + off, m, d_in,
                                      h->mlp_omega_scale);
    f.w32 = s.r.w32 + 8 * off;
    const long long blocks = std::min<long long>((m + brx::kRowsPerBlock - 1) / brx::kRowsPerBlock,
                                                 (long long)h->num_sms * 8);
    brx::mlp_xrows_kernel<<<(unsigned)blocks, brx::kRowsPerBlock, brx::xrows_smem(d_in), cs>>>(h->g, f, X);
    brx::InferArgs a{};
    a.X = X;
    a.status = s.r.status + off;
    a.n = m;
    a.d_in = d_in;
    a.B = B;
    a.W = static_cast<const __nv_bfloat16*>(h->mlp_w.p);
    a.bias = static_cast<const float*>(h->mlp_b.p);
    a.n_out = h->mlp_dims.n_out;
    a.res_scale = h->mlp_res_scale;
    a.clip = h->mlp_clip;
    a.values_out = static_cast<char*>(values_out) + out_row * (size_t)off;
    a.out_f64 = !out_f32;
    const long long tiles = (m + brx::kInferRows - 1) / brx::kInferRows;
    if (h->mlp_tc) {
      brx::TcArgs t{};
      t.X = X;
      t.status = a.status;
      t.n = m;
      t.d_in = d_in;
      t.n_out = a.n_out;
      t.B = B;
      t.Wt = static_cast<const uint4*>(h->mlp_wt.p);
      t.bias = static_cast<const float*>(h->mlp_bt.p);
      t.res_scale = a.res_scale;
      t.clip = a.clip;
      t.values_out = a.values_out;
      t.out_f64 = a.out_f64;
      t.err = h->err;
      t.stall = h->test_stall ? 1 : 0;
      const long long grid = std::min<long long>((tiles + brx::kTcSlots - 1) / brx::kTcSlots, (long long)h->num_sms);
      brx::mlp_infer_tc_kernel<<<(unsigned)grid, brx::kTcThreads, brx::tc_smem(d_in, a.n_out).total, cs>>>(t);
    } else {
      const long long grid = std::min<long long>((tiles + groups - 1) / groups, (long long)h->num_sms);
      brx::mlp_infer_kernel<<<(unsigned)grid, brx::kGroupThreads * groups, smem, cs>>>(a);
    }
    launches += 2;
  }
  return launches;
}

}  // namespace brx_detail
