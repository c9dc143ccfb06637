// K3+K4: gather and weighted sum of vertex data, fused with the rotation
// back by R (and the Γ permutation/phase for phonon eigenvectors).
//
// One CTA handles a tile of q (in node-sorted order so that neighbouring q
// share vertex rows); threads map to (q, branch, element-chunk).  The
// interpolated rows of the tile accumulate in registers, land in shared
// memory, and are rotated and written out from there so that global stores
// are coalesced rows of the output.
//
// Reference: Interpolator::interpolate_at_mix (src/interpolator_at.tpp:92-127),
// antiphase (src/utilities.tpp:567-578), PermutationTable::safe_get
// (src/permutation_table.hpp:193-198), rip_real / rip_recip / rip_axial
// (src/interpolator_{real,recip,axial}.tpp) and rip_gamma_complex
// (src/interpolator_gamma.tpp:49-139).
#include <cuda_bf16.h>

#include "brx_kernels.h"

namespace brx {

constexpr int kChunkMax = 24;  // elements accumulated per thread

template <typename T>
struct Ar;
template <>
struct Ar<double> {  // FP64: explicitly rounded, never contracted
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
};
template <>
struct Ar<float> {  // FP32: the compiler may fuse into FMAs
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
  static __device__ __forceinline__ float add(float a, float b) { return a + b; }
  static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
};

template <typename St, bool CPLX>
struct Ld;
template <>
struct Ld<double, false> {
  template <typename A>
  static __device__ __forceinline__ void get(const void* b, long long i, A& re, A& im) {
    re = (A)__ldg(reinterpret_cast<const double*>(b) + i);
    im = 0;
  }
};
template <>
struct Ld<double, true> {
  template <typename A>
  static __device__ __forceinline__ void get(const void* b, long long i, A& re, A& im) {
    double2 v = __ldg(reinterpret_cast<const double2*>(b) + i);
    re = (A)v.x;
    im = (A)v.y;
  }
};
template <>
struct Ld<float, false> {
  template <typename A>
  static __device__ __forceinline__ void get(const void* b, long long i, A& re, A& im) {
    re = (A)__ldg(reinterpret_cast<const float*>(b) + i);
    im = 0;
  }
};
template <>
struct Ld<float, true> {
  template <typename A>
  static __device__ __forceinline__ void get(const void* b, long long i, A& re, A& im) {
    float2 v = __ldg(reinterpret_cast<const float2*>(b) + i);
    re = (A)v.x;
    im = (A)v.y;
  }
};
template <>
struct Ld<__nv_bfloat16, false> {
  template <typename A>
  static __device__ __forceinline__ void get(const void* b, long long i, A& re, A& im) {
    re = (A)__bfloat162float(reinterpret_cast<const __nv_bfloat16*>(b)[i]);
    im = 0;
  }
};
template <>
struct Ld<__nv_bfloat16, true> {
  template <typename A>
  static __device__ __forceinline__ void get(const void* b, long long i, A& re, A& im) {
    __nv_bfloat162 v = reinterpret_cast<const __nv_bfloat162*>(b)[i];
    float2 f = __bfloat1622float2(v);
    re = (A)f.x;
    im = (A)f.y;
  }
};

__device__ __forceinline__ int perm_lookup(const GatherParams& p, long long i, long long j) {
  if (p.n_keys == 0 || i == j) return -1;
  long long key = i * p.n_vertices + j, lo = 0, hi = p.n_keys;
  while (lo < hi) {
    long long mid = (lo + hi) >> 1;
    if (__ldg(p.keys + mid) < key) lo = mid + 1; else hi = mid;
  }
  if (lo < p.n_keys && __ldg(p.keys + lo) == key) {
    int id = __ldg(p.perm_ids + lo);
    if (id >= 0 && id < p.n_perms) return id;
  }
  return -1;
}

struct TileLayout {
  size_t q, nw, vi, pid, rot, ident, w, ph, R, out, total;
};

template <typename Acc>
__host__ __device__ inline TileLayout tile_layout(int QT, int B, int s, int comps, int n_atoms, bool gamma) {
  TileLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = (o + 15) & ~size_t(15);
    o = at + bytes;
    return at;
  };
  L.q = take(sizeof(long long) * QT);
  L.nw = take(sizeof(int) * QT);
  L.vi = take(sizeof(int) * 8 * QT);
  L.pid = take(sizeof(int) * 8 * QT);
  L.rot = take(sizeof(int) * 2 * QT);
  L.ident = take(sizeof(int) * QT);
  L.w = take(sizeof(Acc) * 8 * QT);
  L.ph = take(gamma ? sizeof(Acc) * 4 * (size_t)n_atoms * QT : 0);
  L.R = take(sizeof(Acc) * 18 * QT);
  L.out = take(sizeof(Acc) * (size_t)QT * B * s * comps);
  L.total = (o + 15) & ~size_t(15);
  return L;
}

template <typename Acc, typename St, bool CPLX, typename Out>
__global__ void __launch_bounds__(kGatherThreads)
gather_kernel(GatherParams p) {
  using A = Ar<Acc>;
  extern __shared__ __align__(16) unsigned char sm[];
  const int QT = p.q_tile, B = p.B, s = p.s, NC = p.n_chunks, CL = p.chunk_len;
  constexpr int comps = CPLX ? 2 : 1;
  const bool gamma = p.rot_mode == ROT_GAMMA;
  const int n_atoms_tab = gamma ? p.nvec : 0;
  const TileLayout L = tile_layout<Acc>(QT, B, s, comps, n_atoms_tab, gamma);
  long long* s_q = reinterpret_cast<long long*>(sm + L.q);
  int* s_nw = reinterpret_cast<int*>(sm + L.nw);
  int* s_vi = reinterpret_cast<int*>(sm + L.vi);
  int* s_pid = reinterpret_cast<int*>(sm + L.pid);
  int* s_rot = reinterpret_cast<int*>(sm + L.rot);
  int* s_id = reinterpret_cast<int*>(sm + L.ident);
  Acc* s_w = reinterpret_cast<Acc*>(sm + L.w);
  Acc* s_ph = reinterpret_cast<Acc*>(sm + L.ph);
  Acc* s_R = reinterpret_cast<Acc*>(sm + L.R);
  Acc* s_out = reinterpret_cast<Acc*>(sm + L.out);
  const long long n_tiles = (p.n + QT - 1) / QT;

  for (long long tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    // ---- phase A: records of the tile ----
    for (int t = threadIdx.x; t < QT; t += blockDim.x) {
      long long j = tile * QT + t;
      long long qi = -1;
      int nw = 0;
      if (j < p.n) {
        long long c = p.order ? (long long)p.order[j] : j;
        if (p.status[c] == 0) { qi = c; nw = p.nw[c]; }
      }
      s_q[t] = qi;
      s_nw[t] = nw;
      for (int x = 0; x < 8; ++x) {
        s_vi[8 * t + x] = qi >= 0 ? p.vidx[8 * qi + x] : 0;
        s_w[8 * t + x] = qi >= 0 ? (Acc)p.w[8 * qi + x] : (Acc)0;
      }
      int r0 = 0, r1 = 0;
      if (qi >= 0 && p.rot_mode != ROT_NONE) { r0 = p.rot[2 * qi]; r1 = p.rot[2 * qi + 1]; }
      s_rot[2 * t] = r0;
      s_rot[2 * t + 1] = r1;
      int ident = 1;
      if (p.rot_mode != ROT_NONE && qi >= 0) {
        const int32_t* W = p.ops + 9 * r0;
        ident = (W[0] == 1 && W[1] == 0 && W[2] == 0 && W[3] == 0 && W[4] == 1 && W[5] == 0 && W[6] == 0 &&
                 W[7] == 0 && W[8] == 1);
        // R (slot 0..8) and R⁻¹ (slot 9..17) in the arithmetic type
        for (int e = 0; e < 9; ++e) {
          if (gamma && p.gamma_cart) {
            s_R[18 * t + e] = (Acc)p.rot_cart[9 * r0 + e];
            s_R[18 * t + 9 + e] = (Acc)p.rot_cart[9 * r1 + e];
          } else {
            s_R[18 * t + e] = (Acc)p.ops[9 * r0 + e];
            s_R[18 * t + 9 + e] = (Acc)p.ops[9 * r1 + e];
          }
        }
      }
      s_id[t] = ident;
    }
    __syncthreads();
    // permutation ids per (q, vertex); Γ phases per (q, atom)
    for (int it = threadIdx.x; it < 8 * QT; it += blockDim.x) {
      int t = it >> 3, x = it & 7;
      s_pid[it] = (s_q[t] >= 0 && x < s_nw[t]) ? perm_lookup(p, s_vi[8 * t], s_vi[it]) : -1;
    }
    if (gamma) {
      for (int it = threadIdx.x; it < QT * n_atoms_tab; it += blockDim.x) {
        int t = it / n_atoms_tab, k = it % n_atoms_tab;
        long long qi = s_q[t];
        Acc v[4] = {1, 0, 1, 0};
        if (qi >= 0) {
          const double q0 = p.q_ir[3 * qi], q1 = p.q_ir[3 * qi + 1], q2 = p.q_ir[3 * qi + 2];
          for (int h = 0; h < 2; ++h) {
            int r = s_rot[2 * t + h];
            const double* d = p.gamma_vectors + 3 * __ldg(p.gamma_vidx + k * p.n_ops + r);
            double dq = 0.0;
            dq = __dadd_rn(dq, __dmul_rn(q0, d[0]));
            dq = __dadd_rn(dq, __dmul_rn(q1, d[1]));
            dq = __dadd_rn(dq, __dmul_rn(q2, d[2]));
            double frac = dq - rint(dq);  // exact: e^{2πi n} = 1
            double sn, cs;
            sincospi(2.0 * frac, &sn, &cs);
            v[2 * h] = (Acc)cs;
            v[2 * h + 1] = (Acc)sn;
          }
        }
        // slots: R phase (re, im), R⁻¹ phase (re, im)
        for (int e = 0; e < 4; ++e) s_ph[4 * it + e] = v[e];
      }
    }
    __syncthreads();

    // ---- phase B: gather into the shared tile ----
    const int items = QT * B * NC;
    const int rounds = (items + blockDim.x - 1) / blockDim.x;
    for (int rd = 0; rd < rounds; ++rd) {
      const int item = rd * blockDim.x + threadIdx.x;
      const bool valid = item < items;
      const int t = valid ? item / (B * NC) : 0;
      const int rem = valid ? item % (B * NC) : 0;
      const int b = rem / NC, c = rem % NC;
      const long long qi = valid ? s_q[t] : -1;
      const int nw = qi >= 0 ? s_nw[t] : 0;
      const int e0 = c * CL;
      const int e1 = min(s, e0 + CL);
      Acc ar[kChunkMax], ai[kChunkMax];
#pragma unroll
      for (int i = 0; i < kChunkMax; ++i) { ar[i] = 0; ai[i] = 0; }
      const long long piv = s_vi[8 * t];
      for (int x = 0; x < 8; ++x) {
        const bool act = x < nw;
        if (!act && NC == 1) break;
        const long long v = act ? s_vi[8 * t + x] : 0;
        int pb = b;
        if (act) {
          int pid = s_pid[8 * t + x];
          if (pid >= 0) pb = __ldg(p.perms + (long long)pid * B + b);
        }
        Acc er = 1, ei = 0;
        if (CPLX && p.phase_allowed && x > 0) {
          Acc rdot = 0, idot = 0;
          if (act) {
            const long long r0 = (piv * B + b) * s, r1 = (v * B + pb) * s;
            for (int e = e0; e < e1; ++e) {
              Acc xr, xi, yr, yi;
              Ld<St, CPLX>::get(p.data, r0 + e, xr, xi);
              Ld<St, CPLX>::get(p.data, r1 + e, yr, yi);
              rdot = A::add(rdot, A::add(A::mul(xr, yr), A::mul(xi, yi)));
              idot = A::add(idot, A::sub(A::mul(xr, yi), A::mul(xi, yr)));
            }
          }
          if (NC > 1) {
            for (int off = 1; off < NC; off <<= 1) {
              rdot = A::add(rdot, __shfl_xor_sync(0xffffffffu, rdot, off));
              idot = A::add(idot, __shfl_xor_sync(0xffffffffu, idot, off));
            }
          }
          if (act) {
            Acc mag = sqrt(A::add(A::mul(rdot, rdot), A::mul(idot, idot)));
            if (mag > (Acc)0) {
              er = rdot / mag;
              ei = -(idot / mag);
            }
          }
        }
        if (act) {
          const Acc wx = s_w[8 * t + x];
          const Acc wr = A::mul(wx, er), wi = A::mul(wx, ei);
          const long long r1 = (v * B + pb) * s;
#pragma unroll
          for (int i = 0; i < kChunkMax; ++i) {
            if (e0 + i < e1) {
              Acc dr, di;
              Ld<St, CPLX>::get(p.data, r1 + e0 + i, dr, di);
              if (CPLX) {
                ar[i] = A::add(ar[i], A::sub(A::mul(wr, dr), A::mul(wi, di)));
                ai[i] = A::add(ai[i], A::add(A::mul(wr, di), A::mul(wi, dr)));
              } else {
                ar[i] = A::add(ar[i], A::mul(wx, dr));
              }
            }
          }
        }
      }
      if (valid) {
        Acc* dst = s_out + ((size_t)(t * B + b) * s) * comps;
#pragma unroll
        for (int i = 0; i < kChunkMax; ++i) {
          if (e0 + i < e1) {
            dst[(e0 + i) * comps] = ar[i];
            if (CPLX) dst[(e0 + i) * comps + 1] = ai[i];
          }
        }
      }
    }
    __syncthreads();

    // ---- phase C: rotate and store ----
    const int G = p.nsc + p.nvec + p.nmat;
    const int citems = QT * B * G;
    Out* out = reinterpret_cast<Out*>(p.out);
    for (int it = threadIdx.x; it < citems; it += blockDim.x) {
      const int t = it / (B * G);
      const int rem = it % (B * G);
      const int b = rem / G, g = rem % G;
      const long long qi = s_q[t];
      if (qi < 0) continue;
      const Acc* src = s_out + ((size_t)(t * B + b) * s) * comps;
      Out* dst = out + ((size_t)qi * B + b) * (size_t)s * comps;
      const bool rotate = p.rot_mode != ROT_NONE && (gamma || !s_id[t]);
      const Acc* R = s_R + 18 * t;
      const Acc* Ri = R + 9;
      if (g < p.nsc) {
        dst[g * comps] = (Out)src[g * comps];
        if (CPLX) dst[g * comps + 1] = (Out)src[g * comps + 1];
        continue;
      }
      if (g < p.nsc + p.nvec) {
        const int k = g - p.nsc;
        const int e = p.nsc + 3 * k;
        Acc vr[3], vi[3];
        for (int j = 0; j < 3; ++j) { vr[j] = src[(e + j) * comps]; vi[j] = CPLX ? src[(e + j) * comps + 1] : (Acc)0; }
        if (!rotate) {
          for (int j = 0; j < 3; ++j) {
            dst[(e + j) * comps] = (Out)vr[j];
            if (CPLX) dst[(e + j) * comps + 1] = (Out)vi[j];
          }
          continue;
        }
        // the 3×3 applied to this vector
        Acc M[9];
        Acc scale = 1;
        if (p.rot_mode == ROT_RECIP) {
          for (int a = 0; a < 3; ++a) for (int bb = 0; bb < 3; ++bb) M[3 * a + bb] = R[3 * bb + a];
        } else if (p.rot_mode == ROT_AXIAL) {
          for (int j = 0; j < 9; ++j) M[j] = Ri[j];
          scale = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) +
                  R[2] * (R[3] * R[7] - R[4] * R[6]);
        } else if (p.rot_mode == ROT_GAMMA) {
          for (int j = 0; j < 9; ++j) M[j] = Ri[j];
        } else {
          for (int j = 0; j < 9; ++j) M[j] = R[j];
        }
        Acc tr[3], ti[3];
        for (int a = 0; a < 3; ++a) {
          Acc sr = 0, si = 0;
          for (int kk = 0; kk < 3; ++kk) {
            sr = A::add(sr, A::mul(M[3 * a + kk], vr[kk]));
            if (CPLX) si = A::add(si, A::mul(M[3 * a + kk], vi[kk]));
          }
          tr[a] = sr;
          ti[a] = si;
        }
        int de = e;
        if (p.rot_mode == ROT_GAMMA) {
          const int r1 = s_rot[2 * t + 1];
          de = p.nsc + 3 * __ldg(p.gamma_F0 + k * p.n_ops + r1);
          const Acc pr = s_ph[4 * (t * n_atoms_tab + k) + 2], pi = s_ph[4 * (t * n_atoms_tab + k) + 3];
          for (int a = 0; a < 3; ++a) {
            Acc xr = A::sub(A::mul(pr, tr[a]), A::mul(pi, ti[a]));
            Acc xi = A::add(A::mul(pr, ti[a]), A::mul(pi, tr[a]));
            tr[a] = xr;
            ti[a] = xi;
          }
        } else if (p.rot_mode == ROT_AXIAL) {
          for (int a = 0; a < 3; ++a) { tr[a] = A::mul(scale, tr[a]); ti[a] = A::mul(scale, ti[a]); }
        }
        for (int a = 0; a < 3; ++a) {
          dst[(de + a) * comps] = (Out)tr[a];
          if (CPLX) dst[(de + a) * comps + 1] = (Out)ti[a];
        }
        continue;
      }
      // 3×3 matrices
      const int m = g - p.nsc - p.nvec;
      const int e = p.nsc + 3 * p.nvec + 9 * m;
      Acc Xr[9], Xi[9];
      for (int j = 0; j < 9; ++j) { Xr[j] = src[(e + j) * comps]; Xi[j] = CPLX ? src[(e + j) * comps + 1] : (Acc)0; }
      if (!rotate) {
        for (int j = 0; j < 9; ++j) {
          dst[(e + j) * comps] = (Out)Xr[j];
          if (CPLX) dst[(e + j) * comps + 1] = (Out)Xi[j];
        }
        continue;
      }
      Acc Lm[9], Rm[9];  // result = Lm · (X · Rm)
      if (p.rot_mode == ROT_RECIP) {
        for (int a = 0; a < 3; ++a) for (int bb = 0; bb < 3; ++bb) { Lm[3 * a + bb] = R[3 * bb + a]; Rm[3 * a + bb] = Ri[3 * bb + a]; }
      } else if (p.rot_mode == ROT_AXIAL) {
        for (int j = 0; j < 9; ++j) { Lm[j] = Ri[j]; Rm[j] = R[j]; }
      } else {
        for (int j = 0; j < 9; ++j) { Lm[j] = R[j]; Rm[j] = Ri[j]; }
      }
      Acc Tr[9], Ti[9], Yr[9], Yi[9];
      for (int a = 0; a < 3; ++a)
        for (int bb = 0; bb < 3; ++bb) {
          Acc sr = 0, si = 0;
          for (int kk = 0; kk < 3; ++kk) {
            sr = A::add(sr, A::mul(Xr[3 * a + kk], Rm[3 * kk + bb]));
            si = A::add(si, A::mul(Xi[3 * a + kk], Rm[3 * kk + bb]));
          }
          Tr[3 * a + bb] = sr;
          Ti[3 * a + bb] = si;
        }
      for (int a = 0; a < 3; ++a)
        for (int bb = 0; bb < 3; ++bb) {
          Acc sr = 0, si = 0;
          for (int kk = 0; kk < 3; ++kk) {
            sr = A::add(sr, A::mul(Lm[3 * a + kk], Tr[3 * kk + bb]));
            si = A::add(si, A::mul(Lm[3 * a + kk], Ti[3 * kk + bb]));
          }
          Yr[3 * a + bb] = sr;
          Yi[3 * a + bb] = si;
        }
      const int de = e;
      for (int j = 0; j < 9; ++j) {
        dst[(de + j) * comps] = (Out)Yr[j];
        if (CPLX) dst[(de + j) * comps + 1] = (Out)Yi[j];
      }
    }
    __syncthreads();
  }
}

template <typename Acc>
static size_t smem_for(const GatherParams& p, bool cplx, int qt) {
  const bool gamma = p.rot_mode == ROT_GAMMA;
  const int na = gamma ? p.nvec : 0;
  return tile_layout<Acc>(qt, p.B, p.s, cplx ? 2 : 1, na, gamma).total;
}

size_t gather_smem_bytes(const GatherParams& p, int store_kind, bool cplx, int q_tile) {
  return store_kind == ST_F64 ? smem_for<double>(p, cplx, q_tile) : smem_for<float>(p, cplx, q_tile);
}

int gather_pick_tile(const GatherParams& p, int store_kind, bool cplx, size_t smem_budget) {
  int qt = 64;
  while (qt > 1 && gather_smem_bytes(p, store_kind, cplx, qt) > smem_budget) qt >>= 1;
  return qt;
}

template <typename Acc, typename St, bool CPLX, typename Out>
static void launch_t(const GatherParams& p, int num_sms, cudaStream_t s) {
  size_t smem = gather_smem_bytes(p, std::is_same<Acc, double>::value ? ST_F64 : ST_F32, CPLX, p.q_tile);
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(gather_kernel<Acc, St, CPLX, Out>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    configured = true;
  }
  long long tiles = (p.n + p.q_tile - 1) / p.q_tile;
  int per_sm = (int)((200 * 1024) / (smem > 0 ? smem : 1));
  if (per_sm < 1) per_sm = 1;
  if (per_sm > 8) per_sm = 8;
  long long cap = (long long)num_sms * per_sm;
  long long grid = tiles < cap ? tiles : cap;
  if (grid < 1) grid = 1;
  gather_kernel<Acc, St, CPLX, Out><<<(unsigned)grid, kGatherThreads, smem, s>>>(p);
}

int launch_gather(const GatherParams& p, int store_kind, bool cplx, bool out_f32, int num_sms, size_t,
                  cudaStream_t s) {
  if (p.n <= 0) return 0;
#define BRX_DISPATCH(ACC, ST)                                                     \
  do {                                                                            \
    if (cplx) {                                                                   \
      if (out_f32) launch_t<ACC, ST, true, float>(p, num_sms, s);                 \
      else launch_t<ACC, ST, true, double>(p, num_sms, s);                        \
    } else {                                                                      \
      if (out_f32) launch_t<ACC, ST, false, float>(p, num_sms, s);                \
      else launch_t<ACC, ST, false, double>(p, num_sms, s);                       \
    }                                                                             \
  } while (0)
  switch (store_kind) {
    case ST_F64: BRX_DISPATCH(double, double); break;
    case ST_F32: BRX_DISPATCH(float, float); break;
    default: BRX_DISPATCH(float, __nv_bfloat16); break;
  }
#undef BRX_DISPATCH
  return 1;
}

// ---------------------------------------------------------------------------
// counting sort of q by trellis node (failed q go to the last bucket)
// ---------------------------------------------------------------------------
__global__ void node_hist_kernel(const int32_t* node, const int32_t* status, long long n, long long n_nodes,
                                 int32_t* counts) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long key = status[i] ? n_nodes : (long long)node[2 * i];
    atomicAdd(counts + key, 1);
  }
}

// single-CTA exclusive scan of counts[0..m) into counts, cursor copy in counts[m..2m)
__global__ void node_scan_kernel(int32_t* counts, long long m) {
  __shared__ long long part[1024];
  const int T = blockDim.x;
  long long per = (m + T - 1) / T;
  long long b = threadIdx.x * per, e = min(m, b + per);
  long long sum = 0;
  for (long long i = b; i < e; ++i) sum += counts[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long run = 0;
    for (int i = 0; i < T; ++i) { long long v = part[i]; part[i] = run; run += v; }
  }
  __syncthreads();
  long long run = part[threadIdx.x];
  for (long long i = b; i < e; ++i) {
    long long v = counts[i];
    counts[i] = (int32_t)run;
    counts[m + i] = (int32_t)run;
    run += v;
  }
}

__global__ void node_scatter_kernel(const int32_t* node, const int32_t* status, long long n, long long n_nodes,
                                    int32_t* cursor, int32_t* order) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long key = status[i] ? n_nodes : (long long)node[2 * i];
    int pos = atomicAdd(cursor + key, 1);
    order[pos] = (int32_t)i;
  }
}

size_t node_sort_scratch_ints(long long n_nodes) { return 2 * (size_t)(n_nodes + 1); }

void launch_node_sort(const int32_t* node, const int32_t* status, long long n, long long n_nodes, int32_t* counts,
                      int32_t* order, cudaStream_t s) {
  if (n <= 0) return;
  long long m = n_nodes + 1;
  cudaMemsetAsync(counts, 0, sizeof(int32_t) * m, s);
  long long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  node_hist_kernel<<<(unsigned)blocks, 256, 0, s>>>(node, status, n, n_nodes, counts);
  node_scan_kernel<<<1, 1024, 0, s>>>(counts, m);
  node_scatter_kernel<<<(unsigned)blocks, 256, 0, s>>>(node, status, n, n_nodes, counts + m, order);
}

}  // namespace brx
