// K3+K4: gather and weighted sum of vertex data, fused with the rotation
// back by R (and the Γ permutation/phase for phonon eigenvectors).
//
// q are grouped by the vertex set they interpolate from and their pivot
// vertex (a counting sort on the group key the locate kernel writes).  A
// persistent CTA takes one group at a time from a work queue, stages the
// group's vertex rows in shared memory one block of modes at a time, forms
// the antiphase factors once for the whole group, and then writes every q's
// rotated rows.  Vertex data are read once per group rather than once per q,
// and global loads and stores are contiguous rows.
//
// Reference: Interpolator::interpolate_at_mix (src/interpolator_at.tpp:92-127),
// antiphase (src/utilities.tpp:567-578), PermutationTable::safe_get
// (src/permutation_table.hpp:193-198), rip_real / rip_recip / rip_axial
// (src/interpolator_{real,recip,axial}.tpp) and rip_gamma_complex
// (src/interpolator_gamma.tpp:49-139).
#include <cuda_bf16.h>

#include <algorithm>
#include <type_traits>

#include "../../include/brx.h"
#include "brx_kernels.h"

namespace brx {

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

// Shared-memory row of staged vertex data: s elements of St (complex: pairs)
// padded so that consecutive rows start on different banks.
template <typename St, bool CPLX>
__host__ __device__ inline int row_stride(int s) {
  return CPLX ? 2 * s + 2 : s + 1;  // in St units
}

template <typename Acc, typename St, bool CPLX>
__device__ __forceinline__ void ldY(const St* y, Acc& re, Acc& im) {
  if constexpr (std::is_same<St, __nv_bfloat16>::value) {
    if (CPLX) {
      const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(y));
      re = (Acc)f.x;
      im = (Acc)f.y;
    } else {
      re = (Acc)__bfloat162float(*y);
      im = 0;
    }
  } else {
    if (CPLX) {
      using V2 = typename std::conditional<std::is_same<St, float>::value, float2, double2>::type;
      const V2 v = *reinterpret_cast<const V2*>(y);
      re = (Acc)v.x;
      im = (Acc)v.y;
    } else {
      re = (Acc)*y;
      im = 0;
    }
  }
}

// copy one complex or real element (global → shared) in the storage type
template <typename St, bool CPLX>
__device__ __forceinline__ void cpY(St* dst, const St* src) {
  if constexpr (CPLX) {
    if constexpr (std::is_same<St, float>::value) {
      *reinterpret_cast<float2*>(dst) = __ldg(reinterpret_cast<const float2*>(src));
    } else if constexpr (std::is_same<St, double>::value) {
      *reinterpret_cast<double2*>(dst) = __ldg(reinterpret_cast<const double2*>(src));
    } else {
      *reinterpret_cast<__nv_bfloat162*>(dst) = *reinterpret_cast<const __nv_bfloat162*>(src);
    }
  } else {
    *dst = src[0];
  }
}

struct GroupLayout {
  size_t q, oq, rot, ident, w, R, ph, M, de, e, Y, total;
};

// e_modes: antiphase entries per slot; ybuf: elements of one of the two
// staging buffers of vertex rows
template <typename Acc, typename St>
__host__ __device__ inline GroupLayout group_layout_dims(int QM, int e_modes, int na, long long ybuf) {
  GroupLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = (o + 15) & ~size_t(15);
    o = at + bytes;
    return at;
  };
  L.q = take(sizeof(long long) * QM);
  L.oq = take(sizeof(long long) * QM);
  L.rot = take(sizeof(int) * 2 * QM);
  L.ident = take(sizeof(int) * 2 * QM);
  L.w = take(sizeof(Acc) * 8 * QM);
  L.R = take(sizeof(Acc) * 18 * QM);
  L.ph = take(sizeof(Acc) * 2 * (size_t)na * QM);
  L.M = take(sizeof(Acc) * 12 * QM);
  L.de = take(sizeof(int) * (size_t)(na > 0 ? na : 1) * QM);
  L.e = take(sizeof(Acc) * 2 * 8 * (size_t)e_modes);
  L.Y = take(sizeof(St) * 2 * (size_t)ybuf);
  L.total = (o + 15) & ~size_t(15);
  return L;
}

template <typename Acc, typename St, bool CPLX>
__host__ __device__ inline GroupLayout group_layout(int QM, int MB, int s, int na) {
  return group_layout_dims<Acc, St>(QM, MB, na, 8LL * MB * row_stride<St, CPLX>(s));
}

// Store ne (1 or 3) interpolated elements; complex values as 2-wide vectors.
template <typename Out, bool CPLX, typename Acc>
__device__ __forceinline__ void store_group(Out* dst, const Acc* vr, const Acc* vi, int ne) {
  if (CPLX) {
    using V2 = typename std::conditional<std::is_same<Out, float>::value, float2, double2>::type;
    V2* d = reinterpret_cast<V2*>(dst);
    for (int k = 0; k < ne; ++k) {
      V2 v;
      v.x = (Out)vr[k];
      v.y = (Out)vi[k];
      d[k] = v;
    }
  } else {
    for (int k = 0; k < ne; ++k) dst[k] = (Out)vr[k];
  }
}

// One q's 3×3 matrix element group: weighted sum of the staged rows (with
// their antiphase) then R·M·R⁻¹ (real lattice), Rᵀ·M·(R⁻¹)ᵀ (reciprocal) or
// R⁻¹·M·R (axial).
template <typename Acc, typename St, bool CPLX, typename Out>
__device__ void matrix_item(const GatherParams& p, const St* s_Y, int rs, const Acc* s_e, const Acc* wj, const Acc* R,
                            int ident, bool gamma, int pivot, int nslot, int MB, int b, int e0, Out* dst,
                            bool pre = false) {
  using A = Ar<Acc>;
  constexpr int comps = CPLX ? 2 : 1;
  Acc vr[9], vi[9];
  for (int k = 0; k < 9; ++k) { vr[k] = 0; vi[k] = 0; }
  for (int x = pivot; x < nslot; ++x) {
    // pre: the staged rows past the pivot already carry their antiphase, as
    // differences from the pivot row, whose weight is then 1
    const Acc wx = (pre && x == pivot) ? (Acc)1 : wj[x];
    if (wx == (Acc)0) continue;
    const Acc er = pre ? (Acc)1 : s_e[2 * (x * MB + b)], ei = pre ? (Acc)0 : s_e[2 * (x * MB + b) + 1];
    const Acc wr = A::mul(wx, er), wi = A::mul(wx, ei);
    const St* y = s_Y + (size_t)(x * MB + b) * rs + e0 * comps;
    for (int k = 0; k < 9; ++k) {
      Acc dr, di;
      ldY<Acc, St, CPLX>(y + k * comps, dr, di);
      if (CPLX) {
        vr[k] = A::add(vr[k], A::sub(A::mul(wr, dr), A::mul(wi, di)));
        vi[k] = A::add(vi[k], A::add(A::mul(wr, di), A::mul(wi, dr)));
      } else {
        vr[k] = A::add(vr[k], A::mul(wx, dr));
      }
    }
  }
  if (p.rot_mode != ROT_NONE && !gamma && !ident) {
    const Acc* Ri = R + 9;
    Acc Lm[9], Rm[9];
    if (p.rot_mode == ROT_RECIP) {
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) { Lm[3 * a + c] = R[3 * c + a]; Rm[3 * a + c] = Ri[3 * c + a]; }
    } else if (p.rot_mode == ROT_AXIAL) {
      for (int k = 0; k < 9; ++k) { Lm[k] = Ri[k]; Rm[k] = R[k]; }
    } else {
      for (int k = 0; k < 9; ++k) { Lm[k] = R[k]; Rm[k] = Ri[k]; }
    }
    Acc Tr[9], Ti[9];
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) {
        Acc sr = 0, si = 0;
        for (int k = 0; k < 3; ++k) {
          sr = A::add(sr, A::mul(vr[3 * a + k], Rm[3 * k + c]));
          si = A::add(si, A::mul(vi[3 * a + k], Rm[3 * k + c]));
        }
        Tr[3 * a + c] = sr;
        Ti[3 * a + c] = si;
      }
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) {
        Acc sr = 0, si = 0;
        for (int k = 0; k < 3; ++k) {
          sr = A::add(sr, A::mul(Lm[3 * a + k], Tr[3 * k + c]));
          si = A::add(si, A::mul(Lm[3 * a + k], Ti[3 * k + c]));
        }
        vr[3 * a + c] = sr;
        vi[3 * a + c] = si;
      }
  }
  for (int k = 0; k < 9; ++k) {
    dst[(e0 + k) * comps] = (Out)vr[k];
    if (CPLX) dst[(e0 + k) * comps + 1] = (Out)vi[k];
  }
}

// FP64 rotation (and Γ permutation and phase) of one interpolated 3-vector
// with the q's matrix M (already transposed, inverted or scaled as the
// rotation mode needs) and its code (bits 1-9: non-zero entries; 4 bits per
// row from bit 10: a row that is a single ±1 entry).  GB300 issues FP64 at
// 1/64 of the FP32 rate, so every skipped multiply counts: a signed
// permutation (cubic operations, and the z row of hexagonal ones) costs no
// arithmetic at all.  Returns the destination element offset.
template <typename Acc, bool CPLX>
__device__ __forceinline__ int rotate_vector_f64(const GatherParams& p, bool gamma, const Acc* M, int code,
                                                 const Acc* ph, int k, int r_inv, int e0, Acc* vr, Acc* vi) {
  Acc tr[3], ti[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int single = (code >> (10 + 4 * a)) & 15;
    if (single) {
      const int c = (single - 1) % 3;
      const Acc sr = c == 0 ? vr[0] : (c == 1 ? vr[1] : vr[2]);
      const Acc si = c == 0 ? vi[0] : (c == 1 ? vi[1] : vi[2]);
      tr[a] = single > 3 ? -sr : sr;
      ti[a] = single > 3 ? -si : si;
      continue;
    }
    Acc sr = 0, si = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (!((code >> (1 + 3 * a + c)) & 1)) continue;
      const Acc m = M[3 * a + c];
      sr = fma(m, vr[c], sr);
      if (CPLX) si = fma(m, vi[c], si);
    }
    tr[a] = sr;
    ti[a] = si;
  }
  int de = e0;
  if (gamma) {
    de = p.nsc + 3 * __ldg(p.gamma_F0 + k * p.n_ops + r_inv);
    const Acc pr = ph[0], pi = ph[1];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      vr[a] = fma(pr, tr[a], -(pi * ti[a]));
      vi[a] = fma(pr, ti[a], pi * tr[a]);
    }
  } else {
#pragma unroll
    for (int a = 0; a < 3; ++a) { vr[a] = tr[a]; vi[a] = ti[a]; }
  }
  return de;
}

// Asynchronous global → shared copy of one staged element (cp.async):
// 4, 8 or 16 bytes, so the copy of the next block of rows overlaps compute.
template <typename St, bool CPLX>
__device__ __forceinline__ void cp_async_elem(St* dst, const St* src) {
  constexpr int bytes = (CPLX ? 2 : 1) * (int)sizeof(St);
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (bytes == 16) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
  } else if constexpr (bytes == 8) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
  } else if constexpr (bytes == 4) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
  } else {
    *dst = *src;  // 2-byte elements: a plain copy
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Group bookkeeping kept in shared memory for the current and the next group.
struct GroupInfo {
  int key, start, count;  // count < 0: no group
  int nslot, pivot;
  int vid[8];
  int pid[8];
  int kid[8];  // antiphase-table key of (pivot, slot) or -1 (FP64 complex data)
};

// index of key i·N + j in the antiphase table's sorted keys, or -1
__device__ __forceinline__ int phase_key(const GatherParams& p, long long i, long long j) {
  if (!p.ph_table || i == j) return -1;
  long long key = i * p.n_vertices + j, lo = 0, hi = p.n_ph_keys;
  while (lo < hi) {
    long long mid = (lo + hi) >> 1;
    if (__ldg(p.ph_keys + mid) < key) lo = mid + 1; else hi = mid;
  }
  return (lo < p.n_ph_keys && __ldg(p.ph_keys + lo) == key) ? (int)lo : -1;
}

// Warp 0 takes the next work descriptor and decodes its vertex slots.  In a
// batch (gb.items set) it also finds the descriptor's interpolator and
// copies that item's parameters into *slot.
__device__ __forceinline__ void fetch_group(const GatherBatch& gb, int n_groups, GatherParams* slot, GroupInfo* gi,
                                            int lane) {
  int g = 0;
  if (lane == 0) g = atomicAdd(gb.counter, 1);
  g = __shfl_sync(0xffffffffu, g, 0);
  if (g >= n_groups) {
    if (lane == 0) gi->count = -1;
    return;
  }
  const GroupDesc d = gb.reverse ? gb.groups[-1 - g] : gb.groups[g];
  int key = d.key;
  if (gb.items) {
    int item = 0;
    if (lane == 0) {
      int lo = 0, hi = gb.n_items - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(gb.key_off + mid) <= key) lo = mid;
        else hi = mid - 1;
      }
      item = lo;
    }
    item = __shfl_sync(0xffffffffu, item, 0);
    const int* src = reinterpret_cast<const int*>(gb.items + item);
    int* dst = reinterpret_cast<int*>(slot);
    for (int w = lane; w < (int)(sizeof(GatherParams) / sizeof(int)); w += 32) dst[w] = __ldg(src + w);
    __syncwarp();
    key -= slot->key_base;
  }
  const GatherParams& p = *slot;
  int nslot, pivot, vid = 0;
  if (key < 8 * p.n_cube) {
    pivot = key & 7;
    nslot = 8;
    if (lane < 8) vid = __ldg(p.cube_vertices + 8 * (long long)__ldg(p.rank_cube + (key >> 3)) + 7 - lane);
  } else {
    const long long t = (key - 8LL * p.n_cube) >> 2;
    pivot = (int)((key - 8LL * p.n_cube) & 3);
    nslot = 4;
    if (lane < 4) vid = __ldg(p.tet_vertices + 4 * t + lane);
  }
  const int pv = __shfl_sync(0xffffffffu, vid, pivot);
  if (lane < 8) {
    gi->vid[lane] = vid;
    gi->pid[lane] = lane < nslot ? perm_lookup(p, pv, vid) : -1;
    gi->kid[lane] = lane < nslot ? phase_key(p, pv, vid) : -1;
  }
  if (lane == 0) {
    gi->key = key;
    gi->start = d.start;
    gi->count = d.count;
    gi->nslot = nslot;
    gi->pivot = pivot;
  }
}

// Issue the asynchronous copies of rows [b0, b0 + mb) of the group's used
// slots into a staging buffer; one warp per row.
template <typename St, bool CPLX>
__device__ __forceinline__ void issue_rows(const GatherParams& p, const GroupInfo& gi, int b0, int mb, int MB, int rs,
                                           St* Y, int warp, int lane, int nwarp) {
  constexpr int comps = CPLX ? 2 : 1;
  const St* data = reinterpret_cast<const St*>(p.data);
  const int s = p.s, B = p.B;
  const int ns = gi.nslot - gi.pivot;
  for (int r = warp; r < ns * mb; r += nwarp) {
    const int b = r % mb, x = gi.pivot + r / mb;
    const int pid = gi.pid[x];
    const int row = pid >= 0 ? __ldg(p.perms + (long long)pid * B + b0 + b) : b0 + b;
    const St* src = data + ((long long)gi.vid[x] * B + row) * s * comps;
    St* dst = Y + (size_t)(x * MB + b) * rs;
    for (int e = lane; e < s; e += 32) cp_async_elem<St, CPLX>(dst + e * comps, src + e * comps);
  }
}

// FP32 output items of one block of modes.  Work unit = (mode, element
// group) × a share of the group's q: the unit's rows of every slot, with
// their antiphase, stay in registers while it loops over its q.  NS is the
// number of vertex slots (8 for a cube node, 4 for a tetrahedron).
// The q loop of one vector work unit (FP32): weighted sum of the unit's
// slot rows held in registers, rotation and Γ phase per q, three complex
// elements stored at the q's output offset.
template <int NS, typename Acc, bool CPLX, typename Out>
__device__ __forceinline__ void vector_unit(const Acc (&yr)[NS][3], const Acc (&yi)[NS][3], const Acc* s_w,
                                            const Acc* s_M, const int* s_rotf, const Acc* s_ph, const int* s_de,
                                            const long long* s_oq, int qs, int count, int qsplit, bool gamma, int na,
                                            int k_atom, int e0, long long row_off, Out* out) {
  constexpr int comps = CPLX ? 2 : 1;
  for (int j = qs; j < count; j += qsplit) {
    Acc wv[8];
    {
      const float4 w0 = *reinterpret_cast<const float4*>(s_w + 8 * j);
      wv[0] = w0.x; wv[1] = w0.y; wv[2] = w0.z; wv[3] = w0.w;
      if (NS == 8) {
        const float4 w1 = *reinterpret_cast<const float4*>(s_w + 8 * j + 4);
        wv[4] = w1.x; wv[5] = w1.y; wv[6] = w1.z; wv[7] = w1.w;
      }
    }
    Acc vr[3] = {0, 0, 0}, vi[3] = {0, 0, 0};
#pragma unroll
    for (int x = 0; x < NS; ++x) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        vr[k] += wv[x] * yr[x][k];
        if (CPLX) vi[k] += wv[x] * yi[x][k];
      }
    }
    int de = e0;
    if (s_rotf[j]) {
      const float4 m0 = *reinterpret_cast<const float4*>(s_M + 12 * j);
      const float4 m1 = *reinterpret_cast<const float4*>(s_M + 12 * j + 4);
      const float m8 = s_M[12 * j + 8];
      const Acc M[9] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w, m8};
      Acc tr[3], ti[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        tr[a] = M[3 * a] * vr[0] + M[3 * a + 1] * vr[1] + M[3 * a + 2] * vr[2];
        ti[a] = M[3 * a] * vi[0] + M[3 * a + 1] * vi[1] + M[3 * a + 2] * vi[2];
      }
      if (gamma) {
        de = s_de[j * na + k_atom];
        const float2 ph = *reinterpret_cast<const float2*>(s_ph + 2 * (j * na + k_atom));
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          vr[a] = ph.x * tr[a] - ph.y * ti[a];
          vi[a] = ph.x * ti[a] + ph.y * tr[a];
        }
      } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) { vr[a] = tr[a]; vi[a] = ti[a]; }
      }
    }
    store_group<Out, CPLX>(out + s_oq[j] + row_off + (long long)de * comps, vr, vi, 3);
  }
}

template <int NS, typename Acc, typename St, bool CPLX, typename Out>
__device__ __forceinline__ void reg_tile_items(const GatherParams& p, const St* s_Y, int rs, const Acc* s_e,
                                               const Acc* s_w, const Acc* s_R, const int* s_id, const Acc* s_M,
                                               const int* s_rotf, const Acc* s_ph, const int* s_de,
                                               const long long* s_q, const long long* s_oq, long long qb,
                                               int count, int pivot, int MB, int b0, int mb, int G, int na,
                                               Out* out) {
  constexpr int comps = CPLX ? 2 : 1;
  const int B = p.B, s = p.s;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int nitem = mb * G;
  const int units = p.qsplit > 0 ? p.qsplit : 2;
  int qsplit = (units * nth + nitem - 1) / nitem;
  if (qsplit > count) qsplit = count;
  if (qsplit < 1) qsplit = 1;
  const bool gamma = p.rot_mode == ROT_GAMMA;
  for (int it = tid; it < nitem * qsplit; it += nth) {
    const int item = it % nitem, qs = it / nitem;
    const int b = item / G, gi = item % G;
    const int bb = b0 + b;
    int e0, ne;
    if (gi < p.nsc) { e0 = gi; ne = 1; }
    else if (gi < p.nsc + p.nvec) { e0 = p.nsc + 3 * (gi - p.nsc); ne = 3; }
    else { e0 = p.nsc + 3 * p.nvec + 9 * (gi - p.nsc - p.nvec); ne = 9; }
    if (ne == 9) {
      for (int j = qs; j < count; j += qsplit)
        matrix_item<Acc, St, CPLX, Out>(p, s_Y, rs, s_e, s_w + 8 * j, s_R + 18 * j, s_id[j], false, pivot, NS, MB,
                                        b, e0, out + ((size_t)(s_q[j] - qb) * B + bb) * (size_t)s * comps);
      continue;
    }
    Acc yr[NS][3], yi[NS][3];
#pragma unroll
    for (int x = 0; x < NS; ++x) {
      const bool usex = x >= pivot;
      const Acc er = usex ? s_e[2 * (x * MB + b)] : (Acc)0;
      const Acc ei = usex ? s_e[2 * (x * MB + b) + 1] : (Acc)0;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        Acc dr = 0, di = 0;
        if (usex && k < ne) ldY<Acc, St, CPLX>(s_Y + (size_t)(x * MB + b) * rs + (e0 + k) * comps, dr, di);
        yr[x][k] = er * dr - ei * di;
        yi[x][k] = er * di + ei * dr;
      }
    }
    const int k_atom = gi - p.nsc;
    const size_t row_off = (size_t)bb * s * comps;
    if (ne == 3) {
      vector_unit<NS, Acc, CPLX, Out>(yr, yi, s_w, s_M, s_rotf, s_ph, s_de, s_oq, qs, count, qsplit, gamma, na, k_atom,
                                      e0, (long long)row_off, out);
      continue;
    }
    for (int j = qs; j < count; j += qsplit) {
      Acc wv[8];
      {
        const float4 w0 = *reinterpret_cast<const float4*>(s_w + 8 * j);
        wv[0] = w0.x; wv[1] = w0.y; wv[2] = w0.z; wv[3] = w0.w;
        if (NS == 8) {
          const float4 w1 = *reinterpret_cast<const float4*>(s_w + 8 * j + 4);
          wv[4] = w1.x; wv[5] = w1.y; wv[6] = w1.z; wv[7] = w1.w;
        }
      }
      Acc vr[3] = {0, 0, 0}, vi[3] = {0, 0, 0};
#pragma unroll
      for (int x = 0; x < NS; ++x) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          vr[k] += wv[x] * yr[x][k];
          if (CPLX) vi[k] += wv[x] * yi[x][k];
        }
      }
      Out* dst = out + (size_t)(s_q[j] - qb) * B * s * comps + row_off;
      int de = e0;
      if (ne == 3 && s_rotf[j]) {
        const float4 m0 = *reinterpret_cast<const float4*>(s_M + 12 * j);
        const float4 m1 = *reinterpret_cast<const float4*>(s_M + 12 * j + 4);
        const float m8 = s_M[12 * j + 8];
        const Acc M[9] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w, m8};
        Acc tr[3], ti[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          tr[a] = M[3 * a] * vr[0] + M[3 * a + 1] * vr[1] + M[3 * a + 2] * vr[2];
          ti[a] = M[3 * a] * vi[0] + M[3 * a + 1] * vi[1] + M[3 * a + 2] * vi[2];
        }
        if (gamma) {
          de = s_de[j * na + k_atom];
          const float2 ph = *reinterpret_cast<const float2*>(s_ph + 2 * (j * na + k_atom));
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            vr[a] = ph.x * tr[a] - ph.y * ti[a];
            vi[a] = ph.x * ti[a] + ph.y * tr[a];
          }
        } else {
#pragma unroll
          for (int a = 0; a < 3; ++a) { vr[a] = tr[a]; vi[a] = ti[a]; }
        }
      }
      store_group<Out, CPLX>(dst + (size_t)de * comps, vr, vi, ne);
    }
  }
}

// Persistent gather over work descriptors.  With single set, every group
// belongs to that interpolator; otherwise gb.items describes a batch and
// each group's item parameters are fetched with it.  The parameters of the
// current and of the next group live in s_p[cur] and s_p[cur ^ 1].
template <typename Acc, typename St, bool CPLX, typename Out>
__device__ __forceinline__ void gather_groups(const GatherParams* single, const GatherBatch& gb) {
  using A = Ar<Acc>;
  // FP32 arithmetic: rows held in registers across the q of a group.
  // FP64: the reference's operation order, rows read from shared memory.
  constexpr bool kRegTile = sizeof(Acc) == 4;
  constexpr int comps = CPLX ? 2 : 1;
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ GroupInfo s_g[2];
  __shared__ GatherParams s_p[2];
  const int QM = gb.qmax;
  const GroupLayout L = group_layout_dims<Acc, St>(QM, gb.e_modes, gb.ph_atoms, gb.ybuf);
  long long* s_q = reinterpret_cast<long long*>(sm + L.q);
  long long* s_oq = reinterpret_cast<long long*>(sm + L.oq);
  int* s_rot = reinterpret_cast<int*>(sm + L.rot);
  int* s_id = reinterpret_cast<int*>(sm + L.ident);
  Acc* s_w = reinterpret_cast<Acc*>(sm + L.w);
  Acc* s_R = reinterpret_cast<Acc*>(sm + L.R);
  Acc* s_ph = reinterpret_cast<Acc*>(sm + L.ph);
  Acc* s_M = reinterpret_cast<Acc*>(sm + L.M);
  int* s_de = reinterpret_cast<int*>(sm + L.de);
  int* s_rotf = s_id + QM;  // second half of the ident block
  Acc* s_e = reinterpret_cast<Acc*>(sm + L.e);
  St* const s_Y0 = reinterpret_cast<St*>(sm + L.Y);
  const size_t ybuf = (size_t)gb.ybuf;
  const int n_groups = *gb.n_groups;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nwarp = nth >> 5;
  if (single) {
    const int* src = reinterpret_cast<const int*>(single);
    for (int w = tid; w < (int)(sizeof(GatherParams) / sizeof(int)); w += nth) {
      reinterpret_cast<int*>(&s_p[0])[w] = src[w];
      reinterpret_cast<int*>(&s_p[1])[w] = src[w];
    }
    __syncthreads();
  }

  if (warp == 0) fetch_group(gb, n_groups, &s_p[0], &s_g[0], lane);
  __syncthreads();
  if (s_g[0].count < 0) return;
  {
    const GatherParams& pn = s_p[0];
    issue_rows<St, CPLX>(pn, s_g[0], 0, min(pn.MB, pn.B), pn.MB, row_stride<St, CPLX>(pn.s), s_Y0, warp, lane,
                         nwarp);
  }
  cp_async_commit();
  int cur = 0, buf = 0;

  for (;;) {
    const GroupInfo& gc = s_g[cur];
    const GatherParams& p = s_p[cur];
    const int B = p.B, s = p.s, MB = p.MB;
    const int rs = row_stride<St, CPLX>(s);
    const bool gamma = p.rot_mode == ROT_GAMMA;
    const int na = gamma ? p.nvec : 0;
    const int G = p.nsc + p.nvec + p.nmat;
    const int nblk = (B + MB - 1) / MB;
    const long long qb = p.q_base;
    Out* out = reinterpret_cast<Out*>(p.out);
    // the next group is taken now so that its first rows can load early
    if (warp == 0) fetch_group(gb, n_groups, &s_p[cur ^ 1], &s_g[cur ^ 1], lane);
    const int count = gc.count, start = gc.start, nslot = gc.nslot, pivot = gc.pivot;
    // per-q records: weights by slot, R and R⁻¹
    for (int j = tid; j < count; j += nth) {
      const long long qi = p.order[start + j];
      s_q[j] = qi;
      s_oq[j] = (qi - qb) * (long long)B * s * comps;
      Acc wsl[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      const int nw = p.nw[qi];
      for (int k = 0; k < nw; ++k) {
        const int v = p.vidx[8 * qi + k];
        const Acc wk = sizeof(Acc) == 4 ? (Acc)p.w32[8 * qi + k] : (Acc)p.w[8 * qi + k];
        for (int x = 0; x < nslot; ++x)
          if (gc.vid[x] == v) wsl[x] = wk;
      }
      for (int x = 0; x < 8; ++x) s_w[8 * j + x] = wsl[x];
      int r0 = 0, r1 = 0, ident = 1;
      if (p.rot_mode != ROT_NONE) {
        r0 = p.rot[2 * qi];
        r1 = p.rot[2 * qi + 1];
        const int32_t* W = p.ops + 9 * r0;
        ident = (W[0] == 1 && W[1] == 0 && W[2] == 0 && W[3] == 0 && W[4] == 1 && W[5] == 0 && W[6] == 0 &&
                 W[7] == 0 && W[8] == 1);
        for (int e = 0; e < 9; ++e) {
          if (gamma && p.gamma_cart) {
            s_R[18 * j + e] = (Acc)p.rot_cart[9 * r0 + e];
            s_R[18 * j + 9 + e] = (Acc)p.rot_cart[9 * r1 + e];
          } else {
            s_R[18 * j + e] = (Acc)p.ops[9 * r0 + e];
            s_R[18 * j + 9 + e] = (Acc)p.ops[9 * r1 + e];
          }
        }
      }
      s_rot[2 * j] = r0;
      s_rot[2 * j + 1] = r1;
      s_id[j] = ident;
      // the matrix applied to 3-vectors, and whether to apply it: bit 0 set
      // when it applies; for the FP64 path bits 1-9 mark its non-zero entries
      // and 4 bits per row from bit 10 name a row that is a single ±1 entry
      // (1 + column, + 3 when negative), which then costs no arithmetic
      {
        const Acc* R = s_R + 18 * j;
        const Acc* Ri = R + 9;
        Acc scale = 1;
        if (p.rot_mode == ROT_AXIAL)
          scale = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) +
                  R[2] * (R[3] * R[7] - R[4] * R[6]);
        const bool apply = p.rot_mode != ROT_NONE && (gamma || !ident);
        int code = apply ? 1 : 0;
        for (int a = 0; a < 3; ++a) {
          int nz = 0, single = 0;
          for (int c = 0; c < 3; ++c) {
            Acc m;
            if (p.rot_mode == ROT_RECIP) m = R[3 * c + a];
            else if (gamma || p.rot_mode == ROT_AXIAL) m = scale * Ri[3 * a + c];
            else m = R[3 * a + c];
            s_M[12 * j + 3 * a + c] = m;
            if (apply && m != (Acc)0) {
              code |= 1 << (1 + 3 * a + c);
              ++nz;
              single = (m == (Acc)1) ? 1 + c : (m == (Acc)-1 ? 4 + c : 0);
            }
          }
          if (nz == 1) code |= single << (10 + 4 * a);
        }
        s_rotf[j] = code;
      }
    }
    __syncthreads();
    if (gamma) {
      for (int it = tid; it < count * na; it += nth) {
        const int j = it / na, k = it % na;
        const long long qi = s_q[j];
        s_de[it] = p.nsc + 3 * __ldg(p.gamma_F0 + k * p.n_ops + s_rot[2 * j + 1]);
        const double* d = p.gamma_vectors + 3 * __ldg(p.gamma_vidx + k * p.n_ops + s_rot[2 * j + 1]);
        double dq = 0.0;
        dq = __dadd_rn(dq, __dmul_rn(p.q_ir[3 * qi], d[0]));
        dq = __dadd_rn(dq, __dmul_rn(p.q_ir[3 * qi + 1], d[1]));
        dq = __dadd_rn(dq, __dmul_rn(p.q_ir[3 * qi + 2], d[2]));
        const double frac = dq - rint(dq);  // e^{2πi n} = 1 exactly
        if constexpr (sizeof(Acc) == 4) {
          // FP32 arithmetic: the reduced argument is exact, sin/cos in FP32
          float sn, cs;
          sincospif(2.0f * (float)frac, &sn, &cs);
          s_ph[2 * it] = cs;
          s_ph[2 * it + 1] = sn;
        } else {
          double sn, cs;
          sincospi(2.0 * frac, &sn, &cs);
          s_ph[2 * it] = (Acc)cs;
          s_ph[2 * it + 1] = (Acc)sn;
        }
      }
    }
    // ---- blocks of modes, double-buffered ----
    for (int bi = 0; bi < nblk; ++bi) {
      const int b0 = bi * MB;
      const int mb = min(MB, B - b0);
      cp_async_wait_all();
      __syncthreads();
      {
        // rows for the following block: this group's next block, or the
        // first block of the next group
        const GroupInfo& gn = s_g[cur ^ 1];
        if (bi + 1 < nblk) {
          issue_rows<St, CPLX>(p, gc, b0 + MB, min(MB, B - b0 - MB), MB, rs, (s_Y0 + (buf ^ 1) * ybuf), warp, lane, nwarp);
        } else if (gn.count >= 0) {
          const GatherParams& pn = s_p[cur ^ 1];
          issue_rows<St, CPLX>(pn, gn, 0, min(pn.MB, pn.B), pn.MB, row_stride<St, CPLX>(pn.s),
                               (s_Y0 + (buf ^ 1) * ybuf), warp, lane, nwarp);
        }
        cp_async_commit();
      }
      const St* s_Y = s_Y0 + buf * ybuf;
      const int ns = nslot - pivot;
      // antiphase factors, one per (slot, mode), in the reference's sum order
      for (int it = tid; it < ns * mb; it += nth) {
        const int b = it % mb, x = pivot + it / mb;
        Acc er = 1, ei = 0;
        const int kid = gc.kid[x];
        if (CPLX && p.phase_allowed && x != pivot && kid >= 0) {
          // formed once per vertex pair when the data were set
          const double2 t = __ldg(p.ph_table + (long long)kid * B + b0 + b);
          er = (Acc)t.x;
          ei = (Acc)t.y;
        } else if (CPLX && p.phase_allowed && x != pivot) {
          const St* a = s_Y + (size_t)(pivot * MB + b) * rs;
          const St* c = s_Y + (size_t)(x * MB + b) * rs;
          Acc rd = 0, id = 0;
          for (int e = 0; e < s; ++e) {
            Acc ar, ai, br, bi2;
            ldY<Acc, St, CPLX>(a + 2 * e, ar, ai);
            ldY<Acc, St, CPLX>(c + 2 * e, br, bi2);
            rd = A::add(rd, A::add(A::mul(ar, br), A::mul(ai, bi2)));
            id = A::add(id, A::sub(A::mul(ar, bi2), A::mul(ai, br)));
          }
          const Acc mag = sqrt(A::add(A::mul(rd, rd), A::mul(id, id)));
          if (mag > (Acc)0) {
            er = rd / mag;
            ei = -(id / mag);
          }
        }
        s_e[2 * (x * MB + b)] = er;
        s_e[2 * (x * MB + b) + 1] = ei;
      }
      __syncthreads();
      // FP64: every staged row of a slot past the pivot is multiplied by its
      // antiphase once here and stored as its difference from the pivot row
      // (whose factor is 1): the weights sum to 1, so a q's sum is
      // y_pivot + Σ w_x (e_x y_x − y_pivot), one FMA per weight and
      // component and none for the pivot.  A group of one q (small chunks
      // of host-buffer queries) instead takes the complex weight w·e in its
      // sum: 2 FMAs more per element, but no pass.
      const bool phased = !kRegTile && CPLX && p.phase_allowed;
      const bool pre = phased && count >= 2;
      if constexpr (!kRegTile && CPLX) {
        if (pre) {
          St* Yw = s_Y0 + buf * ybuf;
          const int rows = (ns - 1) * mb;
          for (int it = tid; it < rows * s; it += nth) {
            const int e = it % s, r = it / s;
            const int b = r % mb, x = pivot + 1 + r / mb;
            const Acc er = s_e[2 * (x * MB + b)], ei = s_e[2 * (x * MB + b) + 1];
            St* y = Yw + (size_t)(x * MB + b) * rs + 2 * e;
            const St* yp = Yw + (size_t)(pivot * MB + b) * rs + 2 * e;
            const Acc dr = y[0], di = y[1];
            y[0] = fma(er, dr, -(ei * di)) - yp[0];
            y[1] = fma(er, di, ei * dr) - yp[1];
          }
          __syncthreads();
        }
      }
      const int nitem = mb * G;
      if constexpr (kRegTile) {
        if (nslot == 4)
          reg_tile_items<4, Acc, St, CPLX, Out>(p, s_Y, rs, s_e, s_w, s_R, s_id, s_M, s_rotf, s_ph, s_de, s_q, s_oq,
                                                qb, count, pivot, MB, b0, mb, G, na, out);
        else
          reg_tile_items<8, Acc, St, CPLX, Out>(p, s_Y, rs, s_e, s_w, s_R, s_id, s_M, s_rotf, s_ph, s_de, s_q, s_oq,
                                                qb, count, pivot, MB, b0, mb, G, na, out);
      } else {
        const int items = count * nitem;
        for (int it = tid; it < items; it += nth) {
          const int gi = it % G;
          const int jb = it / G;
          const int b = jb % mb, j = jb / mb;
          const int bb = b0 + b;
          const Acc* wj = s_w + 8 * j;
          Out* dst = out + ((size_t)(s_q[j] - qb) * B + bb) * (size_t)s * comps;
          int e0, ne;
          if (gi < p.nsc) { e0 = gi; ne = 1; }
          else if (gi < p.nsc + p.nvec) { e0 = p.nsc + 3 * (gi - p.nsc); ne = 3; }
          else { e0 = p.nsc + 3 * p.nvec + 9 * (gi - p.nsc - p.nvec); ne = 9; }
          if (ne == 9) {
            matrix_item<Acc, St, CPLX, Out>(p, s_Y, rs, s_e, wj, s_R + 18 * j, s_id[j], gamma, pivot, nslot, MB, b,
                                            e0, dst, pre);
            continue;
          }
          // Σ_x w_x·(e_x·d_x) over the weighted vertices, one FMA per weight
          // and component on the antiphased rows (without a phase, e_x = 1)
          Acc vr[3] = {0, 0, 0}, vi[3] = {0, 0, 0};
          for (int x = pivot; x < nslot; ++x) {
            const Acc wx = wj[x];
            if (wx == (Acc)0) continue;
            const St* y = s_Y + (size_t)(x * MB + b) * rs + e0 * comps;
            if (pre && x == pivot) {  // the differences' base: the pivot row itself
              for (int k = 0; k < ne; ++k) ldY<Acc, St, CPLX>(y + k * comps, vr[k], vi[k]);
              continue;
            }
            if (phased && !pre && x != pivot) {
              const Acc wr = wx * s_e[2 * (x * MB + b)], wi = wx * s_e[2 * (x * MB + b) + 1];
              for (int k = 0; k < ne; ++k) {
                Acc dr, di;
                ldY<Acc, St, CPLX>(y + k * comps, dr, di);
                vr[k] = fma(wr, dr, fma(-wi, di, vr[k]));
                vi[k] = fma(wr, di, fma(wi, dr, vi[k]));
              }
              continue;
            }
            for (int k = 0; k < ne; ++k) {
              Acc dr, di;
              ldY<Acc, St, CPLX>(y + k * comps, dr, di);
              vr[k] = fma(wx, dr, vr[k]);
              if (CPLX) vi[k] = fma(wx, di, vi[k]);
            }
          }
          int de = e0;
          const int rotf = s_rotf[j];
          if (ne == 3 && rotf) {
            const int k = gi - p.nsc;
            de = rotate_vector_f64<Acc, CPLX>(p, gamma, s_M + 12 * j, rotf, s_ph + 2 * (j * na + k), k,
                                              s_rot[2 * j + 1], e0, vr, vi);
          }
          store_group<Out, CPLX>(dst + (size_t)de * comps, vr, vi, ne);
        }
      }
      buf ^= 1;
    }
    __syncthreads();  // this group's records and rows are no longer read
    cur ^= 1;
    if (s_g[cur].count < 0) break;
  }
  cp_async_wait_all();
}

// Blocks per SM the FP64 complex gather is compiled for: four 128-thread
// blocks (16 warps) fit the register file at 128 registers a thread, and its
// FP64 pipe waits less with more warps to pick from
template <typename Acc, bool CPLX>
constexpr int kGatherMinBlocks = (sizeof(Acc) == 8 && CPLX) ? 4 : 1;

template <typename Acc, typename St, bool CPLX, typename Out>
__global__ void __launch_bounds__(kGatherThreads, kGatherMinBlocks<Acc, CPLX>) group_gather_kernel(GatherParams p) {
  GatherBatch gb{};
  gb.groups = p.groups;
  gb.n_groups = p.n_groups;
  gb.counter = p.counter;
  gb.qmax = p.qmax;
  gb.e_modes = p.MB;
  gb.ph_atoms = p.rot_mode == ROT_GAMMA ? p.nvec : 0;
  gb.ybuf = 8LL * p.MB * row_stride<St, CPLX>(p.s);
  gather_groups<Acc, St, CPLX, Out>(&p, gb);
}

template <typename Acc, typename St, bool CPLX, typename Out>
__global__ void __launch_bounds__(kGatherThreads) group_gather_batch_kernel(GatherBatch gb) {
  gather_groups<Acc, St, CPLX, Out>(nullptr, gb);
}

// Scalar-only interpolators (eigenvalues): one thread per (q, branch),
// out = Σ_x w_x d[v_x][perm_x(b)] in the reference's order.  The rows are
// small enough to stay in L2, so no grouping is needed.
// ---------------------------------------------------------------------------
// FP32 gather, warp-independent (vector and scalar elements, no matrices)
// ---------------------------------------------------------------------------
// Per group the CTA stages the q records once (two barriers), then every
// warp works alone on its own blocks of MBw modes: one bulk copy
// (cp.async.bulk, completion on the warp's mbarrier) per vertex row into one
// of the warp's two staging buffers while the other is in use, the
// antiphase of each (slot, mode) by two lanes, and one (mode, element group)
// unit per lane over all q of the group, rows held in registers.  No CTA
// barrier inside the mode loop.  Waits are bounded (about a second); on
// expiry the query reports BRX_ERR_TIMEOUT.
constexpr int kWarpGatherMaxWarps = 8;
constexpr long long kGatherSpin = 2000000000LL;

struct WarpLayout {
  size_t q, oq, w, M, rotf, ph, de, e, off, sq, qc, Y, mbar, total;
  size_t ybuf;  // bytes of one staging buffer
};

// QM q per group; e_modes antiphase entries per slot and warp; na Γ phases
// per q; ybuf bytes per staging buffer (two per warp)
// sf_atoms: atoms of the structure factor (0: vectors are written)
__host__ __device__ inline WarpLayout warp_layout(int QM, int e_modes, int na, long long ybuf, int warps,
                                                  int sf_atoms = 0) {
  WarpLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = (o + 15) & ~size_t(15);
    o = at + bytes;
    return at;
  };
  const int nan = na > 0 ? na : 1;
  L.q = take(8 * (size_t)QM);
  L.oq = take(8 * (size_t)QM);
  L.w = take(8 * 8 * (size_t)QM);    // 8 weights per q, each as a (w, w) pair
  L.M = take(8 * 10 * (size_t)QM);   // 3×3 per q as (m, m) pairs, padded to 10
  L.rotf = take(4 * (size_t)QM);
  L.ph = take(4 * 2 * (size_t)nan * QM);
  L.de = take(4 * (size_t)nan * QM);
  L.e = take(4 * 2 * 8 * (size_t)e_modes * warps);
  L.off = take(2 * 8 * (size_t)e_modes * warps);
  L.sq = take(8 * (size_t)sf_atoms * QM);    // c_k e^{2πi Q·x_k} per (q, atom)
  L.qc = take(16 * (size_t)(sf_atoms > 0 ? QM : 0));  // Q·B per q
  L.ybuf = ((size_t)ybuf + 15) & ~size_t(15);
  L.Y = take(2 * L.ybuf * warps);
  L.mbar = take(16 * (size_t)warps);
  L.total = (o + 15) & ~size_t(15);
  return L;
}

// Shape of one interpolator in the warp gather: modes per warp block MBw
// (at most 32 units of (mode, element group) per warp where G ≤ 32, within
// the launch's e_modes and ybuf), staged row stride: the data row rounded up to 16 bytes
// (a row copied from a 16-byte aligned address below its start fits) plus
// 16 bytes that shift successive rows across the shared-memory banks.
struct WarpItem {
  int B, s, G, na, MBw, nblk, row_bytes;
  bool gamma;
};

template <typename St, bool CPLX>
__host__ __device__ inline WarpItem warp_item(const GatherParams& P, int e_modes, long long ybuf) {
  WarpItem w;
  w.B = P.B;
  w.s = P.s;
  w.G = P.nsc + P.nvec;
  w.gamma = P.rot_mode == ROT_GAMMA;
  w.na = w.gamma ? P.nvec : 0;
  w.row_bytes = ((P.s * (CPLX ? 2 : 1) * (int)sizeof(St) + 15) & ~15) + 16;
  int m = w.G > 0 ? 32 / w.G : 32;
  if (m < 1) m = 1;
  if (m > w.B) m = w.B;
  if (m > e_modes) m = e_modes;
  while (m > 1 && 8LL * m * w.row_bytes > ybuf) --m;
  w.MBw = m;
  w.nblk = (w.B + m - 1) / m;
  return w;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void g_mbar_init(uint32_t m) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(m) : "memory");
}
__device__ __forceinline__ void g_expect(uint32_t m, uint32_t bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;\n" ::"r"(m), "r"(bytes) : "memory");
}
__device__ __forceinline__ void g_arrive(uint32_t m) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(m) : "memory");
}
__device__ __forceinline__ void g_bulk(uint32_t dst, const void* src, uint32_t bytes, uint32_t m) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(m)
               : "memory");
}
__device__ __forceinline__ bool g_wait(uint32_t m, uint32_t phase, long long limit = kGatherSpin) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(m), "r"(phase)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > limit) return false;
  }
}
// BRX_FLAG_TEST_TIMEOUT: about a millisecond on a barrier nothing completes
constexpr long long kStallCycles = 2000000LL;

// One lane's (mode, element group) unit of the warp gather over its q.
// Values travel as (re, im) pairs on the packed FP32 pipe: the NS corner
// rows with their antiphase once, then per q the weighted corner sum
// (one __ffma2_rn per corner and element), the 3×3 rotation on pairs, the
// Γ phase, and the store.  Weights and matrix entries sit in shared memory
// as (w, w) pairs.  ne: 1 for a scalar element, 3 for a vector.
template <int NS, typename St, bool CPLX, typename Out>
__device__ __forceinline__ void warp_unit(const unsigned char* Yb, const unsigned char* so, int row_bytes, int MBw,
                                          int mm, const float* s_e, int pivot, int e0, int ne, const float2* s_w2,
                                          const float2* s_M2, const int* s_rotf, const float* s_ph, const int* s_de,
                                          const long long* s_oq, int j0, int count, int jstep, bool gamma, int na,
                                          int k_atom, long long row_off, Out* out) {
  constexpr int comps = CPLX ? 2 : 1;
  float2 y[NS][3];
#pragma unroll
  for (int x = 0; x < NS; ++x) {
    const bool usex = x >= pivot;
    const float er = usex ? s_e[2 * (x * MBw + mm)] : 0.f, ei = usex ? s_e[2 * (x * MBw + mm) + 1] : 0.f;
    const St* yp = reinterpret_cast<const St*>(Yb + (size_t)(x * MBw + mm) * row_bytes + so[x * MBw + mm]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float dr = 0.f, di = 0.f;
      if (usex && k < ne) ldY<float, St, CPLX>(yp + (e0 + k) * comps, dr, di);
      y[x][k] = make_float2(er * dr - ei * di, er * di + ei * dr);
    }
  }
  const float2 zero = make_float2(0.f, 0.f);
  for (int j = j0; j < count; j += jstep) {
    float2 wp[NS];
#pragma unroll
    for (int h = 0; h < NS / 2; ++h) {
      const float4 t = reinterpret_cast<const float4*>(s_w2 + 8 * j)[h];
      wp[2 * h] = make_float2(t.x, t.y);
      wp[2 * h + 1] = make_float2(t.z, t.w);
    }
    Out* dst = out + s_oq[j] + row_off;
    if (ne == 1) {
      float2 v = zero;
#pragma unroll
      for (int x = 0; x < NS; ++x) v = __ffma2_rn(wp[x], y[x][0], v);
      dst += (long long)e0 * comps;
      if (CPLX) {
        dst[0] = (Out)v.x;
        dst[1] = (Out)v.y;
      } else {
        dst[0] = (Out)v.x;
      }
      continue;
    }
    float2 v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      v[k] = zero;
#pragma unroll
      for (int x = 0; x < NS; ++x) v[k] = __ffma2_rn(wp[x], y[x][k], v[k]);
    }
    int de = e0;
    if (s_rotf[j]) {
      float2 M[9];
      const float4* m4 = reinterpret_cast<const float4*>(s_M2 + 10 * j);
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const float4 t = m4[h];
        M[2 * h] = make_float2(t.x, t.y);
        M[2 * h + 1] = make_float2(t.z, t.w);
      }
      M[8] = s_M2[10 * j + 8];
      float2 t[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        t[a] = __fmul2_rn(M[3 * a], v[0]);
        t[a] = __ffma2_rn(M[3 * a + 1], v[1], t[a]);
        t[a] = __ffma2_rn(M[3 * a + 2], v[2], t[a]);
      }
      if (gamma) {
        de = s_de[j * na + k_atom];
        const float2 ph = *reinterpret_cast<const float2*>(s_ph + 2 * (j * na + k_atom));
#pragma unroll
        for (int a = 0; a < 3; ++a) v[a] = make_float2(ph.x * t[a].x - ph.y * t[a].y, ph.x * t[a].y + ph.y * t[a].x);
      } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) v[a] = t[a];
      }
    }
    // outputs are written once: streaming stores (evict first) keep the
    // vertex rows, which neighbouring groups read again, in L2
    dst += (long long)de * comps;
    if (CPLX) {
      using V2 = typename std::conditional<std::is_same<Out, float>::value, float2, double2>::type;
      V2* d2 = reinterpret_cast<V2*>(dst);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        V2 o;
        o.x = (Out)v[k].x;
        o.y = (Out)v[k].y;
        __stcs(d2 + k, o);
      }
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) __stcs(dst + k, (Out)v[k].x);
    }
  }
}

// Structure factor of one block of modes (vector data only, mb·G ≤ 32
// units, every lane of the warp taking part): per q the unit's Γ-rotated
// eigenvector e_k of atom k, dotted with Q_c and weighted by c_k e^{2πi Q·x_k},
// summed over the G atoms of the mode by a segmented shuffle reduction; the
// mode's first lane writes |F|² at out[q·B + mode].
template <int NS, typename St>
__device__ __forceinline__ void warp_block_sf(const unsigned char* Yb, const unsigned char* so, int row_bytes, int MBw,
                                              int mb, int G, const float* s_e, int pivot, const float2* s_w2,
                                              const float2* s_M2, const int* s_rotf, const float* s_ph,
                                              const int* s_de, const long long* s_oq, const float2* s_sq,
                                              const float4* s_qc, int nsf, int count, int wslice, int qs, int wq,
                                              bool gamma, int na, int b0, float* out) {
  const int lane = threadIdx.x & 31;
  const int U = mb * G;
  const bool active = lane < qs * U;
  const int u = active ? lane % U : 0;
  const int lslice = active ? lane / U : 0;
  const int mm = u / G, gi = u % G;
  const int e0 = 3 * gi;
  // the unit's corner rows with their antiphase (as warp_unit does)
  float2 y[NS][3];
#pragma unroll
  for (int x = 0; x < NS; ++x) {
    const bool usex = x >= pivot;
    const float er = usex ? s_e[2 * (x * MBw + mm)] : 0.f, ei = usex ? s_e[2 * (x * MBw + mm) + 1] : 0.f;
    const St* yp = reinterpret_cast<const St*>(Yb + (size_t)(x * MBw + mm) * row_bytes + so[x * MBw + mm]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float dr = 0.f, di = 0.f;
      if (usex) ldY<float, St, true>(yp + (e0 + k) * 2, dr, di);
      y[x][k] = make_float2(er * dr - ei * di, er * di + ei * dr);
    }
  }
  const float2 zero = make_float2(0.f, 0.f);
  const int jstep = wq * qs, jbase = wslice * qs;
  const int trips = count > jbase ? (count - jbase + jstep - 1) / jstep : 0;
  // this lane's term of F for q j: c_k e^{2πi Q·x_k} (Q_c · e_k)
  auto term = [&](int j) -> float2 {
    float2 wp[NS];
#pragma unroll
    for (int h = 0; h < NS / 2; ++h) {
      const float4 w4 = reinterpret_cast<const float4*>(s_w2 + 8 * j)[h];
      wp[2 * h] = make_float2(w4.x, w4.y);
      wp[2 * h + 1] = make_float2(w4.z, w4.w);
    }
    float2 v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      v[k] = zero;
#pragma unroll
      for (int x = 0; x < NS; ++x) v[k] = __ffma2_rn(wp[x], y[x][k], v[k]);
    }
    int de = e0;
    if (s_rotf[j]) {
      float2 M[9];
      const float4* m4 = reinterpret_cast<const float4*>(s_M2 + 10 * j);
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const float4 tm = m4[h];
        M[2 * h] = make_float2(tm.x, tm.y);
        M[2 * h + 1] = make_float2(tm.z, tm.w);
      }
      M[8] = s_M2[10 * j + 8];
      float2 tr[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        tr[a] = __fmul2_rn(M[3 * a], v[0]);
        tr[a] = __ffma2_rn(M[3 * a + 1], v[1], tr[a]);
        tr[a] = __ffma2_rn(M[3 * a + 2], v[2], tr[a]);
      }
      if (gamma) {
        de = s_de[j * na + gi];
        const float2 ph = *reinterpret_cast<const float2*>(s_ph + 2 * (j * na + gi));
#pragma unroll
        for (int a = 0; a < 3; ++a)
          v[a] = make_float2(ph.x * tr[a].x - ph.y * tr[a].y, ph.x * tr[a].y + ph.y * tr[a].x);
      } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) v[a] = tr[a];
      }
    }
    const float4 qc = s_qc[j];
    const float2 d = make_float2(qc.x * v[0].x + qc.y * v[1].x + qc.z * v[2].x,
                                 qc.x * v[0].y + qc.y * v[1].y + qc.z * v[2].y);
    const float2 f = s_sq[j * nsf + de / 3];
    return make_float2(f.x * d.x - f.y * d.y, f.x * d.y + f.y * d.x);
  };
  // two q per round: their reductions interleave (independent shuffle
  // chains); segments of G lanes hold one mode's atoms of one q, and rounds
  // with an offset of G or more are skipped (G is the same for every lane)
  for (int t = 0; t < trips; t += 2) {
    const int ja = jbase + t * jstep + lslice, jb = ja + jstep;
    const bool la = active && ja < count, lb = active && t + 1 < trips && jb < count;
    float2 ca = la ? term(ja) : zero;
    float2 cb = lb ? term(jb) : zero;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      if (off >= G) continue;
      const float ax = __shfl_down_sync(0xffffffffu, ca.x, off);
      const float ay = __shfl_down_sync(0xffffffffu, ca.y, off);
      const float bx = __shfl_down_sync(0xffffffffu, cb.x, off);
      const float by = __shfl_down_sync(0xffffffffu, cb.y, off);
      if (gi + off < G) {
        ca.x += ax;
        ca.y += ay;
        cb.x += bx;
        cb.y += by;
      }
    }
    if (gi == 0) {
      if (la) __stcs(out + s_oq[ja] + b0 + mm, ca.x * ca.x + ca.y * ca.y);
      if (lb) __stcs(out + s_oq[jb] + b0 + mm, cb.x * cb.x + cb.y * cb.y);
    }
  }
}

// single: the one interpolator's parameters (gb.items null); otherwise a
// batch whose groups carry their item's parameters.  gb.qmax, e_modes,
// ph_atoms and ybuf give the shared-memory layout in either case.
template <typename St, bool CPLX, typename Out, bool SF = false>
__global__ void __launch_bounds__(kWarpGatherMaxWarps * 32, 2) warp_gather_kernel(GatherParams p, GatherBatch gb) {
  using Acc = float;
  constexpr int comps = CPLX ? 2 : 1;
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ GatherParams s_par[2];
  __shared__ GroupInfo s_g[2];
  __shared__ int s_abort;
  __shared__ __align__(8) unsigned long long s_stall_bar;  // BRX_FLAG_TEST_TIMEOUT: never completed
  const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31, nwarps = nth >> 5;
  const bool batch = gb.items != nullptr;
  bool stall = !batch && p.stall;
  if (!batch)
    for (int w = tid; w < (int)(sizeof(GatherParams) / sizeof(int)); w += nth) {
      reinterpret_cast<int*>(&s_par[0])[w] = reinterpret_cast<const int*>(&p)[w];
      reinterpret_cast<int*>(&s_par[1])[w] = reinterpret_cast<const int*>(&p)[w];
    }
  const int QM = gb.qmax;
  const WarpLayout L = warp_layout(QM, gb.e_modes, gb.ph_atoms, gb.ybuf, nwarps, SF ? gb.sf_atoms : 0);
  float2* s_sq = reinterpret_cast<float2*>(sm + L.sq);
  float4* s_qc = reinterpret_cast<float4*>(sm + L.qc);
  long long* s_q = reinterpret_cast<long long*>(sm + L.q);
  long long* s_oq = reinterpret_cast<long long*>(sm + L.oq);
  float2* s_w2 = reinterpret_cast<float2*>(sm + L.w);
  float2* s_M2 = reinterpret_cast<float2*>(sm + L.M);
  int* s_rotf = reinterpret_cast<int*>(sm + L.rotf);
  Acc* s_ph = reinterpret_cast<Acc*>(sm + L.ph);
  int* s_de = reinterpret_cast<int*>(sm + L.de);
  Acc* s_e = reinterpret_cast<Acc*>(sm + L.e) + (size_t)warp * 2 * 8 * gb.e_modes;
  unsigned char* s_off = sm + L.off + (size_t)warp * 2 * 8 * gb.e_modes;  // row start in its staged copy
  unsigned char* Yw = sm + L.Y + (size_t)warp * 2 * L.ybuf;
  const uint32_t mbar = smem_addr(sm + L.mbar) + 16 * warp;
  if (lane == 0) {
    g_mbar_init(mbar);
    g_mbar_init(mbar + 8);
  }
  if (tid == 0) {
    s_abort = 0;
    g_mbar_init(smem_addr(&s_stall_bar));
  }
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  __syncthreads();
  const int n_groups = *gb.n_groups;
  uint32_t phase[2] = {0u, 0u};
  bool pending[2] = {false, false};
  bool ok = true;

  // rows of block blk of a group into buffer buf: one bulk copy per (used
  // slot, mode), the item's own row size and modes per block.  A copy
  // starts at the 16-byte boundary at or below its row and covers whole
  // 16-byte units (the data buffers carry 16 bytes of slack at their end);
  // each lane adds its copies' bytes to the barrier's expected count before
  // issuing them, and lane 0 arrives once all lanes have.
  auto issue = [&](const GatherParams& P, const WarpItem& it, const GroupInfo& gi, int blk, int buf) {
    const int b0 = blk * it.MBw, mb = min(it.MBw, it.B - b0), ns = gi.nslot - gi.pivot;
    const int rows = ns * mb;
    const uint32_t row_g = (uint32_t)(it.s * comps * (int)sizeof(St));
    const uint32_t m = mbar + 8 * buf;
    unsigned char* Yb = Yw + (size_t)buf * L.ybuf;
    const unsigned char* data = static_cast<const unsigned char*>(P.data);
    for (int r = lane; r < rows; r += 32) {
      const int x = gi.pivot + r / mb, mm = r % mb, b = b0 + mm;
      const int pid = gi.pid[x];
      const int row = pid >= 0 ? __ldg(P.perms + (long long)pid * it.B + b) : b;
      const unsigned char* src = data + ((long long)gi.vid[x] * it.B + row) * (long long)row_g;
      const uint32_t off = (uint32_t)((uintptr_t)src & 15);
      const uint32_t cb = (off + row_g + 15) & ~15u;
      s_off[buf * 8 * gb.e_modes + x * it.MBw + mm] = (unsigned char)off;
      g_expect(m, cb);
      g_bulk(smem_addr(Yb + (size_t)(x * it.MBw + mm) * it.row_bytes), src - off, cb, m);
    }
    __syncwarp();
    if (lane == 0) g_arrive(m);
    pending[buf] = true;
  };

  int cur = 0, buf = 0;
  if (warp == 0) fetch_group(gb, n_groups, &s_par[0], &s_g[0], lane);
  __syncthreads();
  if (s_g[0].count >= 0) {
    const WarpItem it0 = warp_item<St, CPLX>(s_par[0], gb.e_modes, L.ybuf);
    const int wq0 = it0.nblk >= nwarps ? 1 : nwarps / it0.nblk;
    if (warp < it0.nblk * wq0) issue(s_par[0], it0, s_g[0], warp % it0.nblk, 0);
  }
  for (;;) {
    const GroupInfo& gc = s_g[cur];
    if (gc.count < 0 || s_abort) break;
    const GatherParams& p = s_par[cur];
    const WarpItem itm = warp_item<St, CPLX>(p, gb.e_modes, L.ybuf);
    const int B = itm.B, s = itm.s, MBw = itm.MBw, G = itm.G, na = itm.na, nblk = itm.nblk;
    const bool gamma = itm.gamma;
    Out* out = reinterpret_cast<Out*>(p.out);
    // the next descriptor is taken now; its first rows load before the
    // group barrier at the end
    if (warp == 0) fetch_group(gb, n_groups, &s_par[cur ^ 1], &s_g[cur ^ 1], lane);
    const int count = gc.count, start = gc.start, nslot = gc.nslot, pivot = gc.pivot;
    // per-q records over all threads: weights by slot, the 3×3 applied to
    // vectors, output offsets ...
    for (int j = tid; j < count; j += nth) {
      const long long qi = p.order[start + j];
      s_q[j] = qi;
      s_oq[j] = (qi - p.q_base) * (long long)B * (SF ? 1 : s * comps);
      Acc wsl[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      const int nw = p.nw[qi];
      for (int k = 0; k < nw; ++k) {
        const int v = p.vidx[8 * qi + k];
        const Acc wk = p.w32[8 * qi + k];
        for (int x = 0; x < nslot; ++x)
          if (gc.vid[x] == v) wsl[x] = wk;
      }
      for (int x = 0; x < 8; ++x) s_w2[8 * j + x] = make_float2(wsl[x], wsl[x]);
      int rotf = 0;
      if (p.rot_mode != ROT_NONE) {
        const int r0 = p.rot[2 * qi], r1 = p.rot[2 * qi + 1];
        Acc R[9], Ri[9];
        for (int e = 0; e < 9; ++e) {
          if (gamma && p.gamma_cart) {
            R[e] = (Acc)p.rot_cart[9 * r0 + e];
            Ri[e] = (Acc)p.rot_cart[9 * r1 + e];
          } else {
            R[e] = (Acc)p.ops[9 * r0 + e];
            Ri[e] = (Acc)p.ops[9 * r1 + e];
          }
        }
        const int32_t* W = p.ops + 9 * r0;
        const bool ident = W[0] == 1 && W[1] == 0 && W[2] == 0 && W[3] == 0 && W[4] == 1 && W[5] == 0 &&
                           W[6] == 0 && W[7] == 0 && W[8] == 1;
        Acc scale = 1;
        if (p.rot_mode == ROT_AXIAL)
          scale = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) +
                  R[2] * (R[3] * R[7] - R[4] * R[6]);
        for (int a = 0; a < 3; ++a)
          for (int c = 0; c < 3; ++c) {
            Acc mv;
            if (p.rot_mode == ROT_RECIP) mv = R[3 * c + a];
            else if (gamma || p.rot_mode == ROT_AXIAL) mv = scale * Ri[3 * a + c];
            else mv = R[3 * a + c];
            s_M2[10 * j + 3 * a + c] = make_float2(mv, mv);
          }
        rotf = (gamma || !ident) ? 1 : 0;
      }
      s_rotf[j] = rotf;
    }
    // ... and the Γ permutation and phase of every (q, atom)
    if (gamma) {
      for (int t = tid; t < count * na; t += nth) {
        const int j = t / na, k = t - j * na;
        const long long qi = p.order[start + j];
        const int r1 = p.rot[2 * qi + 1];
        s_de[t] = p.nsc + 3 * __ldg(p.gamma_F0 + k * p.n_ops + r1);
        const double* d = p.gamma_vectors + 3 * __ldg(p.gamma_vidx + k * p.n_ops + r1);
        double dq = 0.0;
        dq = __dadd_rn(dq, __dmul_rn(p.q_ir[3 * qi], d[0]));
        dq = __dadd_rn(dq, __dmul_rn(p.q_ir[3 * qi + 1], d[1]));
        dq = __dadd_rn(dq, __dmul_rn(p.q_ir[3 * qi + 2], d[2]));
        const double frac = dq - rint(dq);  // e^{2πi n} = 1 exactly
        float sn, cs;
        sincospif(2.0f * (float)frac, &sn, &cs);
        s_ph[2 * t] = cs;
        s_ph[2 * t + 1] = sn;
      }
    }
    if constexpr (SF) {
      // c_k e^{2πi Q·x_k} for every (q, atom), and Q·B per q (FP64, then FP32)
      const int nsf = gb.sf_atoms;
      for (int t = tid; t < count * nsf; t += nth) {
        const int j = t / nsf, k = t - j * nsf;
        const long long qi = p.order[start + j];
        const double* Qv = p.sf_Q + 3 * qi;
        const double* A = p.sf_atom + 4 * k;
        double dq = 0.0;
        dq = __dadd_rn(dq, __dmul_rn(Qv[0], A[1]));
        dq = __dadd_rn(dq, __dmul_rn(Qv[1], A[2]));
        dq = __dadd_rn(dq, __dmul_rn(Qv[2], A[3]));
        const double frac = dq - rint(dq);
        float sn, cs;
        sincospif(2.0f * (float)frac, &sn, &cs);
        const float ck = (float)A[0];
        s_sq[t] = make_float2(ck * cs, ck * sn);
      }
      for (int j = tid; j < count; j += nth) {
        const long long qi = p.order[start + j];
        const double* Qv = p.sf_Q + 3 * qi;
        double xyz[3];
        for (int i = 0; i < 3; ++i) {
          double acc = 0.0;
          for (int k = 0; k < 3; ++k) acc = __dadd_rn(acc, __dmul_rn(p.sf_B[3 * k + i], Qv[k]));
          xyz[i] = acc;
        }
        s_qc[j] = make_float4((float)xyz[0], (float)xyz[1], (float)xyz[2], 0.f);
      }
    }
    __syncthreads();
    // fewer blocks than warps: wq warps share each block, taking every
    // wq-th q from their slice (a warp beyond nblk·wq idles this group)
    const int wq = nblk >= nwarps ? 1 : nwarps / nblk;
    const int wslice = wq > 1 ? warp / nblk : 0;
    const int bfirst = wq > 1 ? (warp < nblk * wq ? warp % nblk : nblk) : warp;
    const int bstep = wq > 1 ? nblk : nwarps;
    for (int blk = bfirst; blk < nblk && ok; blk += bstep) {
      if (blk + bstep < nblk) issue(p, itm, gc, blk + bstep, buf ^ 1);
      bool got;
      if (stall) {
        // test of the error path: the copies of this block stay pending and
        // are drained at exit
        got = g_wait(smem_addr(&s_stall_bar), 0, kStallCycles);
        stall = false;
      } else {
        got = g_wait(mbar + 8 * buf, phase[buf]);
      }
      got = __all_sync(0xffffffffu, got);
      if (!got) {
        ok = false;
        break;
      }
      phase[buf] ^= 1u;
      pending[buf] = false;
      const unsigned char* Yb = Yw + (size_t)buf * L.ybuf;
      const unsigned char* so = s_off + buf * 8 * gb.e_modes;
      const int row_bytes = itm.row_bytes;
      const int b0 = blk * MBw, mb = min(MBw, B - b0);
      // antiphase of every (slot, mode), two lanes each
      const int npairs = (nslot - pivot) * mb;
      for (int r = 0; r < 2 * npairs; r += 32) {
        const int t = r + lane, pr = t >> 1, half = t & 1;
        Acc rd = 0, id = 0;
        int x = pivot, mm = 0;
        if (pr < npairs) {
          x = pivot + pr / mb;
          mm = pr % mb;
          if (CPLX && p.phase_allowed && x != pivot) {
            const St* a = reinterpret_cast<const St*>(Yb + (size_t)(pivot * MBw + mm) * row_bytes +
                                                      so[pivot * MBw + mm]);
            const St* c = reinterpret_cast<const St*>(Yb + (size_t)(x * MBw + mm) * row_bytes + so[x * MBw + mm]);
            for (int e = half; e < s; e += 2) {
              Acc ar, ai, br, bi;
              ldY<Acc, St, CPLX>(a + 2 * e, ar, ai);
              ldY<Acc, St, CPLX>(c + 2 * e, br, bi);
              rd += ar * br + ai * bi;
              id += ar * bi - ai * br;
            }
          }
        }
        rd += __shfl_xor_sync(0xffffffffu, rd, 1);
        id += __shfl_xor_sync(0xffffffffu, id, 1);
        if (pr < npairs && half == 0) {
          Acc er = 1, ei = 0;
          if (CPLX && p.phase_allowed && x != pivot) {
            const Acc mag = sqrtf(rd * rd + id * id);
            if (mag > (Acc)0) {
              er = rd / mag;
              ei = -(id / mag);
            }
          }
          s_e[2 * (x * MBw + mm)] = er;
          s_e[2 * (x * MBw + mm) + 1] = ei;
        }
      }
      __syncwarp();
      // one (mode, element group) unit per lane over its q: with U < 32
      // units, lane slices of U lanes take every qs-th q of the warp's share
      const int U = mb * G;
      const int qs = U >= 32 ? 1 : 32 / U;
      const int lslice = U >= 32 ? 0 : lane / U;
      const int jstep = wq * qs, j0 = wslice * qs + lslice;
      if constexpr (SF) {
        float* sfo = reinterpret_cast<float*>(p.out);
        if (nslot == 8)
          warp_block_sf<8, St>(Yb, so, row_bytes, MBw, mb, G, s_e, pivot, s_w2, s_M2, s_rotf, s_ph, s_de, s_oq,
                               s_sq, s_qc, gb.sf_atoms, count, wslice, qs, wq, gamma, na, b0, sfo);
        else
          warp_block_sf<4, St>(Yb, so, row_bytes, MBw, mb, G, s_e, pivot, s_w2, s_M2, s_rotf, s_ph, s_de, s_oq,
                               s_sq, s_qc, gb.sf_atoms, count, wslice, qs, wq, gamma, na, b0, sfo);
      }
      for (int u = U >= 32 ? lane : lane % U; !SF && u < U && lslice < qs; u += 32) {
        const int mm = u / G, gi = u % G, bb = b0 + mm;
        const int e0 = gi < p.nsc ? gi : p.nsc + 3 * (gi - p.nsc);
        const int ne = gi < p.nsc ? 1 : 3;
        const long long row_off = (long long)bb * s * comps;
        if (nslot == 8)
          warp_unit<8, St, CPLX, Out>(Yb, so, row_bytes, MBw, mm, s_e, pivot, e0, ne, s_w2, s_M2, s_rotf, s_ph, s_de,
                                      s_oq, j0, count, jstep, gamma, na, gi - p.nsc, row_off, out);
        else
          warp_unit<4, St, CPLX, Out>(Yb, so, row_bytes, MBw, mm, s_e, pivot, e0, ne, s_w2, s_M2, s_rotf, s_ph, s_de,
                                      s_oq, j0, count, jstep, gamma, na, gi - p.nsc, row_off, out);
      }
      __syncwarp();  // the buffer may be refilled
      buf ^= 1;
    }
    // this warp's first block of the next group (both buffers are free)
    const GroupInfo& gn = s_g[cur ^ 1];
    if (ok && gn.count >= 0) {
      const WarpItem itn = warp_item<St, CPLX>(s_par[cur ^ 1], gb.e_modes, L.ybuf);
      const int wqn = itn.nblk >= nwarps ? 1 : nwarps / itn.nblk;
      if (warp < itn.nblk * wqn) issue(s_par[cur ^ 1], itn, gn, warp % itn.nblk, buf);
    }
    if (!ok && lane == 0) {
      atomicExch(&s_abort, 1);
      atomicOr(&p.err->flags, 1 << BRX_ERR_TIMEOUT);
      atomicAdd(&p.err->count, 1);
    }
    __syncthreads();  // records are no longer read
    cur ^= 1;
  }
  // no copy may land after exit
  for (int b = 0; b < 2; ++b)
    if (pending[b]) g_wait(mbar + 8 * b, phase[b]);
}

// Interpolated values of branch b for q at record index qi (batch-wide),
// written at output row qo.
template <typename Acc, typename St, bool CPLX, typename Out>
__device__ __forceinline__ void scalar_one(const GatherParams& p, long long qi, long long qo, int b) {
  using A = Ar<Acc>;
  constexpr int comps = CPLX ? 2 : 1;
  const St* data = reinterpret_cast<const St*>(p.data);
  Out* out = reinterpret_cast<Out*>(p.out);
  const int B = p.B, s = p.s;
  if (p.status[qi]) return;
  const int nw = p.nw[qi];
  const int piv = p.vidx[8 * qi];
  for (int e = 0; e < s; ++e) {
    Acc vr = 0, vi = 0;
    for (int x = 0; x < nw; ++x) {
      const int v = p.vidx[8 * qi + x];
      const int pid = perm_lookup(p, piv, v);
      const int row = pid >= 0 ? __ldg(p.perms + (long long)pid * B + b) : b;
      Acc dr, di;
      Ld<St, CPLX>::get(data, ((long long)v * B + row) * s + e, dr, di);
      const Acc w = sizeof(Acc) == 4 ? (Acc)p.w32[8 * qi + x] : (Acc)p.w[8 * qi + x];
      vr = A::add(vr, A::mul(w, dr));
      if (CPLX) vi = A::add(vi, A::mul(w, di));
    }
    Out* dst = out + ((size_t)qo * B + b) * (size_t)s * comps + (size_t)e * comps;
    dst[0] = (Out)vr;
    if (CPLX) dst[1] = (Out)vi;
  }
}

template <typename Acc, typename St, bool CPLX, typename Out>
__global__ void scalar_gather_kernel(GatherParams p) {
  const int B = p.B;
  const long long total = p.n * (long long)B;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const long long qi = it / B;
    scalar_one<Acc, St, CPLX, Out>(p, qi, qi, (int)(it % B));
  }
}

// FP32 scalar values without a permutation table, W consecutive branches
// per thread (B a multiple of W, 4W-byte aligned rows): the record is read
// once per W outputs, vertex rows and outputs move as float2/float4, and
// the indexing is 32-bit (a chunk holds at most 2^24 q, B ≤ 96).  Same sum
// order as scalar_one.
template <int W>
__global__ void scalar_gather_vec_kernel(GatherParams p) {
  using V = typename std::conditional<W == 4, float4, float2>::type;
  const int B = p.B, nch = B / W;
  const int total = (int)p.n * nch;
  const float* data = static_cast<const float*>(p.data);
  float* out = static_cast<float*>(p.out);
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < total; it += gridDim.x * blockDim.x) {
    const int qi = it / nch, c = it - qi * nch;
    if (p.status[qi]) continue;
    const int nw = p.nw[qi];
    float acc[W];
#pragma unroll
    for (int k = 0; k < W; ++k) acc[k] = 0.f;
    for (int x = 0; x < nw; ++x) {
      const int v = p.vidx[8 * qi + x];
      const float w = p.w32[8 * qi + x];
      const V d = __ldg(reinterpret_cast<const V*>(data + (size_t)v * B) + c);
      const float* dv = reinterpret_cast<const float*>(&d);
#pragma unroll
      for (int k = 0; k < W; ++k) acc[k] = Ar<float>::add(acc[k], Ar<float>::mul(w, dv[k]));
    }
    V o;
    float* ov = reinterpret_cast<float*>(&o);
#pragma unroll
    for (int k = 0; k < W; ++k) ov[k] = acc[k];
    reinterpret_cast<V*>(out + (size_t)qi * B)[c] = o;
  }
}

// Scalar-only items of a batch: one thread per (item, q, branch); qb_off[i]
// is the first pair of item i.
template <typename Acc, typename St, bool CPLX, typename Out>
__global__ void scalar_gather_batch_kernel(const GatherParams* items, const long long* qb_off, int n_items,
                                           long long total) {
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = n_items - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(qb_off + mid) <= it) lo = mid;
      else hi = mid - 1;
    }
    const GatherParams& p = items[lo];
    const long long local = it - __ldg(qb_off + lo);
    const long long qo = local / p.B;
    scalar_one<Acc, St, CPLX, Out>(p, p.q_base + qo, qo, (int)(local % p.B));
  }
}

// FP32 scalar values of a batch without permutation tables: one thread per
// (item, q, chunk of 4 branches), qc_off[i] the first chunk of item i; the
// record is read once per chunk, rows and outputs move as float4 where the
// item's B is a multiple of 4 and its data and output are 16-byte aligned,
// else element by element.  Same sum order as scalar_one.
__global__ void scalar_gather_batch_vec_kernel(const GatherParams* items, const long long* qc_off, int n_items,
                                               long long total) {
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = n_items - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(qc_off + mid) <= it) lo = mid;
      else hi = mid - 1;
    }
    const GatherParams& p = items[lo];
    const int B = p.B, nch = (B + 3) >> 2;
    const int local = (int)(it - __ldg(qc_off + lo));
    const int qo = local / nch, c = local - qo * nch;
    const long long qi = p.q_base + qo;
    if (p.status[qi]) continue;
    const int nw = p.nw[qi];
    const float* data = static_cast<const float*>(p.data);
    float* out = static_cast<float*>(p.out) + (size_t)qo * B + 4 * c;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    if ((B & 3) == 0 && (((uintptr_t)data | (uintptr_t)out) & 15) == 0) {
      for (int x = 0; x < nw; ++x) {
        const int v = p.vidx[8 * qi + x];
        const float w = p.w32[8 * qi + x];
        const float4 d = __ldg(reinterpret_cast<const float4*>(data + (size_t)v * B) + c);
        acc[0] = Ar<float>::add(acc[0], Ar<float>::mul(w, d.x));
        acc[1] = Ar<float>::add(acc[1], Ar<float>::mul(w, d.y));
        acc[2] = Ar<float>::add(acc[2], Ar<float>::mul(w, d.z));
        acc[3] = Ar<float>::add(acc[3], Ar<float>::mul(w, d.w));
      }
      *reinterpret_cast<float4*>(out) = make_float4(acc[0], acc[1], acc[2], acc[3]);
    } else {
      const int nb = min(4, B - 4 * c);
      for (int x = 0; x < nw; ++x) {
        const int v = p.vidx[8 * qi + x];
        const float w = p.w32[8 * qi + x];
        const float* row = data + (size_t)v * B + 4 * c;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (k < nb) acc[k] = Ar<float>::add(acc[k], Ar<float>::mul(w, __ldg(row + k)));
      }
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k < nb) out[k] = acc[k];
    }
  }
}

template <typename Acc, typename St, bool CPLX>
static size_t layout_bytes(const GatherParams& p, int MB) {
  const int na = p.rot_mode == ROT_GAMMA ? p.nvec : 0;
  return group_layout<Acc, St, CPLX>(p.qmax, MB, p.s, na).total;
}

size_t gather_smem_bytes(const GatherParams& p, int store_kind, bool cplx, int MB) {
  if (store_kind == ST_F64) return cplx ? layout_bytes<double, double, true>(p, MB) : layout_bytes<double, double, false>(p, MB);
  if (store_kind == ST_F32) return cplx ? layout_bytes<float, float, true>(p, MB) : layout_bytes<float, float, false>(p, MB);
  return cplx ? layout_bytes<float, __nv_bfloat16, true>(p, MB) : layout_bytes<float, __nv_bfloat16, false>(p, MB);
}

int gather_pick_modes(const GatherParams& p, int store_kind, bool cplx, size_t smem_budget) {
  int mb = p.B;
  while (mb > 1 && gather_smem_bytes(p, store_kind, cplx, mb) > smem_budget) mb = (mb + 1) / 2;
  // spread the modes evenly over the blocks
  const int nblk = (p.B + mb - 1) / mb;
  return (p.B + nblk - 1) / nblk;
}

// Launch shape of the warp-independent FP32 gather over n interpolators:
// vectors and scalars only, data at 16-byte aligned addresses with 16 bytes
// of slack at the end.  Shared memory is sized from the largest item: the
// first of (8 warps, then 4) × (modes per block from the most down to 1)
// within the budget per CTA, else the first the device holds.  Fills gb's
// layout fields and warps; false when the classic kernel must run.  Raises
// the kernel's shared-memory limit (not capturable: call before a stream
// capture).
template <typename St, bool CPLX, typename Out, bool SF = false>
static bool warp_plan(const GatherParams* P, int n, int qmax, size_t budget, GatherBatch* gb, size_t* smem_out,
                      int* per_sm_out) {
  const int comps = CPLX ? 2 : 1;
  int mmax = 1, na = 0;
  for (int i = 0; i < n; ++i) {
    const GatherParams& p = P[i];
    const int G = p.nsc + p.nvec;
    if (p.nmat != 0 || (uintptr_t)p.data % 16 != 0 || G < 1 || p.B < 1) return false;
    mmax = std::max(mmax, std::min(std::max(1, 32 / G), p.B));
    na = std::max(na, p.rot_mode == ROT_GAMMA ? p.nvec : 0);
  }
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // pass 0: the first shape within the budget; pass 1 (nothing fits the
  // budget): of the shapes the device holds, the most resident warps per
  // SM, then the most modes per block
  int best_w = 0, best_cap = 0, best_res = 0;
  for (int pass = 0; pass < 3; ++pass) {
    const size_t limit = pass == 0 ? std::min(budget, (size_t)optin) : (size_t)optin;
    for (int warps : {kWarpGatherMaxWarps, kWarpGatherMaxWarps / 2}) {
      for (int cap = mmax; cap >= 1; --cap) {
        if (pass == 2 && (warps != best_w || cap != best_cap)) continue;
        long long yb = 16;
        for (int i = 0; i < n; ++i) {
          const GatherParams& p = P[i];
          const int G = p.nsc + p.nvec;
          const int m = std::min(std::min(std::max(1, 32 / G), p.B), cap);
          yb = std::max(yb, 8LL * m * ((((long long)p.s * comps * (long long)sizeof(St) + 15) & ~15LL) + 16));
        }
        const int nsf = SF ? P[0].sf_atoms : 0;
        const size_t smem = warp_layout(qmax, cap, na, yb, warps, nsf).total;
        if (smem > limit) continue;
        cudaFuncSetAttribute(warp_gather_kernel<St, CPLX, Out, SF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, warp_gather_kernel<St, CPLX, Out, SF>, warps * 32,
                                                      smem);
        if (per_sm < 1) break;
        if (pass == 1) {
          if (per_sm * warps > best_res) {
            best_res = per_sm * warps;
            best_w = warps;
            best_cap = cap;
          }
          continue;
        }
        gb->qmax = qmax;
        gb->e_modes = cap;
        gb->ph_atoms = na;
        gb->ybuf = yb;
        gb->warps = warps;
        gb->sf_atoms = nsf;
        *smem_out = smem;
        *per_sm_out = per_sm;
        return true;
      }
    }
  }
  return false;
}

template <typename St, bool CPLX, typename Out>
static bool launch_warp(const GatherParams& p, int num_sms, size_t budget, cudaStream_t s) {
  if (p.variant == 1) return false;
  GatherBatch gb{};
  size_t smem = 0;
  int per_sm = 0;
  if (!warp_plan<St, CPLX, Out>(&p, 1, p.qmax, budget, &gb, &smem, &per_sm)) return false;
  gb.groups = p.groups;
  gb.n_groups = p.n_groups;
  gb.counter = p.counter;
  long long grid = (long long)num_sms * per_sm;
  if (grid > p.n) grid = p.n > 0 ? p.n : 1;
  warp_gather_kernel<St, CPLX, Out><<<(unsigned)grid, gb.warps * 32, smem, s>>>(p, gb);
  return true;
}

// The structure-factor gather (FP32 / BF16 complex vector data, no scalars
// beside the vectors, at most 32 atoms): false when it cannot run.
template <typename St>
static bool launch_sf_t(const GatherParams& p, int num_sms, size_t budget, cudaStream_t s) {
  if (p.nsc != 0 || p.nmat != 0 || p.nvec < 1 || p.nvec > 32 || p.nvec != p.sf_atoms) return false;
  GatherBatch gb{};
  size_t smem = 0;
  int per_sm = 0;
  // the most resident warps (its records are larger than the vectors gather's)
  (void)budget;
  if (!warp_plan<St, true, float, true>(&p, 1, p.qmax, 0, &gb, &smem, &per_sm)) return false;
  gb.groups = p.groups;
  gb.n_groups = p.n_groups;
  gb.counter = p.counter;
  long long grid = (long long)num_sms * per_sm;
  if (grid > p.n) grid = p.n > 0 ? p.n : 1;
  warp_gather_kernel<St, true, float, true><<<(unsigned)grid, gb.warps * 32, smem, s>>>(p, gb);
  return true;
}

template <typename Acc, typename St, bool CPLX, typename Out>
static void launch_t(const GatherParams& p, int num_sms, size_t budget, cudaStream_t s) {
  if (p.nvec == 0 && p.nmat == 0 && !p.phase_allowed) {
    if constexpr (std::is_same<Acc, float>::value && std::is_same<St, float>::value && !CPLX &&
                  std::is_same<Out, float>::value) {
      const int W = (p.B % 4 == 0) ? 4 : (p.B % 2 == 0 ? 2 : 0);
      const bool aligned = ((uintptr_t)p.data % (4 * W ? 4 * W : 1)) == 0 && ((uintptr_t)p.out % (4 * W ? 4 * W : 1)) == 0;
      if (W && aligned && p.s == 1 && p.n_keys == 0 && p.w32 && p.n * (long long)p.B < (1LL << 31)) {
        const long long total = p.n * (long long)(p.B / W);
        long long blocks = (total + 255) / 256;
        if (blocks > (long long)num_sms * 16) blocks = (long long)num_sms * 16;
        if (W == 4) scalar_gather_vec_kernel<4><<<(unsigned)blocks, 256, 0, s>>>(p);
        else scalar_gather_vec_kernel<2><<<(unsigned)blocks, 256, 0, s>>>(p);
        return;
      }
    }
    long long total = p.n * (long long)p.B;
    long long blocks = (total + 255) / 256;
    if (blocks > (long long)num_sms * 16) blocks = (long long)num_sms * 16;
    scalar_gather_kernel<Acc, St, CPLX, Out><<<(unsigned)blocks, 256, 0, s>>>(p);
    return;
  }
  if constexpr (sizeof(Acc) == 4)
    if (launch_warp<St, CPLX, Out>(p, num_sms, budget, s)) return;
  const size_t smem = layout_bytes<Acc, St, CPLX>(p, p.MB);
  // the limit belongs to the current device: set on every launch (a host
  // call, no stream work)
  cudaFuncSetAttribute(group_gather_kernel<Acc, St, CPLX, Out>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       200 * 1024);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, group_gather_kernel<Acc, St, CPLX, Out>, kGatherThreads,
                                                smem);
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)num_sms * per_sm;
  if (grid > p.n) grid = p.n > 0 ? p.n : 1;
  group_gather_kernel<Acc, St, CPLX, Out><<<(unsigned)grid, kGatherThreads, smem, s>>>(p);
}

template <typename Acc, typename St, bool CPLX, typename Out>
static cudaError_t preload_t() {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, group_gather_kernel<Acc, St, CPLX, Out>);
  if (e != cudaSuccess) return e;
  if constexpr (sizeof(Acc) == 4)
    if ((e = cudaFuncGetAttributes(&a, warp_gather_kernel<St, CPLX, Out>)) != cudaSuccess) return e;
  return cudaFuncGetAttributes(&a, scalar_gather_kernel<Acc, St, CPLX, Out>);
}

template <typename Acc, typename St>
static cudaError_t preload_store() {
  cudaError_t e;
  if ((e = preload_t<Acc, St, true, float>()) != cudaSuccess) return e;
  if ((e = preload_t<Acc, St, true, double>()) != cudaSuccess) return e;
  if ((e = preload_t<Acc, St, false, float>()) != cudaSuccess) return e;
  return preload_t<Acc, St, false, double>();
}

__global__ void key_hist_kernel(const int32_t* key, long long n, int32_t* counts);
__global__ void scan_reduce_kernel(const int32_t* in, long long m, int32_t* block_sums);
__global__ void scan_blocks_kernel(int32_t* block_sums, int nb);
__global__ void scan_apply_kernel(const int32_t* in, long long m, const int32_t* block_sums, int32_t* out,
                                  int32_t* out2);
__global__ void key_scatter_kernel(const int32_t* key, long long n, int32_t* cursor, int32_t* order);
__global__ void make_groups_kernel(const int32_t* counts, const int32_t* offsets, long long n_keys, int qmax,
                                   GroupDesc* groups, int32_t* n_groups, GroupSplit split, const int32_t* dpos0,
                                   const int32_t* dpos1);
__global__ void group_count_kernel(const int32_t* counts, long long n_keys, int qmax, GroupSplit split, int cls,
                                   int32_t* nd);

cudaError_t preload_grouping_kernels() {
  cudaFuncAttributes a;
  cudaError_t e;
  if ((e = cudaFuncGetAttributes(&a, key_hist_kernel)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&a, scan_reduce_kernel)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&a, scan_blocks_kernel)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&a, scan_apply_kernel)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&a, key_scatter_kernel)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&a, group_count_kernel)) != cudaSuccess) return e;
  return cudaFuncGetAttributes(&a, make_groups_kernel);
}

cudaError_t preload_locate_kernel();

cudaError_t preload_query_kernels() {
  cudaError_t e;
  cudaFuncAttributes a;
  if ((e = cudaFuncGetAttributes(&a, scalar_gather_vec_kernel<4>)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&a, scalar_gather_vec_kernel<2>)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&a, scalar_gather_batch_vec_kernel)) != cudaSuccess) return e;
  if ((e = preload_store<double, double>()) != cudaSuccess) return e;
  if ((e = preload_store<float, float>()) != cudaSuccess) return e;
  if ((e = preload_store<float, __nv_bfloat16>()) != cudaSuccess) return e;
  if ((e = preload_grouping_kernels()) != cudaSuccess) return e;
  return preload_locate_kernel();
}

// Antiphase of every (key, mode) of FP64 complex data: key k = i·N + j
// names the pivot vertex i and the vertex j; row b of i against row
// perm_ij(b) of j, with the arithmetic and the order of the group gather's
// own antiphase loop (so a factor read from the table equals the one the
// loop forms), e = conj(z)/|z| with z = Σ_e conj(a_e)·c_e.
__global__ void phase_table_kernel(GatherParams p, const long long* keys, long long n_keys, double2* out) {
  using A = Ar<double>;
  const double* data = static_cast<const double*>(p.data);
  const int B = p.B, s = p.s;
  const long long total = n_keys * (long long)B;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long k = t / B;
    const int b = (int)(t - k * B);
    const long long key = __ldg(keys + k);
    const long long i = key / p.n_vertices, j = key - i * p.n_vertices;
    const int pid = perm_lookup(p, i, j);
    const int row = pid >= 0 ? __ldg(p.perms + (long long)pid * B + b) : b;
    const double2* a = reinterpret_cast<const double2*>(data + (i * B + b) * (long long)s * 2);
    const double2* c = reinterpret_cast<const double2*>(data + (j * B + row) * (long long)s * 2);
    double rd = 0, id = 0;
    for (int e = 0; e < s; ++e) {
      const double2 x = __ldg(a + e), y = __ldg(c + e);
      rd = A::add(rd, A::add(A::mul(x.x, y.x), A::mul(x.y, y.y)));
      id = A::add(id, A::sub(A::mul(x.x, y.y), A::mul(x.y, y.x)));
    }
    const double mag = sqrt(A::add(A::mul(rd, rd), A::mul(id, id)));
    double2 r = make_double2(1.0, 0.0);
    if (mag > 0.0) r = make_double2(rd / mag, -(id / mag));
    out[t] = r;
  }
}

void launch_phase_table(const GatherParams& p, const long long* keys, long long n_keys, double2* out,
                        cudaStream_t s) {
  const long long total = n_keys * (long long)p.B;
  if (total <= 0) return;
  long long blocks = (total + 255) / 256;
  if (blocks > 152LL * 64) blocks = 152LL * 64;
  phase_table_kernel<<<(unsigned)blocks, 256, 0, s>>>(p, keys, n_keys, out);
}

int launch_structure_factor(const GatherParams& p, int store_kind, int num_sms, size_t budget, cudaStream_t s) {
  if (p.n <= 0) return 0;
  if (store_kind == ST_F64) return -1;
  cudaMemsetAsync(p.counter, 0, sizeof(int32_t), s);
  const bool ok = store_kind == ST_F32 ? launch_sf_t<float>(p, num_sms, budget, s)
                                       : launch_sf_t<__nv_bfloat16>(p, num_sms, budget, s);
  return ok ? 1 : -1;
}

int launch_gather(const GatherParams& p, int store_kind, bool cplx, bool out_f32, int num_sms, size_t budget,
                  cudaStream_t s) {
  if (p.n <= 0) return 0;
  cudaMemsetAsync(p.counter, 0, sizeof(int32_t), s);
#define BRX_DISPATCH(ACC, ST)                                                     \
  do {                                                                            \
    if (cplx) {                                                                   \
      if (out_f32) launch_t<ACC, ST, true, float>(p, num_sms, budget, s);                 \
      else launch_t<ACC, ST, true, double>(p, num_sms, budget, s);                        \
    } else {                                                                      \
      if (out_f32) launch_t<ACC, ST, false, float>(p, num_sms, budget, s);                \
      else launch_t<ACC, ST, false, double>(p, num_sms, budget, s);                       \
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
// batched launches
// ---------------------------------------------------------------------------
#define BRX_STORE_TYPES(STORE, ...)                                                      \
  do {                                                                                   \
    if ((STORE) == ST_F64) { using Acc = double; using St = double; __VA_ARGS__; }       \
    else if ((STORE) == ST_F32) { using Acc = float; using St = float; __VA_ARGS__; }    \
    else { using Acc = float; using St = __nv_bfloat16; __VA_ARGS__; }                   \
  } while (0)

size_t gather_batch_smem(int store_kind, bool cplx, int qmax, int e_modes, int ph_atoms, long long ybuf) {
  size_t r = 0;
  (void)cplx;
  BRX_STORE_TYPES(store_kind, r = group_layout_dims<Acc, St>(qmax, e_modes, ph_atoms, ybuf).total);
  return r;
}

long long gather_ybuf(int store_kind, bool cplx, int MB, int s) {
  long long r = 0;
  BRX_STORE_TYPES(store_kind, r = cplx ? 8LL * MB * row_stride<St, true>(s) : 8LL * MB * row_stride<St, false>(s));
  return r;
}

template <typename Acc, typename St, bool CPLX, typename Out>
static int batch_ctas(size_t smem) {
  cudaFuncSetAttribute(group_gather_batch_kernel<Acc, St, CPLX, Out>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       200 * 1024);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, group_gather_batch_kernel<Acc, St, CPLX, Out>,
                                                kGatherThreads, smem);
  return per_sm;
}

bool gather_warp_plan(int store_kind, bool cplx, bool out_f32, const GatherParams* items, int n, int qmax,
                      size_t budget, GatherBatch* gb, size_t* smem, int* ctas_per_sm) {
  if (store_kind == ST_F64) return false;
  bool r = false;
  BRX_STORE_TYPES(store_kind, {
    if constexpr (sizeof(Acc) == 4) {
      if (cplx) r = out_f32 ? warp_plan<St, true, float>(items, n, qmax, budget, gb, smem, ctas_per_sm)
                            : warp_plan<St, true, double>(items, n, qmax, budget, gb, smem, ctas_per_sm);
      else r = out_f32 ? warp_plan<St, false, float>(items, n, qmax, budget, gb, smem, ctas_per_sm)
                       : warp_plan<St, false, double>(items, n, qmax, budget, gb, smem, ctas_per_sm);
    }
  });
  return r;
}

long long gather_shape_key(const GatherParams& p, int store_kind, bool cplx, bool out_f32, size_t budget) {
  if (p.variant != 1) {
    GatherBatch gb{};
    size_t smem = 0;
    int ctas = 0;
    if (gather_warp_plan(store_kind, cplx, out_f32, &p, 1, p.qmax, budget, &gb, &smem, &ctas))
      return (1LL << 48) | ((long long)p.qmax << 32) | ((long long)gb.warps << 24) | ((long long)gb.e_modes << 12) |
             (long long)ctas;
  }
  return (2LL << 48) | ((long long)p.qmax << 32) | (long long)gather_pick_modes(p, store_kind, cplx, budget);
}

int gather_max_ctas(int store_kind, bool cplx, bool out_f32, size_t smem) {
  int r = 0;
  BRX_STORE_TYPES(store_kind, {
    if (cplx) r = out_f32 ? batch_ctas<Acc, St, true, float>(smem) : batch_ctas<Acc, St, true, double>(smem);
    else r = out_f32 ? batch_ctas<Acc, St, false, float>(smem) : batch_ctas<Acc, St, false, double>(smem);
  });
  return r;
}

// ctas: CTAs per SM, from gather_max_ctas (which also raises the kernel's
// shared-memory limit); nothing here but the launch, so that a stream
// capture can record it
template <typename Acc, typename St, bool CPLX, typename Out>
static void batch_launch_t(const GatherBatch& gb, int num_sms, size_t smem, int ctas, cudaStream_t s) {
  if (ctas < 1) ctas = 1;
  if constexpr (sizeof(Acc) == 4) {
    if (gb.warps > 0) {
      warp_gather_kernel<St, CPLX, Out><<<(unsigned)(num_sms * ctas), gb.warps * 32, smem, s>>>(GatherParams{}, gb);
      return;
    }
  }
  group_gather_batch_kernel<Acc, St, CPLX, Out><<<(unsigned)(num_sms * ctas), kGatherThreads, smem, s>>>(gb);
}

void launch_gather_batch(const GatherBatch& gb, int store_kind, bool cplx, bool out_f32, int num_sms, size_t smem,
                         int ctas_per_sm, cudaStream_t s) {
  cudaMemsetAsync(gb.counter, 0, sizeof(int32_t), s);
  BRX_STORE_TYPES(store_kind, {
    if (cplx) {
      if (out_f32) batch_launch_t<Acc, St, true, float>(gb, num_sms, smem, ctas_per_sm, s);
      else batch_launch_t<Acc, St, true, double>(gb, num_sms, smem, ctas_per_sm, s);
    } else {
      if (out_f32) batch_launch_t<Acc, St, false, float>(gb, num_sms, smem, ctas_per_sm, s);
      else batch_launch_t<Acc, St, false, double>(gb, num_sms, smem, ctas_per_sm, s);
    }
  });
}

void launch_scalar_batch_vec(const GatherParams* items, const long long* qc_off, int n_items, long long total,
                             int num_sms, cudaStream_t s) {
  if (total <= 0) return;
  long long blocks = (total + 255) / 256;
  if (blocks > (long long)num_sms * 16) blocks = (long long)num_sms * 16;
  scalar_gather_batch_vec_kernel<<<(unsigned)blocks, 256, 0, s>>>(items, qc_off, n_items, total);
}

void launch_scalar_batch(const GatherParams* items, const long long* qb_off, int n_items, long long total,
                         int store_kind, bool cplx, bool out_f32, int num_sms, cudaStream_t s) {
  if (total <= 0) return;
  long long blocks = (total + 255) / 256;
  if (blocks > (long long)num_sms * 16) blocks = (long long)num_sms * 16;
  BRX_STORE_TYPES(store_kind, {
    if (cplx) {
      if (out_f32) scalar_gather_batch_kernel<Acc, St, true, float><<<(unsigned)blocks, 256, 0, s>>>(items, qb_off, n_items, total);
      else scalar_gather_batch_kernel<Acc, St, true, double><<<(unsigned)blocks, 256, 0, s>>>(items, qb_off, n_items, total);
    } else {
      if (out_f32) scalar_gather_batch_kernel<Acc, St, false, float><<<(unsigned)blocks, 256, 0, s>>>(items, qb_off, n_items, total);
      else scalar_gather_batch_kernel<Acc, St, false, double><<<(unsigned)blocks, 256, 0, s>>>(items, qb_off, n_items, total);
    }
  });
}
#undef BRX_STORE_TYPES

// ---------------------------------------------------------------------------
// grouping: counting sort of q by group key, then one work descriptor per
// group (at most qmax q each)
// ---------------------------------------------------------------------------
// Lanes of a warp holding the same key add once, through their lowest lane:
// trellises with few tetrahedra put millions of q on a handful of keys.
__global__ void key_hist_kernel(const int32_t* key, long long n, int32_t* counts) {
  const int lane = threadIdx.x & 31;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int32_t k = key[i];
    const unsigned peers = __match_any_sync(__activemask(), k);
    if (lane == __ffs(peers) - 1) atomicAdd(counts + k, __popc(peers));
  }
}

constexpr int kScanThreads = 1024, kScanPer = 8;

// exclusive scan, three passes: block sums, scan of block sums, block scans
__global__ void scan_reduce_kernel(const int32_t* in, long long m, int32_t* block_sums) {
  __shared__ int32_t red[kScanThreads];
  const long long base = (long long)blockIdx.x * kScanThreads * kScanPer;
  int32_t s = 0;
  for (int k = 0; k < kScanPer; ++k) {
    long long i = base + (long long)k * kScanThreads + threadIdx.x;
    if (i < m) s += in[i];
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int off = kScanThreads / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = red[0];
}

__global__ void scan_blocks_kernel(int32_t* block_sums, int nb) {
  if (threadIdx.x == 0) {
    int32_t run = 0;
    for (int i = 0; i < nb; ++i) {
      int32_t v = block_sums[i];
      block_sums[i] = run;
      run += v;
    }
  }
}

__global__ void scan_apply_kernel(const int32_t* in, long long m, const int32_t* block_sums, int32_t* out,
                                  int32_t* out2) {
  __shared__ int32_t tsum[kScanThreads];
  const long long base = (long long)blockIdx.x * kScanThreads * kScanPer;
  // each thread owns kScanPer consecutive elements
  int32_t loc[kScanPer];
  int32_t s = 0;
  for (int k = 0; k < kScanPer; ++k) {
    long long i = base + (long long)threadIdx.x * kScanPer + k;
    loc[k] = i < m ? in[i] : 0;
    s += loc[k];
  }
  tsum[threadIdx.x] = s;
  __syncthreads();
  // Hillis–Steele inclusive scan of the thread sums
  for (int off = 1; off < kScanThreads; off <<= 1) {
    int32_t v = threadIdx.x >= off ? tsum[threadIdx.x - off] : 0;
    __syncthreads();
    tsum[threadIdx.x] += v;
    __syncthreads();
  }
  int32_t run = block_sums[blockIdx.x] + (threadIdx.x ? tsum[threadIdx.x - 1] : 0);
  for (int k = 0; k < kScanPer; ++k) {
    long long i = base + (long long)threadIdx.x * kScanPer + k;
    if (i < m) {
      out[i] = run;
      if (out2) out2[i] = run;
    }
    run += loc[k];
  }
}

__global__ void key_scatter_kernel(const int32_t* key, long long n, int32_t* cursor, int32_t* order) {
  const int lane = threadIdx.x & 31;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int32_t k = key[i];
    const unsigned peers = __match_any_sync(__activemask(), k);
    const int leader = __ffs(peers) - 1;
    int pos = 0;
    if (lane == leader) pos = atomicAdd(cursor + k, __popc(peers));
    pos = __shfl_sync(peers, pos, leader) + __popc(peers & ((1u << lane) - 1u));
    order[pos] = (int32_t)i;
  }
}

// Class of key k: 1 for keys of a class-1 item of the split, else 0.
__device__ __forceinline__ int key_class(const GroupSplit& split, long long k) {
  if (!split.item_class) return 0;
  int lo = 0, hi = split.n_items - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(split.key_off + mid) <= k) lo = mid;
    else hi = mid - 1;
  }
  return __ldg(split.item_class + lo) == 1 ? 1 : 0;
}

// Work descriptors of every key of class cls (one per qm q), 0 elsewhere and
// in the last bucket (failed q): m = n_keys + 1 entries.
__global__ void group_count_kernel(const int32_t* counts, long long n_keys, int qmax, GroupSplit split, int cls,
                                   int32_t* nd) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k <= n_keys;
       k += (long long)gridDim.x * blockDim.x) {
    int v = 0;
    const int c = k < n_keys ? counts[k] : 0;
    if (c > 0 && key_class(split, k) == cls) {
      const int qm = cls ? split.qmax : qmax;
      v = (c + qm - 1) / qm;
    }
    nd[k] = v;
  }
}

// One work descriptor per qmax q of every key, at the key's place in the
// exclusive scans dpos0 (class 0) and dpos1 (class 1) of the descriptor
// counts, so descriptors follow key order (the gathers take them in that
// order, and neighbouring keys share vertex rows).  With split.item_class
// set, keys of class-1 items take split.qmax q per descriptor and go to the
// second list, written downwards from split.groups_end.
__global__ void make_groups_kernel(const int32_t* counts, const int32_t* offsets, long long n_keys, int qmax,
                                   GroupDesc* groups, int32_t* n_groups, GroupSplit split, const int32_t* dpos0,
                                   const int32_t* dpos1) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *n_groups = dpos0[n_keys];
    if (split.item_class) *split.n_groups = dpos1[n_keys];
  }
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n_keys; k += (long long)gridDim.x * blockDim.x) {
    const int c = counts[k];
    if (c <= 0) continue;
    const bool second = key_class(split, k) == 1;
    const int qm = second ? split.qmax : qmax;
    const int nd = (c + qm - 1) / qm;
    const int slot = second ? dpos1[k] : dpos0[k];
    for (int d = 0; d < nd; ++d) {
      GroupDesc g;
      g.key = (int32_t)k;
      g.start = offsets[k] + d * qm;
      g.count = min(qm, c - d * qm);
      if (second) split.groups_end[-1 - (slot + d)] = g;
      else groups[slot + d] = g;
    }
  }
}

size_t group_scratch_ints(long long n_keys) {
  const long long m = n_keys + 1;
  const long long nb = (m + kScanThreads * kScanPer - 1) / (kScanThreads * kScanPer);
  return (size_t)(5 * m + nb + 8);
}

int launch_grouping(const int32_t* key, long long n, long long n_keys, int qmax, int32_t* scratch, int32_t* order,
                    GroupDesc* groups, int32_t* n_groups, cudaStream_t s, const GroupSplit& split) {
  if (n <= 0) return 0;
  const long long m = n_keys + 1;  // last bucket: failed q
  const long long nb = (m + kScanThreads * kScanPer - 1) / (kScanThreads * kScanPer);
  int32_t* counts = scratch;
  int32_t* offsets = scratch + m;
  int32_t* cursor = scratch + 2 * m;
  int32_t* bsums = scratch + 3 * m;
  int32_t* dpos0 = scratch + 3 * m + nb;
  int32_t* dpos1 = dpos0 + m;
  cudaMemsetAsync(counts, 0, sizeof(int32_t) * m, s);
  long long blocks = (n + 255) / 256;
  if (blocks > 8192) blocks = 8192;
  key_hist_kernel<<<(unsigned)blocks, 256, 0, s>>>(key, n, counts);
  scan_reduce_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(counts, m, bsums);
  scan_blocks_kernel<<<1, 32, 0, s>>>(bsums, (int)nb);
  scan_apply_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(counts, m, bsums, offsets, cursor);
  key_scatter_kernel<<<(unsigned)blocks, 256, 0, s>>>(key, n, cursor, order);
  long long kb = (m + 255) / 256;
  if (kb > 8192) kb = 8192;
  int launches = 5;
  // descriptor positions per class: counts into the free cursor array, then
  // an exclusive scan
  for (int cls = 0; cls < (split.item_class ? 2 : 1); ++cls) {
    int32_t* dpos = cls ? dpos1 : dpos0;
    group_count_kernel<<<(unsigned)kb, 256, 0, s>>>(counts, n_keys, qmax, split, cls, cursor);
    scan_reduce_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(cursor, m, bsums);
    scan_blocks_kernel<<<1, 32, 0, s>>>(bsums, (int)nb);
    scan_apply_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(cursor, m, bsums, dpos, nullptr);
    launches += 4;
  }
  make_groups_kernel<<<(unsigned)kb, 256, 0, s>>>(counts, offsets, n_keys, qmax, groups, n_groups, split, dpos0,
                                                  dpos1);
  return launches + 1;
}

}  // namespace brx
