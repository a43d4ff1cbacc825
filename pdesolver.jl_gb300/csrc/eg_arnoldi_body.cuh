// eg_arnoldi_body.cuh -- the persistent GMRES solve as a device function,
// shared by the single-problem cooperative kernel (eg_arnoldi.cu) and the
// batched kernel that runs several problems' solves in one launch
// (eg_arnoldi_batch.cu).  The algorithm and its data flow are described in
// eg_arnoldi.cu.
#pragma once
#include <cooperative_groups.h>

#include <algorithm>

#include "eg_internal.h"
#include "eg_kernels.cuh"
#include "eg_krylov.cuh"
#include "eg_linalg.h"
#include "eg_tma.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int NT = 512;  // one block per SM (16 warps, up to 128 registers a thread)
constexpr int NW = NT / 32;
constexpr int NB_MAX = 64;  // coupling-block rows handled by the face-side pass
// systems whose element blocks take at most this many bytes run on one block
constexpr size_t kSmallOperatorBytes = size_t(2) << 20;

constexpr int PSTRIDE = 33;  // partial slots per block

// dynamic shared memory of one block, at most (the static GmresShared block
// comes on top, within the 227 KB of an SM)
constexpr size_t kSmemMax = 200 * 1024;
// bytes of operator copies in flight per block (the ring of slots), at most
constexpr size_t kRingBudget = 160 * 1024;
// target bytes of one ring slot (elements per slot chosen to reach it)
constexpr size_t kSlotTarget = 12 * 1024;

// Operator ring of the Arnoldi apply: the block's elements are cut into units
// of `eps` consecutive elements, each unit's operator data (its inverse
// blocks, one contiguous range, and for 2-D dense coupling the neighbours'
// coupling blocks of its faces) is one set of bulk copies into a slot of a
// ring of nslot slots.  One producer thread keeps the slots filled (full /
// empty mbarrier pairs) and runs ahead into the next Arnoldi iteration's
// first units, so those copies are in flight during the grid barriers and
// vector passes; ngroup consumer groups of wpg warps compute z = D^-1 v and
// push C z from the slots.  When all of a block's units fit in the ring it is
// resident: loaded once for the whole solve.
struct RingCfg {
  int on;          // 1: the Arnoldi apply runs through the ring
  int nslot;       // slots of the ring
  int resident;    // 1: every unit has its own slot, loaded once
  int eps;         // elements per unit
  int ngroup;      // consumer groups
  int wpg;         // warps per consumer group
  int cpl_tma;     // coupling blocks arrive in the slot (2-D dense coupling)
  int slot_bytes;  // bytes of one slot (multiple of 128)
  int inv_cap;     // bytes of a slot's inverse-block region (multiple of 16)
  int cpl_bytes;   // bytes of one coupling block
  int fside_smem;  // the block's [epb][F] face-side table is staged in shared memory
  int vj_smem;     // the block's rows of v_j are staged in shared memory per apply
  // dynamic shared memory offsets (bytes)
  int off_ring, off_bar, off_z, off_v, off_vj, off_red, off_fside, off_sz;
};

template <typename T>
struct CoopArgs {
  DevMesh md;
  const T* inv;      // [E][n][n] block inverses (column-major)
  const T* diag;     // [E][n][n] element blocks of J (column-major)
  const T* cpl;      // [I][2][nb][nb] coupling blocks (row-major), or
                     // [I][2][S][NV][NV] when md.sparse_face (face-diagonal)
  const int* spos;   // [F][Np]
  const int* fside;  // [E][F] coupling block of each element face, or -1
  T* cfs;            // [I][2][nb] coupling products of each face side
  const T* bvec;     // [N] right-hand side
  T* x;              // [N] solution (in: initial guess)
  T* V;              // [(m+1)][N]
  T* w;              // [N]
  T* part;           // [4][gridDim][PSTRIDE]
  int* flags;
  double* scal;
  int m, n, E;
  int nb, S, F, nv, ec;  // coupling block size, stencil size, faces, variables, elements per chunk
  int64_t N;
  RingCfg rc;
};

// NV consecutive values of a coupling row (16-byte loads for 2-D FP32)
template <int NV, typename T>
__device__ __forceinline__ void load_row_piece(const T* __restrict__ p, T* out) {
  if constexpr (NV == 4 && sizeof(T) == 4) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = v.w;
  } else {
#pragma unroll
    for (int b = 0; b < NV; ++b) out[b] = p[b];
  }
}

// Push of the coupling of elements c0 .. c0+nl-1 to their neighbours: for
// each interface face f of element e with coupling block fs = slot*2 + side,
// the neighbour's block fs ^ 1 (rows: the neighbour's stencil, columns: e's
// stencil on f) times e's values z_e (shared memory) goes to cfs[fs ^ 1].
// A group of G lanes (16 when nb <= 16, else 32) owns one face; lane gl
// streams rows gl, gl + G, ... of the row-major block.
template <int DIM, typename T>
__device__ void face_push(const CoopArgs<T>& a, const T* __restrict__ sZ, const int* __restrict__ sPerm,
                          int c0, int nl, T* __restrict__ cfs) {
  constexpr int NV = DIM + 2;
  const int nb = a.nb, F = a.F, S = a.S, n = a.n;
  const int G = nb <= 16 ? 16 : 32, gpw = 32 / G;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane / G, gl = lane - grp * G;
  const int ntask = nl * F;
  for (int t = warp * gpw + grp; t < ntask; t += (NT / 32) * gpw) {
    const int le = t / F, f = t - le * F;
    const int fs = a.fside[(int64_t)(c0 + le) * F + f];
    if (fs < 0) continue;
    const int tgt = fs ^ 1;
    const T* zs = sZ + (size_t)le * n;
    const int* pf = sPerm + f * S;
    if (a.md.sparse_face) {
      // face-diagonal coupling [I][2][S][NV][NV]: row (s, r) of the
      // neighbour's side couples to this element's node facing s only
      const int o = a.md.ifaces[5 * (tgt >> 1) + 4];
      const int* facing = (tgt & 1) ? a.md.nbrinv + o * a.md.Nf : a.md.nbrperm + o * a.md.Nf;
      for (int i = gl; i < nb; i += G) {
        const int s = i / NV;
        const T* Cr = a.cpl + (size_t)tgt * nb * NV + (size_t)i * NV;
        const T* zz = zs + pf[facing[s]] * NV;
        T c[NV];
        load_row_piece<NV, T>(Cr, c);
        T acc = T(0);
#pragma unroll
        for (int b = 0; b < NV; ++b) acc += c[b] * zz[b];
        cfs[(size_t)tgt * nb + i] = acc;
      }
      continue;
    }
    for (int i = gl; i < nb; i += G) {
      const T* Cr = a.cpl + ((size_t)tgt * nb + i) * nb;
      T acc0 = T(0), acc1 = T(0);
#pragma unroll 4
      for (int sp = 0; sp < S; ++sp) {
        T c[NV];
        load_row_piece<NV, T>(Cr + sp * NV, c);
        const T* zz = zs + pf[sp] * NV;
#pragma unroll
        for (int b = 0; b < NV; ++b) {
          if (b & 1) acc1 += c[b] * zz[b];
          else acc0 += c[b] * zz[b];
        }
      }
      cfs[(size_t)tgt * nb + i] = acc0 + acc1;
    }
  }
}

__device__ __forceinline__ float wsum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// vector type for the streaming passes over a block's rows: 16-byte loads
template <typename T> struct Vec;
template <> struct Vec<float> {
  using V = float4;
  static constexpr int W = 4;
  __device__ static float dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
  __device__ static V fma(V a, float h, V c) {
    return make_float4(c.x - a.x * h, c.y - a.y * h, c.z - a.z * h, c.w - a.w * h);
  }
  __device__ static V scale(V a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
};
template <> struct Vec<double> {
  using V = double2;
  static constexpr int W = 2;
  __device__ static double dot(V a, V b) { return a.x * b.x + a.y * b.y; }
  __device__ static V fma(V a, double h, V c) { return make_double2(c.x - a.x * h, c.y - a.y * h); }
  __device__ static V scale(V a, double s) { return make_double2(a.x * s, a.y * s); }
};

// partial dots of the block's rows: k < cnt against V[k], k == cnt: x.x
// (when with_xx); warp q owns k = q, q + 16, ...  Rows in units of
// Vec<T>::W when `vec` (the row range and the vector stride are multiples of
// W), else scalar.
template <typename T>
__device__ void block_dots(const T* __restrict__ V, const T* __restrict__ x, int cnt, int with_xx,
                           int64_t N, int64_t r0, int nrow, bool vec, T* __restrict__ pb) {
  using VT = Vec<T>;
  const int lane = threadIdx.x & 31, q = threadIdx.x >> 5;
  const int tot = cnt + (with_xx ? 1 : 0);
  for (int k = q; k < tot; k += NT / 32) {
    const T* v = (k < cnt) ? V + (size_t)k * N + r0 : x + r0;
    const T* xr = x + r0;
    T acc0 = T(0), acc1 = T(0);
    if (vec) {
      const typename VT::V* v4 = reinterpret_cast<const typename VT::V*>(v);
      const typename VT::V* x4 = reinterpret_cast<const typename VT::V*>(xr);
      const int n4 = nrow / VT::W;
      int i = lane;
      for (; i + 32 < n4; i += 64) {
        acc0 += VT::dot(v4[i], x4[i]);
        acc1 += VT::dot(v4[i + 32], x4[i + 32]);
      }
      if (i < n4) acc0 += VT::dot(v4[i], x4[i]);
    } else {
      for (int i = lane; i < nrow; i += 32) acc0 += v[i] * xr[i];
    }
    const T acc = wsum(acc0 + acc1);
    if (lane == 0) pb[k] = acc;
  }
}

// every block: out[k] = sum_b part[b][k] for k < cnt, in block order
template <typename T>
__device__ void block_reduce_all(const T* __restrict__ part, int nblk, int cnt, T* __restrict__ out) {
  const int lane = threadIdx.x & 31, q = threadIdx.x >> 5;
  for (int k = q; k < cnt; k += NT / 32) {
    T v = T(0);
    for (int b = lane; b < nblk; b += 32) v += part[(size_t)b * PSTRIDE + k];
    v = wsum(v);
    if (lane == 0) out[k] = v;
  }
}

// y = (x - sum_{k<cnt} V[k] h[k]) * s on the block's rows, by threads
// t0 .. NT-1 (x and y may alias).  The basis loads of a row are issued in
// batches of 16 before their updates (one round trip to L2 per batch); the
// sum runs over k in order.
template <typename T>
__device__ void block_sub_scale(const T* __restrict__ V, const T* __restrict__ h, int cnt, int64_t N,
                                const T* x, T s, T* y, int64_t r0, int nrow, bool vec, int t0) {
  using VT = Vec<T>;
  if (vec) {
    const int n4 = nrow / VT::W;
    for (int i = threadIdx.x - t0; i < n4; i += NT - t0) {
      const int64_t row = r0 + (int64_t)i * VT::W;
      typename VT::V a = *reinterpret_cast<const typename VT::V*>(x + row);
      for (int k0 = 0; k0 < cnt; k0 += 4) {
        typename VT::V v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (k0 + q < cnt) v[q] = *reinterpret_cast<const typename VT::V*>(V + (size_t)(k0 + q) * N + row);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (k0 + q < cnt) a = VT::fma(v[q], h[k0 + q], a);
      }
      *reinterpret_cast<typename VT::V*>(y + row) = VT::scale(a, s);
    }
  } else {
    for (int i = threadIdx.x - t0; i < nrow; i += NT - t0) {
      const int64_t row = r0 + i;
      T a = x[row];
      for (int k0 = 0; k0 < cnt; k0 += 16) {
        T v[16];
#pragma unroll
        for (int q = 0; q < 16; ++q)
          if (k0 + q < cnt) v[q] = V[(size_t)(k0 + q) * N + row];
#pragma unroll
        for (int q = 0; q < 16; ++q)
          if (k0 + q < cnt) a -= v[q] * h[k0 + q];
      }
      y[row] = a * s;
    }
  }
}

// u = sum_{k<cnt} V[k] y[k] on the block's rows
template <typename T>
__device__ void block_lincomb(const T* __restrict__ V, const T* __restrict__ y, int cnt, int64_t N,
                              T* __restrict__ u, int64_t r0, int nrow) {
  for (int i = threadIdx.x; i < nrow; i += NT) {
    const int64_t row = r0 + i;
    T a0 = T(0), a1 = T(0);
    int k = 0;
    for (; k + 2 <= cnt; k += 2) {
      a0 += V[(size_t)k * N + row] * y[k];
      a1 += V[(size_t)(k + 1) * N + row] * y[k + 1];
    }
    if (k < cnt) a0 += V[(size_t)k * N + row] * y[k];
    u[row] = a0 + a1;
  }
}

// W consecutive values of one row unit
template <typename T, int W>
struct Pack {
  T v[W];
};
template <typename T, int W>
__device__ __forceinline__ Pack<T, W> ldp(const T* p) {
  Pack<T, W> r;
  if constexpr (W == 4 && sizeof(T) == 4) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    r.v[0] = q.x; r.v[1] = q.y; r.v[2] = q.z; r.v[3] = q.w;
  } else if constexpr (W == 2 && sizeof(T) == 8) {
    const double2 q = *reinterpret_cast<const double2*>(p);
    r.v[0] = q.x; r.v[1] = q.y;
  } else {
#pragma unroll
    for (int c = 0; c < W; ++c) r.v[c] = p[c];
  }
  return r;
}
template <typename T, int W>
__device__ __forceinline__ void stp(T* p, const Pack<T, W>& r) {
  if constexpr (W == 4 && sizeof(T) == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
  } else if constexpr (W == 2 && sizeof(T) == 8) {
    *reinterpret_cast<double2*>(p) = make_double2(r.v[0], r.v[1]);
  } else {
#pragma unroll
    for (int c = 0; c < W; ++c) p[c] = r.v[c];
  }
}

// Sum of v[k] over the 32 lanes for each of the KC slots (KC a power of two,
// at most 32), as a transposed butterfly (KC - 1 shuffles for KC = 32):
// afterwards lane l holds the sum of slot l * KC / 32 (the 32 / KC lanes
// l with equal l * KC / 32 hold the same sum).
template <typename T, int KC>
__device__ __forceinline__ void transpose_reduce(T (&v)[KC], int lane) {
  int o = 16;
#pragma unroll
  for (int c = KC; c > 1; c >>= 1, o >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < c / 2; ++i) {
      const T send = up ? v[i] : v[i + c / 2];
      const T keep = up ? v[i + c / 2] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
#pragma unroll
  for (; o > 0; o >>= 1) v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
}

// Partial sums of the block's rows for one Gram-Schmidt reduction:
// pb[k] = V_k . w for k < cnt and pb[cnt] = w . w.  With `gather`, w is
// formed first from the pushed coupling products, w = v_j + the products of
// the faces holding the row's node, and written to a.w.  Each thread owns
// whole row units (W consecutive values) and keeps the sums of all slots in
// registers, so the loads of every basis vector of its rows are in flight
// together; lanes are combined by a transposed butterfly and warps through
// shared memory, always in the same order.
template <int DIM, typename T, int W>
__device__ void gs_dots_w(const CoopArgs<T>& a, const T* __restrict__ vj, bool gather, int cnt, int64_t r0,
                          int nrow, int e0, const int* __restrict__ sSpos, const int* __restrict__ sFside,
                          T* __restrict__ sRed, T* __restrict__ pb) {
  constexpr int NV = DIM + 2;
  constexpr int KC = 8;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nu = nrow / W, n = a.n, F = a.F, Np = a.md.Np, nb = a.nb;
  const int64_t N = a.N;
  T accw = T(0);
  for (int k0 = 0; k0 == 0 || k0 < cnt; k0 += KC) {
    const int nk = min(KC, cnt - k0);
    T acc[KC];
#pragma unroll
    for (int k = 0; k < KC; ++k) acc[k] = T(0);
    for (int i = threadIdx.x; i < nu; i += NT) {
      const int64_t row = r0 + (int64_t)i * W;
      Pack<T, W> wv;
      if (gather && k0 == 0) {
        const int rb = i * W;  // row within the block
        const int le = rb / n, r = rb - le * n;
        wv = ldp<T, W>(vj + row);
        const int fbase = a.rc.fside_smem ? le * F : (e0 + le) * F;
        const int* fsd = a.rc.fside_smem ? sFside : a.fside;
        if (NV % W == 0) {
          // the unit lies inside one node: one W-wide load per face
          const int jn = r / NV, av = r - jn * NV;
          for (int f = 0; f < F; ++f) {
            const int sp = sSpos[f * Np + jn];
            if (sp < 0) continue;
            const int fs = fsd[fbase + f];
            if (fs < 0) continue;
            const Pack<T, W> c = ldp<T, W>(a.cfs + (size_t)fs * nb + sp * NV + av);
#pragma unroll
            for (int q = 0; q < W; ++q) wv.v[q] += c.v[q];
          }
        } else {
#pragma unroll
          for (int q = 0; q < W; ++q) {
            const int rq = r + q;
            const int lq = le + rq / n, rr = rq - (rq / n) * n;
            const int jn = rr / NV, av = rr - jn * NV;
            const int fb = a.rc.fside_smem ? lq * F : (e0 + lq) * F;
            for (int f = 0; f < F; ++f) {
              const int sp = sSpos[f * Np + jn];
              if (sp < 0) continue;
              const int fs = fsd[fb + f];
              if (fs >= 0) wv.v[q] += a.cfs[(size_t)fs * nb + sp * NV + av];
            }
          }
        }
        stp<T, W>(a.w + row, wv);
      } else {
        wv = ldp<T, W>(a.w + row);
      }
      if (k0 == 0) {
#pragma unroll
        for (int q = 0; q < W; ++q) accw += wv.v[q] * wv.v[q];
      }
      // every basis load of the chunk issued before the first dot (one
      // round trip to L2 per chunk and row)
      Pack<T, W> v[KC];
#pragma unroll
      for (int k = 0; k < KC; ++k)
        if (k < nk) v[k] = ldp<T, W>(a.V + (size_t)(k0 + k) * N + row);
#pragma unroll
      for (int k = 0; k < KC; ++k) {
        if (k < nk) {
          T d = T(0);
#pragma unroll
          for (int c = 0; c < W; ++c) d += v[k].v[c] * wv.v[c];
          acc[k] += d;
        }
      }
    }
    transpose_reduce<T, KC>(acc, lane);
    constexpr int LPS = 32 / KC;  // lanes holding each slot's sum
    if (lane % LPS == 0) sRed[warp * 33 + lane / LPS] = acc[0];
    if (k0 == 0) {
      const T ww = wsum(accw);
      if (lane == 0) sRed[warp * 33 + 32] = ww;
    }
    __syncthreads();
    if (threadIdx.x < nk) {
      T v = T(0);
      for (int q = 0; q < NW; ++q) v += sRed[q * 33 + threadIdx.x];
      pb[k0 + threadIdx.x] = v;
    }
    if (k0 == 0 && threadIdx.x == 32) {
      T v = T(0);
      for (int q = 0; q < NW; ++q) v += sRed[q * 33 + 32];
      pb[cnt] = v;
    }
    __syncthreads();
  }
}

template <int DIM, typename T>
__device__ void gs_dots(const CoopArgs<T>& a, const T* __restrict__ vj, bool gather, int cnt, int64_t r0,
                        int nrow, int e0, bool vec, const int* __restrict__ sSpos,
                        const int* __restrict__ sFside, T* __restrict__ sRed, T* __restrict__ pb) {
  if (vec)
    gs_dots_w<DIM, T, Vec<T>::W>(a, vj, gather, cnt, r0, nrow, e0, sSpos, sFside, sRed, pb);
  else
    gs_dots_w<DIM, T, 1>(a, vj, gather, cnt, r0, nrow, e0, sSpos, sFside, sRed, pb);
}

// ---- operator ring (see RingCfg) -----------------------------------------
// Unit u of Arnoldi iteration `it` has the sequence number s = it * nunits +
// u (s = u for a resident ring, loaded once) and travels through slot
// s % nslot, on the slot's n-th use with n = s / nslot: its full barrier
// completes phase n (parity n & 1) when the copies land, and its empty
// barrier completes phase n when the consumer group has released it.
struct RingState {
  int it;           // Arnoldi operator applies done by this block
  long long issued; // producer thread: sequence numbers issued so far
  int failed;       // a bounded wait of this thread gave up: no further waits
};

// the producer thread: issue the copies of unit u (sequence s) into its slot,
// armed on the slot's full barrier
template <typename T>
__device__ void ring_issue(const CoopArgs<T>& a, long long s, int nunits, int e0, int e1,
                           unsigned char* dsm, const int* __restrict__ sFside) {
  const RingCfg& rc = a.rc;
  const int n = a.n, F = a.F;
  const int u = (int)(s % nunits);
  const int slot_id = (int)(s % rc.nslot);
  unsigned char* slot = dsm + rc.off_ring + (size_t)slot_id * rc.slot_bytes;
  uint64_t* full = reinterpret_cast<uint64_t*>(dsm + rc.off_bar) + slot_id;
  const int c0 = e0 + u * rc.eps, nl = min(rc.eps, e1 - c0);
  const size_t nn = (size_t)n * n * sizeof(T);
  const char* src = reinterpret_cast<const char*>(a.inv) + (size_t)c0 * nn;
  const size_t delta = reinterpret_cast<uintptr_t>(src) & 15;
  // a 16-byte aligned range around the unit's inverse blocks (the inverse
  // array is allocated with room for the rounded end)
  const uint32_t binv = (uint32_t)((delta + (size_t)nl * nn + 15) & ~size_t(15));
  uint32_t total = binv;
  if (rc.cpl_tma) {
    for (int le = 0; le < nl; ++le)
      for (int f = 0; f < F; ++f) {
        const int fs = rc.fside_smem ? sFside[(c0 - e0 + le) * F + f] : a.fside[(size_t)(c0 + le) * F + f];
        if (fs >= 0) total += (uint32_t)rc.cpl_bytes;
      }
  }
  mbar_arrive_expect_tx(full, total);
  bulk_g2s(slot, src - delta, binv, full);
  if (rc.cpl_tma) {
    const char* cb = reinterpret_cast<const char*>(a.cpl);
    for (int le = 0; le < nl; ++le)
      for (int f = 0; f < F; ++f) {
        const int fs = rc.fside_smem ? sFside[(c0 - e0 + le) * F + f] : a.fside[(size_t)(c0 + le) * F + f];
        if (fs < 0) continue;
        bulk_g2s(slot + rc.inv_cap + (size_t)(le * F + f) * rc.cpl_bytes,
                 cb + (size_t)(fs ^ 1) * rc.cpl_bytes, (uint32_t)rc.cpl_bytes, full);
      }
  }
}

// The Arnoldi operator apply of iteration `it` through the ring: the
// producer (lane 0 of the last warp) keeps up to nslot units in flight and
// runs ahead into the first units of the next iteration (the operator is the
// same in every iteration) as slots free up; consumer group g takes units g,
// g + ngroup, ...: z = D^-1 v_j per element (inverse blocks from the slot, v
// from the unit's own rows staged in shared memory), then the push of the
// coupling products C z to the neighbours' face sides (cfs), then releases
// the slot.  A resident ring (all units fit in the slots) is loaded once for
// the whole solve.
template <int DIM, int NB, typename T>
__device__ void ring_apply_push(const CoopArgs<T>& a, const T* __restrict__ vj, int e0, int e1,
                                unsigned char* dsm, const int* __restrict__ sPerm,
                                const int* __restrict__ sFside, RingState& rs) {
  constexpr int NV = DIM + 2;
  const RingCfg& rc = a.rc;
  const int n = NB > 0 ? NB : a.n;
  const int F = a.F, S = a.S, nb = a.nb;
  const int warp = threadIdx.x >> 5;
  const int nunits = (e1 - e0 + rc.eps - 1) / rc.eps;
  const int it = rs.it++;
  if (nunits <= 0) return;
  uint64_t* fullb = reinterpret_cast<uint64_t*>(dsm + rc.off_bar);
  uint64_t* emptyb = fullb + rc.nslot;
  // the block's rows of v_j in shared memory (when they fit): the consumer
  // groups read them there instead of one round trip to L2 per unit
  T* sVj = reinterpret_cast<T*>(dsm + rc.off_vj);
  if (rc.vj_smem) {
    for (int t = threadIdx.x; t < (e1 - e0) * n; t += NT) sVj[t] = vj[(size_t)e0 * n + t];
    __syncthreads();
  }
  if (warp == NW - 1) {
    // producer: the whole warp runs the loop and waits (converged); lane 0
    // issues the copies
    const int lane = threadIdx.x & 31;
    const long long upto = rc.resident ? (long long)nunits
                                       : (long long)(it + 1) * nunits + min(rc.nslot, nunits);
    for (long long s = rs.issued; s < upto; ++s) {
      if (s >= rc.nslot && !rs.failed) {
        // the slot's previous use (sequence s - nslot) must be released
        const uint32_t par = (uint32_t)(((s / rc.nslot) - 1) & 1);
        if (!mbar_wait(emptyb + (s % rc.nslot), par)) {
          rs.failed = 1;
          if (lane == 0) atomicOr(a.flags + F_TMO, 1);
        }
      }
      __syncwarp();
      if (lane == 0) {
        fence_proxy_async_smem();
        ring_issue<T>(a, s, nunits, e0, e1, dsm, sFside);
      }
      __syncwarp();
    }
    if (upto > rs.issued) rs.issued = upto;
    return;
  }
  const int g = warp / rc.wpg;
  if (g >= rc.ngroup || g >= nunits) return;
  const int GT = rc.wpg * 32, gt = threadIdx.x - g * GT;
  T* zb = reinterpret_cast<T*>(dsm + rc.off_z) + (size_t)g * rc.eps * n;
  T* vb = reinterpret_cast<T*>(dsm + rc.off_v) + (size_t)g * rc.eps * n;
  for (int u = g; u < nunits; u += rc.ngroup) {
    const long long sq = rc.resident ? (long long)u : (long long)it * nunits + u;
    const int slot_id = (int)(sq % rc.nslot);
    const uint32_t par = rc.resident ? 0u : (uint32_t)((sq / rc.nslot) & 1);
    const unsigned char* slot = dsm + rc.off_ring + (size_t)slot_id * rc.slot_bytes;
    const int c0 = e0 + u * rc.eps, nl = min(rc.eps, e1 - c0);
    const T* vu = vb;
    if (rc.vj_smem)
      vu = sVj + (size_t)(c0 - e0) * n;
    else
      for (int t = gt; t < nl * n; t += GT) vb[t] = vj[(size_t)c0 * n + t];
    // after a wait that gave up, the thread stops waiting (the results are
    // void and the host reports EG_ERR_TIMEOUT)
    if (!rs.failed && !mbar_wait(fullb + slot_id, par)) {
      rs.failed = 1;
      atomicOr(a.flags + F_TMO, 1);
    }
    named_sync(1 + g, GT);
    const T* inv = reinterpret_cast<const T*>(slot + (((size_t)c0 * n * n * sizeof(T)) & 15));
    for (int t = gt; t < nl * n; t += GT) {
      const int le = t / n, r = t - le * n;
      zb[t] = block_row<NB, T>(inv + (size_t)le * n * n, vu + (size_t)le * n, r, n);
    }
    named_sync(1 + g, GT);
    // push: row i of the neighbour's coupling block on face f of element le
    const int nitem = nl * F * nb;
    for (int itm = gt; itm < nitem; itm += GT) {
      const int le = itm / (F * nb), rem = itm - le * (F * nb);
      const int f = rem / nb, i = rem - f * nb;
      const int fs = rc.fside_smem ? sFside[(c0 - e0 + le) * F + f] : a.fside[(size_t)(c0 + le) * F + f];
      if (fs < 0) continue;
      const int tgt = fs ^ 1;
      const T* zs = zb + (size_t)le * n;
      const int* pf = sPerm + f * S;
      T acc = T(0);
      if (a.md.sparse_face) {
        const int o = a.md.ifaces[5 * (tgt >> 1) + 4];
        const int* facing = (tgt & 1) ? a.md.nbrinv + o * a.md.Nf : a.md.nbrperm + o * a.md.Nf;
        const T* Cr = a.cpl + (size_t)tgt * nb * NV + (size_t)i * NV;
        const T* zz = zs + pf[facing[i / NV]] * NV;
        T c[NV];
        load_row_piece<NV, T>(Cr, c);
#pragma unroll
        for (int b = 0; b < NV; ++b) acc += c[b] * zz[b];
      } else if (rc.cpl_tma) {
        // the row's NV-wide pieces in a rotated order (piece (k + i) % S at
        // step k): neighbouring rows start in different banks
        const T* Cr = reinterpret_cast<const T*>(slot + rc.inv_cap + (size_t)(le * F + f) * rc.cpl_bytes) +
                      (size_t)i * nb;
        for (int k = 0; k < S; ++k) {
          int sp = k + i;
          sp = sp % S;
          T c[NV];
          load_row_piece<NV, T>(Cr + sp * NV, c);
          const T* zz = zs + pf[sp] * NV;
#pragma unroll
          for (int b = 0; b < NV; ++b) acc += c[b] * zz[b];
        }
      } else {
        const T* Cr = a.cpl + ((size_t)tgt * nb + i) * nb;
        for (int sp = 0; sp < S; ++sp) {
          T c[NV];
          load_row_piece<NV, T>(Cr + sp * NV, c);
          const T* zz = zs + pf[sp] * NV;
#pragma unroll
          for (int b = 0; b < NV; ++b) acc += c[b] * zz[b];
        }
      }
      a.cfs[(size_t)tgt * nb + i] = acc;
    }
    named_sync(1 + g, GT);
    // release the slot to the producer (a resident ring keeps its units)
    if (gt == 0 && !rc.resident) mbar_arrive(emptyb + slot_id);
  }
}

// before the block exits: the producer waits (bounded) for the copies still
// in flight into the ring (the next iteration's units it issued ahead)
template <typename T>
__device__ void ring_drain(const CoopArgs<T>& a, unsigned char* dsm, RingState& rs, int e0, int e1) {
  // every issued copy is waited for (bounded), also after an earlier wait
  // gave up: the block must not end with copies into its shared memory
  if (!a.rc.on || (threadIdx.x >> 5) != NW - 1) return;
  const int nunits = (e1 - e0 + a.rc.eps - 1) / a.rc.eps;
  if (nunits <= 0) return;
  uint64_t* fullb = reinterpret_cast<uint64_t*>(dsm + a.rc.off_bar);
  // sequences consumed: it * nunits (nunits when resident and used once)
  const long long consumed = a.rc.resident ? (rs.it > 0 ? nunits : 0) : (long long)rs.it * nunits;
  for (long long s = consumed; s < rs.issued; ++s) {
    const uint32_t par = a.rc.resident ? 0u : (uint32_t)((s / a.rc.nslot) & 1);
    if (!mbar_wait(fullb + (s % a.rc.nslot), par)) {
      if ((threadIdx.x & 31) == 0) atomicOr(a.flags + F_TMO, 1);
      return;
    }
  }
}

// Element block times a vector held per element (z_e = A_e x_e) for a chunk
// of the block's elements, the elements' own values staged in shared memory,
// followed by the push of the face couplings C x_e to the neighbours'
// face sides (cfs).  Rows of A x go to out (own rows).
template <int DIM, int NB, typename T>
__device__ void chunk_apply_push(const CoopArgs<T>& a, const T* __restrict__ A, const T* __restrict__ x,
                                 bool stage_product, T* __restrict__ sZ, const int* __restrict__ sPerm,
                                 int c0, int nl, T* __restrict__ out) {
  const int n = NB > 0 ? NB : a.n;
  if (stage_product) {
    // sZ = A x (the coupling acts on the product): z = D^-1 v
    for (int t = threadIdx.x; t < nl * n; t += NT) {
      const int le = t / n, r = t - le * n;
      const int e = c0 + le;
      sZ[t] = block_row<NB, T>(A + (size_t)e * n * n, x + (size_t)e * n, r, n);
    }
    __syncthreads();
  } else {
    // sZ = x (the coupling acts on x), out = A x: D x for the residual
    for (int t = threadIdx.x; t < nl * n; t += NT) sZ[t] = x[(size_t)c0 * n + t];
    __syncthreads();
    for (int t = threadIdx.x; t < nl * n; t += NT) {
      const int le = t / n, r = t - le * n;
      const int e = c0 + le;
      out[(size_t)e * n + r] = block_row<NB, T>(A + (size_t)e * n * n, sZ + (size_t)le * n, r, n);
    }
  }
  face_push<DIM, T>(a, sZ, sPerm, c0, nl, a.cfs);
  __syncthreads();
}

// block-level state of the persistent GMRES (static shared memory of the
// kernel that runs it)
template <typename T>
struct GmresShared {
  int sPerm[64], sSpos[128];
  T sh1[33], sh2[33];
  T scs[32], ssn[32], sg[33], sHc[33], syT[33];
  T sR[32 * 33];  // rotated Hessenberg columns: sR[j * (m+1) + k]
  double sy[33], sdi[33];
  int s_done, s_its, s_reorth, s_jdone, s_conv, s_cycles;
  T s_beta;
  double s_tol, s_bnorm;
};

// barrier of a single-problem launch: the whole cooperative grid
struct GridBarrier {
  cg::grid_group g;
  __device__ bool sync() {
    g.sync();
    return true;
  }
};

// The whole right-preconditioned GMRES(m) solve of J x = b as one persistent
// cooperative kernel (reference: the restarted GMRES behind linearSolve,
// ls_standard.jl:321-371, with the element block-Jacobi preconditioner of
// NewtonBDiagPC, preconditioning.jl:7-139).
//   * cycle start: r = b - J x (element blocks D and the face push), beta =
//     |r|, converged when beta <= max(reltol |b|, abstol) (the true residual),
//     v_0 = r / beta;
//   * Arnoldi on J M^-1 = I + C D^-1: classical Gram-Schmidt with the norm of
//     the orthogonalised vector from the same reduction (|w'|^2 = w.w -
//     |h|^2) and a second classical pass (its reduction also yields w'.w')
//     when |w'|^2 < |w|^2 / 2 (DGKS with eta = 1/sqrt 2); Givens rotations in
//     T by one lane while the other warps form v_{j+1};
//   * cycle end: y = R^-1 g (FP64 back substitution, one warp), x += D^-1 V y
//     on the block's own rows.
// Block b of the problem's nblk blocks owns a contiguous element range (and
// its rows) for the whole solve; barriers over those blocks (the cooperative
// grid, or a problem's part of a batched grid) separate the phases whose data crosses blocks (the
// pushed face products, the dot-product partials).  Every block reduces the
// partials in the same order, so the scalars (Hessenberg entries, rotations,
// the reorthogonalisation test, the convergence decision) are bit-identical
// in every block and all blocks take the same branches.
template <int DIM, int NB, typename T, class Bar>
__device__ void gmres_solve(const CoopArgs<T>& a, const int b, const int nblk, Bar& grid,
                            GmresShared<T>& sm, RingState& rs) {
  constexpr int NV = DIM + 2;
  const int tid = threadIdx.x;
  const int n = NB > 0 ? NB : a.n, m = a.m, M1 = a.m + 1;
  const int64_t N = a.N;
  const int epb = (a.E + nblk - 1) / nblk;
  const int e0 = min(a.E, b * epb), e1 = min(a.E, e0 + epb);
  const int64_t r0 = (int64_t)e0 * n;
  const int nrow = (e1 - e0) * n;
  const bool vec = NB > 0 ? (NB % Vec<T>::W) == 0 : (a.n % Vec<T>::W) == 0;
  T* P0 = a.part;                               // first pass: dots and w.w
  T* P2 = a.part + 2 * (size_t)nblk * PSTRIDE;  // second pass: dots and w'.w'
  extern __shared__ __align__(128) unsigned char dsmem[];
  T* sZ = reinterpret_cast<T*>(dsmem + a.rc.off_sz);  // [ec][n] per-element values of a chunk
  T* sRed = reinterpret_cast<T*>(dsmem + a.rc.off_red);  // [NW][33] cross-warp sums
  int* sFside = reinterpret_cast<int*>(dsmem + a.rc.off_fside);  // [epb][F] when staged
  int* sPerm = sm.sPerm;
  int* sSpos = sm.sSpos;
  T* sh1 = sm.sh1;
  T* sh2 = sm.sh2;
  T* scs = sm.scs;
  T* ssn = sm.ssn;
  T* sg = sm.sg;
  T* sHc = sm.sHc;
  T* syT = sm.syT;
  T* sR = sm.sR;
  double* sy = sm.sy;
  double* sdi = sm.sdi;
  int& s_done = sm.s_done;
  int& s_its = sm.s_its;
  int& s_reorth = sm.s_reorth;
  int& s_jdone = sm.s_jdone;
  int& s_conv = sm.s_conv;
  int& s_cycles = sm.s_cycles;
  T& s_beta = sm.s_beta;
  double& s_tol = sm.s_tol;
  double& s_bnorm = sm.s_bnorm;
  for (int k = tid; k < a.F * a.S; k += NT) sPerm[k] = a.md.perm[k];
  if (a.rc.fside_smem)
    for (int k = tid; k < (e1 - e0) * a.F; k += NT) sFside[k] = a.fside[(size_t)e0 * a.F + k];
  if (a.rc.on && tid == 0) {
    // full[nslot] (armed by the producer), empty[nslot] (one consumer arrival)
    uint64_t* bars = reinterpret_cast<uint64_t*>(dsmem + a.rc.off_bar);
    for (int k = 0; k < 2 * a.rc.nslot; ++k) mbar_init(bars + k, 1);
    fence_mbar_init();
  }
  for (int k = tid; k < a.F * a.md.Np; k += NT) sSpos[k] = a.spos[k];
  // |b|
  block_dots<T>(a.V, a.bvec, 0, 1, N, r0, nrow, vec, P0 + (size_t)b * PSTRIDE);
  if (!grid.sync()) return;
  block_reduce_all<T>(P0, nblk, 1, sh1);
  __syncthreads();
  if (tid == 0) {
    s_bnorm = sqrt(double(sh1[0]));
    s_tol = fmax(a.scal[S_RELTOL] * s_bnorm, a.scal[S_ABSTOL]);
    s_its = 0;
    s_cycles = 0;
  }
  __syncthreads();
  for (;;) {
    // ---- r = b - J x (own rows); the pushed products cross blocks
    for (int c0 = e0; c0 < e1; c0 += a.ec) {
      const int nl = min(a.ec, e1 - c0);
      chunk_apply_push<DIM, NB, T>(a, a.diag, a.x, false, sZ, sPerm, c0, nl, a.w);
    }
    if (!grid.sync()) return;
    for (int t = tid; t < nrow; t += NT) {
      const int le = t / n, r = t - le * n;
      const int j = r / NV, av = r - j * NV;
      const int e = e0 + le;
      const int64_t row = (int64_t)e * n + r;
      T acc = a.w[row];
      for (int f = 0; f < a.F; ++f) {
        const int sp = sSpos[f * a.md.Np + j];
        if (sp < 0) continue;
        const int fs = a.fside[(int64_t)e * a.F + f];
        if (fs >= 0) acc += a.cfs[(size_t)fs * a.nb + sp * NV + av];
      }
      a.w[row] = a.bvec[row] - acc;
    }
    __syncthreads();
    block_dots<T>(a.V, a.w, 0, 1, N, r0, nrow, vec, P0 + (size_t)b * PSTRIDE);
    if (!grid.sync()) return;
    block_reduce_all<T>(P0, nblk, 1, sh1);
    __syncthreads();
    if (tid == 0) {
      const T beta = sqrt(sh1[0]);
      s_beta = beta;
      if (s_cycles == 0 && b == 0) a.scal[S_BETA0] = double(beta);
      const bool conv = !(double(beta) > s_tol);
      s_conv = conv ? 1 : 0;
      s_done = (conv || s_its >= a.flags[F_ITERMAX] || !isfinite(double(beta))) ? 1 : 0;
      s_jdone = 0;
      sg[0] = beta;
      for (int k = 1; k <= m; ++k) sg[k] = T(0);
    }
    __syncthreads();
    if (s_done) break;
    block_sub_scale<T>(a.V, sh1, 0, N, a.w, T(1) / s_beta, a.V, r0, nrow, vec, 0);
    __syncthreads();
    // ---- Arnoldi
    for (int j = 0; j < m; ++j) {
      if (s_done) break;
      const T* vj = a.V + (size_t)j * N;
      T* vn = a.V + (size_t)(j + 1) * N;
      // (1) z = D^-1 v_j per element, push C z to the neighbours' face sides
      if (a.rc.on) {
        ring_apply_push<DIM, NB, T>(a, vj, e0, e1, dsmem, sPerm, sFside, rs);
      } else {
        for (int c0 = e0; c0 < e1; c0 += a.ec) {
          const int nl = min(a.ec, e1 - c0);
          chunk_apply_push<DIM, NB, T>(a, a.inv, vj, true, sZ, sPerm, c0, nl, nullptr);
        }
      }
      if (!grid.sync()) return;
      // (2) w = v_j + the pushed products of the faces holding the row's
      // node, and (3) the first pass h1 = V^T w with w.w, in one reduction
      gs_dots<DIM, T>(a, vj, true, j + 1, r0, nrow, e0, vec, sSpos, sFside, sRed,
                      P0 + (size_t)b * PSTRIDE);
      if (!grid.sync()) return;
      block_reduce_all<T>(P0, nblk, j + 2, sh1);
      __syncthreads();
      if (tid == 0) {
        T hh = T(0);
        for (int k = 0; k <= j; ++k) hh += sh1[k] * sh1[k];
        const T ww = sh1[j + 1];
        const T n2 = ww - hh;
        s_reorth = n2 < T(0.5) * ww;
        sh2[32] = n2;  // |w'|^2
      }
      __syncthreads();
      if (s_reorth) {
        // (4) second pass on w' = w - V h1: h2 = V^T w' and w'.w' in one reduction
        block_sub_scale<T>(a.V, sh1, j + 1, N, a.w, T(1), a.w, r0, nrow, vec, 0);
        __syncthreads();
        gs_dots<DIM, T>(a, vj, false, j + 1, r0, nrow, e0, vec, sSpos, sFside, sRed,
                        P2 + (size_t)b * PSTRIDE);
        if (!grid.sync()) return;
        block_reduce_all<T>(P2, nblk, j + 2, sh2);
        __syncthreads();
        if (tid == 0) {
          T hh = T(0);
          for (int k = 0; k <= j; ++k) hh += sh2[k] * sh2[k];
          const T r = sh2[j + 1] - hh;
          sh2[32] = r > T(0) ? r : T(0);
        }
        __syncthreads();
      }
      const T hn = sqrt(sh2[32]);
      const T inv = hn > T(0) ? T(1) / hn : T(0);
      // (5) lane 0: Hessenberg column j and its Givens rotation (identical in
      //     every block); warps 1.. : v_{j+1} = (w - V h) / hn
      if (tid == 0) {
        for (int k = 0; k <= j; ++k) sHc[k] = s_reorth ? sh1[k] + sh2[k] : sh1[k];
        sHc[j + 1] = hn;
        for (int k = 0; k < j; ++k) {
          const T t0 = scs[k] * sHc[k] + ssn[k] * sHc[k + 1];
          sHc[k + 1] = -ssn[k] * sHc[k] + scs[k] * sHc[k + 1];
          sHc[k] = t0;
        }
        const T den = hypot(sHc[j], sHc[j + 1]);
        s_its += 1;
        if (!(den > T(0)) || !isfinite(den)) {
          s_done = 1;  // breakdown: keep the j columns built so far
        } else {
          scs[j] = sHc[j] / den;
          ssn[j] = sHc[j + 1] / den;
          sHc[j] = den;
          sHc[j + 1] = T(0);
          sg[j + 1] = -ssn[j] * sg[j];
          sg[j] = scs[j] * sg[j];
          s_jdone = j + 1;
          for (int k = 0; k <= j; ++k) sR[j * M1 + k] = sHc[k];
          const double resid = fabs(double(sg[j + 1]));
          if (resid <= s_tol || hn == T(0) || s_its >= a.flags[F_ITERMAX]) s_done = 1;
        }
      } else if (tid >= 32) {
        if (s_reorth)
          block_sub_scale<T>(a.V, sh2, j + 1, N, a.w, inv, vn, r0, nrow, vec, 32);
        else
          block_sub_scale<T>(a.V, sh1, j + 1, N, a.w, inv, vn, r0, nrow, vec, 32);
      }
      __syncthreads();
    }
    // ---- y = R^-1 g (FP64 back substitution by warp 0), x += D^-1 V y
    if (tid < 32) {
      const int nn = s_jdone, lane = tid;
      for (int k = lane; k < nn; k += 32) {
        sdi[k] = 1.0 / double(sR[k * M1 + k]);
        sy[k] = double(sg[k]);
      }
      __syncwarp();
      for (int k = nn - 1; k >= 0; --k) {
        const double yk = sy[k] * sdi[k];
        __syncwarp();
        if (lane == 0) sy[k] = yk;
        for (int i = lane; i < k; i += 32) sy[i] -= double(sR[k * M1 + i]) * yk;
        __syncwarp();
      }
      for (int k = lane; k < nn; k += 32) syT[k] = T(sy[k]);
      if (lane == 0) s_cycles += 1;
    }
    __syncthreads();
    block_lincomb<T>(a.V, syT, s_jdone, N, a.w, r0, nrow);
    __syncthreads();
    for (int t = tid; t < nrow; t += NT) {
      const int le = t / n, r = t - le * n;
      const int e = e0 + le;
      a.x[(size_t)e * n + r] += block_row<NB, T>(a.inv + (size_t)e * n * n, a.w + (size_t)e * n, r, n);
    }
    __syncthreads();
  }
  if (b == 0 && tid == 0) {
    a.flags[F_ITS] = s_its;
    a.flags[F_JDONE] = s_jdone;
    a.flags[F_DONE] = 1;
    a.flags[F_CONV] = s_conv;
    a.flags[F_CYCLES] = s_cycles;
    a.scal[S_BETA] = double(s_beta);
    a.scal[S_RESID] = double(s_beta);
    a.scal[S_BNORM] = s_bnorm;
    a.scal[S_TOL] = s_tol;
  }
}

// The solve, then (on every way out, including a failed barrier of a batched
// launch) a bounded wait for the operator copies still in flight into the
// block's shared memory.
template <int DIM, int NB, typename T, class Bar>
__device__ void gmres_body(const CoopArgs<T>& a, const int b, const int nblk, Bar& grid,
                           GmresShared<T>& sm) {
  extern __shared__ __align__(128) unsigned char dsmem[];
  RingState rs{0, 0, 0};
  gmres_solve<DIM, NB, T, Bar>(a, b, nblk, grid, sm, rs);
  const int epb = (a.E + nblk - 1) / nblk;
  const int e0 = min(a.E, b * epb), e1 = min(a.E, e0 + epb);
  ring_drain<T>(a, dsmem, rs, e0, e1);
}

// kernel arguments of a solver's GMRES solve (chunk size a->ec set by the
// launcher, which knows the grid)
template <typename T>
void coop_args(const eg_ls* ls, CoopArgs<T>* out) {
  const eg_mesh* m = ls->lo->mesh;
  CoopArgs<T>& a = *out;
  a.md = dev_mesh(m);
  a.inv = (const T*)ls->pc->inv;
  a.diag = (const T*)ls->lo->diag;
  a.cpl = (const T*)ls->lo->cpl;
  a.spos = ls->lo->spos;
  a.fside = ls->lo->fside;
  a.cfs = (T*)ls->cfs;
  a.bvec = (const T*)ls->bT;
  a.x = (T*)ls->xT;
  a.nb = ls->lo->nb;
  a.S = m->S;
  a.F = m->F;
  a.nv = m->nv;
  a.V = (T*)ls->V;
  a.w = (T*)ls->w;
  a.part = (T*)ls->part;
  a.flags = ls->dflags;
  a.scal = ls->dscal;
  a.m = ls->m;
  a.n = ls->lo->n;
  a.E = m->E;
  a.N = m->ndof;
  a.ec = 1;
}

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Dynamic shared-memory layout of a solve on nblk blocks: the operator ring
// (2-D dense coupling, or 3-D face-diagonal coupling, when at least two slots
// fit), the cross-warp sums, the block's face-side table when it fits, and
// the chunk buffer of the residual and update passes.  Sets a->rc and a->ec;
// returns the bytes.
template <typename T>
size_t coop_layout(CoopArgs<T>* a, int dim, int nblk) {
  RingCfg& rc = a->rc;
  rc = RingCfg{};
  const int n = a->n, nb = a->nb, F = a->F;
  const int epb = std::max(1, (a->E + nblk - 1) / nblk);
  const size_t es = sizeof(T);
  const size_t nn = (size_t)n * n * es, cb = (size_t)nb * nb * es;
  const bool sparse = a->md.sparse_face != 0;
  const bool ring_ok = dim == 2 ? !sparse : sparse;
  const int cpl_tma = (dim == 2 && !sparse && cb % 16 == 0) ? 1 : 0;
  const size_t per_el = nn + (cpl_tma ? (size_t)F * cb : 0);
  int eps = (int)std::max<size_t>(1, std::min<size_t>(16, kSlotTarget / per_el));
  eps = std::min(eps, epb);
  // room for the 16-byte rounding at both ends of the unit's inverse range
  const size_t inv_cap = align_up((size_t)eps * nn + 32, 16);
  const size_t slot = align_up(inv_cap + (cpl_tma ? (size_t)eps * F * cb : 0), 128);
  const int nunits = (epb + eps - 1) / eps;
  const int cap = (int)std::min<size_t>(16, kRingBudget / slot);
  // Consumer groups: the last warp is the producer.  A streaming ring needs
  // nslot to be a multiple of ngroup: then every use of a slot belongs to one
  // group, which has waited for the slot's previous use before it waits for
  // the next, so a parity wait never sees a phase two uses old (the
  // mbarrier's parity tells only the current phase from the one before).
  // The most groups (of at least two warps) whose multiple keeps three
  // quarters of the slots that fit.
  int nslot = 0, ngroup = 1;
  for (int g = (NW - 1) / 2; g >= 1; --g) {
    const int ns = (cap / g) * g;
    if (ns >= 2 && 4 * ns >= 3 * cap) {
      nslot = ns;
      ngroup = g;
      break;
    }
  }
  size_t off = 0;
  if (ring_ok && nslot >= 2) {
    rc.on = 1;
    rc.resident = nunits <= cap ? 1 : 0;
    if (rc.resident) {
      // every unit has its slot, used once: any grouping is safe
      nslot = nunits;
      ngroup = (NW - 1) / 2;
    }
    rc.nslot = nslot;
    rc.eps = eps;
    rc.ngroup = ngroup;
    rc.wpg = (NW - 1) / ngroup;
    rc.cpl_tma = cpl_tma;
    rc.slot_bytes = (int)slot;
    rc.inv_cap = (int)inv_cap;
    rc.cpl_bytes = (int)cb;
    rc.off_ring = 0;
    off = (size_t)rc.nslot * slot;
    rc.off_bar = (int)off;
    off += align_up((size_t)2 * rc.nslot * 8, 16);
    rc.off_z = (int)off;
    off += align_up((size_t)rc.ngroup * eps * n * es, 16);
    const size_t vj_bytes = align_up((size_t)epb * n * es, 16);
    if (vj_bytes <= 24 * 1024) {
      rc.vj_smem = 1;
      rc.off_vj = (int)off;
      off += vj_bytes;
      rc.off_v = rc.off_vj;  // per-unit staging not used
    } else {
      rc.off_v = (int)off;
      off += align_up((size_t)rc.ngroup * eps * n * es, 16);
    }
  }
  rc.off_red = (int)off;
  off += align_up((size_t)NW * 33 * es, 16);
  const size_t fs_bytes = align_up((size_t)epb * F * sizeof(int), 16);
  if (fs_bytes <= 16 * 1024 && off + fs_bytes + (size_t)n * es <= kSmemMax) {
    rc.fside_smem = 1;
    rc.off_fside = (int)off;
    off += fs_bytes;
  }
  rc.off_sz = (int)off;
  const size_t room = std::min<size_t>(kSmemMax - off, 40 * 1024);
  int ec = (int)(room / ((size_t)n * es));
  ec = std::max(1, std::min(ec, epb));
  a->ec = ec;
  return off + (size_t)ec * n * es;
}

template <int DIM, int NB, typename T>
__global__ void __launch_bounds__(NT, 1) k_gmres_coop(CoopArgs<T> a) {
  __shared__ GmresShared<T> sm;
  GridBarrier bar{cg::this_grid()};
  gmres_body<DIM, NB, T>(a, blockIdx.x, gridDim.x, bar, sm);
}

}  // namespace
