// eg_arnoldi_body.cuh -- the persistent GMRES solve as a device function,
// shared by the single-problem cooperative kernel (eg_arnoldi.cu) and the
// batched kernel that runs several problems' solves in one launch
// (eg_arnoldi_batch.cu).  The algorithm and its data flow are described in
// eg_arnoldi.cu.
#pragma once
#include <cooperative_groups.h>

#include "eg_internal.h"
#include "eg_kernels.cuh"
#include "eg_krylov.cuh"
#include "eg_linalg.h"

namespace cg = cooperative_groups;

namespace {

constexpr int NT = 1024;  // one block per SM
constexpr int NB_MAX = 64;  // coupling-block rows handled by the face-side pass
// systems whose element blocks take at most this many bytes run on one block
constexpr size_t kSmallOperatorBytes = size_t(2) << 20;

constexpr int PSTRIDE = 33;  // partial slots per block

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
  int l2ef;  // operator + basis exceed L2: operator loads marked evict-first
  int nb, S, F, nv, ec;  // coupling block size, stencil size, faces, variables, elements per chunk
  int64_t N;
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

// Loads of the operator blocks (block inverses, coupling blocks) with an L2
// evict-first policy: the operator is streamed once per Arnoldi iteration,
// and its lines should leave L2 before the Krylov basis, which every
// Gram-Schmidt pass reads again.
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ float ld_ef(const float* p, uint64_t pol) {
  float v;
  asm("ld.global.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ double ld_ef(const double* p, uint64_t pol) {
  double v;
  asm("ld.global.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
  return v;
}
// NV consecutive values of a coupling row through ld_ef (16-byte loads for
// 2-D FP32)
template <int NV, typename T>
__device__ __forceinline__ void load_row_piece_ef(const T* __restrict__ p, T* out, uint64_t pol) {
  if constexpr (NV == 4 && sizeof(T) == 4) {
    float4 v;
    asm("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(p), "l"(pol));
    out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = v.w;
  } else {
#pragma unroll
    for (int b = 0; b < NV; ++b) out[b] = ld_ef(p + b, pol);
  }
}
// block_row (eg_krylov.cuh) with the operator block read through ld_ef
template <int NB, typename T>
__device__ __forceinline__ T block_row_ef(const T* __restrict__ A, const T* __restrict__ xe, int r, int n,
                                          uint64_t pol) {
  T acc0 = T(0), acc1 = T(0), acc2 = T(0), acc3 = T(0);
  if (NB > 0) {
#pragma unroll
    for (int c = 0; c < NB; c += 4) {
      acc0 += ld_ef(A + (size_t)c * NB + r, pol) * xe[c];
      if (c + 1 < NB) acc1 += ld_ef(A + (size_t)(c + 1) * NB + r, pol) * xe[c + 1];
      if (c + 2 < NB) acc2 += ld_ef(A + (size_t)(c + 2) * NB + r, pol) * xe[c + 2];
      if (c + 3 < NB) acc3 += ld_ef(A + (size_t)(c + 3) * NB + r, pol) * xe[c + 3];
    }
  } else {
#pragma unroll 4
    for (int c = 0; c < n; ++c) acc0 += ld_ef(A + (size_t)c * n + r, pol) * xe[c];
  }
  return (acc0 + acc1) + (acc2 + acc3);
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
  const uint64_t pol = l2_evict_first();
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
        if (a.l2ef)
          load_row_piece_ef<NV, T>(Cr, c, pol);
        else
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
        if (a.l2ef)
          load_row_piece_ef<NV, T>(Cr + sp * NV, c, pol);
        else
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
      // four row units per lane in flight (both operands), then two
      int i = lane;
      T acc2 = T(0), acc3 = T(0);
      for (; i + 96 < n4; i += 128) {
        const typename VT::V a0 = v4[i], a1 = v4[i + 32], a2 = v4[i + 64], a3 = v4[i + 96];
        const typename VT::V b0 = x4[i], b1 = x4[i + 32], b2 = x4[i + 64], b3 = x4[i + 96];
        acc0 += VT::dot(a0, b0);
        acc1 += VT::dot(a1, b1);
        acc2 += VT::dot(a2, b2);
        acc3 += VT::dot(a3, b3);
      }
      for (; i + 32 < n4; i += 64) {
        acc0 += VT::dot(v4[i], x4[i]);
        acc1 += VT::dot(v4[i + 32], x4[i + 32]);
      }
      if (i < n4) acc0 += VT::dot(v4[i], x4[i]);
      acc0 += acc2;
      acc1 += acc3;
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
// t0 .. NT-1 (x and y may alias)
template <typename T>
__device__ void block_sub_scale(const T* __restrict__ V, const T* __restrict__ h, int cnt, int64_t N,
                                const T* x, T s, T* y, int64_t r0, int nrow, bool vec, int t0) {
  using VT = Vec<T>;
  if (vec) {
    const int n4 = nrow / VT::W;
    for (int i = threadIdx.x - t0; i < n4; i += NT - t0) {
      const int64_t row = r0 + (int64_t)i * VT::W;
      typename VT::V a = *reinterpret_cast<const typename VT::V*>(x + row);
      int k = 0;
      for (; k + 4 <= cnt; k += 4) {
        const typename VT::V v0 = *reinterpret_cast<const typename VT::V*>(V + (size_t)k * N + row);
        const typename VT::V v1 = *reinterpret_cast<const typename VT::V*>(V + (size_t)(k + 1) * N + row);
        const typename VT::V v2 = *reinterpret_cast<const typename VT::V*>(V + (size_t)(k + 2) * N + row);
        const typename VT::V v3 = *reinterpret_cast<const typename VT::V*>(V + (size_t)(k + 3) * N + row);
        a = VT::fma(v0, h[k], a);
        a = VT::fma(v1, h[k + 1], a);
        a = VT::fma(v2, h[k + 2], a);
        a = VT::fma(v3, h[k + 3], a);
      }
      for (; k < cnt; ++k)
        a = VT::fma(*reinterpret_cast<const typename VT::V*>(V + (size_t)k * N + row), h[k], a);
      *reinterpret_cast<typename VT::V*>(y + row) = VT::scale(a, s);
    }
  } else {
    for (int i = threadIdx.x - t0; i < nrow; i += NT - t0) {
      const int64_t row = r0 + i;
      T a = x[row];
      for (int k = 0; k < cnt; ++k) a -= V[(size_t)k * N + row] * h[k];
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
    if (a.l2ef) {
      const uint64_t pol = l2_evict_first();
      for (int t = threadIdx.x; t < nl * n; t += NT) {
        const int le = t / n, r = t - le * n;
        const int e = c0 + le;
        sZ[t] = block_row_ef<NB, T>(A + (size_t)e * n * n, x + (size_t)e * n, r, n, pol);
      }
    } else {
      for (int t = threadIdx.x; t < nl * n; t += NT) {
        const int le = t / n, r = t - le * n;
        const int e = c0 + le;
        sZ[t] = block_row<NB, T>(A + (size_t)e * n * n, x + (size_t)e * n, r, n);
      }
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

// Sum of the pushed face products that land on row (node j, variable av) of
// element e, added to acc in face order: one term per simplex face (DIM + 1 of them) whose stencil holds
// the node and that couples to a neighbour.  The faces are unrolled so that
// their face-side and product loads are all in flight together.
template <int DIM, int NV, typename T>
__device__ __forceinline__ T gather_pushed(const CoopArgs<T>& a, const int* __restrict__ sSpos, int e, int j,
                                           int av, T acc) {
  constexpr int FF = DIM + 1;
  int fs[FF], sp[FF];
#pragma unroll
  for (int f = 0; f < FF; ++f) {
    sp[f] = sSpos[f * a.md.Np + j];
    fs[f] = sp[f] >= 0 ? a.fside[(int64_t)e * FF + f] : -1;
  }
  T v[FF];
#pragma unroll
  for (int f = 0; f < FF; ++f) v[f] = fs[f] >= 0 ? a.cfs[(size_t)fs[f] * a.nb + sp[f] * NV + av] : T(0);
#pragma unroll
  for (int f = 0; f < FF; ++f) acc += v[f];  // face order; a skipped face adds an exact zero
  return acc;
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
  int s_done, s_its, s_reorth, s_jdone, s_conv, s_cycles, s_nreorth;
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
//   * Arnoldi on K = C D^-1 (the coupling part of J M^-1 = I + K): the Krylov
//     spaces of K and I + K are the same, and K V_j = V_{j+1} H_K gives
//     (I + K) V_j = V_{j+1} (H_K + I), so the vectors are orthogonalised
//     without the v_j term that I adds (which would only be subtracted again,
//     with its cancellation) and the identity is added to the Hessenberg
//     column's diagonal; classical Gram-Schmidt with the norm of
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
__device__ void gmres_body(const CoopArgs<T>& a, const int b, const int nblk, Bar& grid,
                           GmresShared<T>& sm) {
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
  extern __shared__ __align__(16) unsigned char dsmem[];
  T* sZ = reinterpret_cast<T*>(dsmem);  // [ec][n] per-element values of a chunk
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
  int& s_nreorth = sm.s_nreorth;
  T& s_beta = sm.s_beta;
  double& s_tol = sm.s_tol;
  double& s_bnorm = sm.s_bnorm;
  for (int k = tid; k < a.F * a.S; k += NT) sPerm[k] = a.md.perm[k];
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
    s_nreorth = 0;
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
      const T acc = gather_pushed<DIM, NV, T>(a, sSpos, e, j, av, a.w[row]);
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
      // (1) per chunk: z = D^-1 v_j (shared memory), push C z to the neighbours
      for (int c0 = e0; c0 < e1; c0 += a.ec) {
        const int nl = min(a.ec, e1 - c0);
        chunk_apply_push<DIM, NB, T>(a, a.inv, vj, true, sZ, sPerm, c0, nl, nullptr);
      }
      if (!grid.sync()) return;
      // (2) w = K v_j: the pushed products of the faces holding the row's node
      for (int t = tid; t < nrow; t += NT) {
        const int le = t / n, r = t - le * n;
        const int jn = r / NV, av = r - jn * NV;
        const int e = e0 + le;
        const int64_t row = (int64_t)e * n + r;
        a.w[row] = gather_pushed<DIM, NV, T>(a, sSpos, e, jn, av, T(0));
      }
      __syncthreads();
      // (3) first pass: h1 = V^T w and w.w in one reduction
      block_dots<T>(a.V, a.w, j + 1, 1, N, r0, nrow, vec, P0 + (size_t)b * PSTRIDE);
      if (!grid.sync()) return;
      block_reduce_all<T>(P0, nblk, j + 2, sh1);
      __syncthreads();
      if (tid == 0) {
        T hh = T(0);
        for (int k = 0; k <= j; ++k) hh += sh1[k] * sh1[k];
        const T ww = sh1[j + 1];
        const T n2 = ww - hh;
        s_reorth = n2 < T(0.5) * ww;
        s_nreorth += s_reorth;
        sh2[32] = n2;  // |w'|^2
      }
      __syncthreads();
      if (s_reorth) {
        // (4) second pass on w' = w - V h1: h2 = V^T w' and w'.w' in one reduction
        block_sub_scale<T>(a.V, sh1, j + 1, N, a.w, T(1), a.w, r0, nrow, vec, 0);
        __syncthreads();
        block_dots<T>(a.V, a.w, j + 1, 1, N, r0, nrow, vec, P2 + (size_t)b * PSTRIDE);
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
        sHc[j] += T(1);  // column j of H_K + I, the Hessenberg matrix of I + K
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
    a.flags[F_NREORTH] = s_nreorth;
    a.scal[S_BETA] = double(s_beta);
    a.scal[S_RESID] = double(s_beta);
    a.scal[S_BNORM] = s_bnorm;
    a.scal[S_TOL] = s_tol;
  }
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
  a.F = m->F;  // DIM + 1 (simplices)
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
  // evict-first operator loads when operator and Krylov basis do not fit the
  // 129 MB L2 together (the operator's lines then give way to the basis)
  const size_t es = sizeof(T);
  const size_t op = (size_t)m->E * a.n * a.n * es + (size_t)m->I * 2 * a.nb * a.nb * es;
  const size_t basis = (size_t)(a.m + 1) * (size_t)a.N * es;
  a.l2ef = op + basis > (size_t(96) << 20) ? 1 : 0;
}

template <int DIM, int NB, typename T>
__global__ void __launch_bounds__(NT, 1) k_gmres_coop(CoopArgs<T> a) {
  __shared__ GmresShared<T> sm;
  GridBarrier bar{cg::this_grid()};
  gmres_body<DIM, NB, T>(a, blockIdx.x, gridDim.x, bar, sm);
}

// barrier of a solve run by one thread-block cluster: the hardware cluster
// barrier (arrive with release, wait with acquire semantics at cluster
// scope, so the pushed products and partial sums written before it are seen
// by every block of the cluster after it)
struct ClusterBarrier {
  cg::cluster_group c;
  __device__ bool sync() {
    c.sync();
    return true;
  }
};

// The same solve by the blocks of one cluster (a small system: one SM
// would be latency-bound, a cooperative grid would need the device-wide
// barrier); the cluster's blocks are co-scheduled by the hardware, so
// several such solves run side by side on other streams.
template <int DIM, int NB, typename T>
__global__ void __launch_bounds__(NT, 1) k_gmres_cluster(CoopArgs<T> a) {
  __shared__ GmresShared<T> sm;
  cg::cluster_group cl = cg::this_cluster();
  ClusterBarrier bar{cl};
  gmres_body<DIM, NB, T>(a, (int)cl.block_rank(), (int)cl.num_blocks(), bar, sm);
}

}  // namespace
