// eg_arnoldi.cu -- one GMRES restart cycle (the Arnoldi loop) as a single
// persistent cooperative kernel.
//
// The Krylov vectors of the Newton systems are small (1.5 MB in FP32 for the
// 8192-triangle p=3 problem), so an Arnoldi step is dominated by
// synchronisation, not by HBM traffic.  One launch per cycle replaces the ~13
// launches per iteration of the stream version:
//   * block b owns a contiguous range of elements (and their rows) for the
//     whole cycle, so the block-Jacobi apply, the coupling apply, the
//     Gram-Schmidt updates and the scaling of the new basis vector touch only
//     its own rows; a grid barrier is needed only where data crosses blocks
//     (neighbour values of z = D^-1 v, and the dot-product partials);
//   * every block reduces the dot-product partials in the same order, so the
//     Hessenberg column, the re-orthogonalisation test (DGKS) and the Givens
//     rotation are bit-identical in every block: no broadcast is needed and
//     all blocks take the same branches (no barrier can be missed);
//   * block 0 alone writes the Hessenberg column, g and the flags that the
//     host and the least-squares kernel read after the launch.
// Per iteration: 2 grid barriers (3 with the second Gram-Schmidt pass).
// The operator is the right-preconditioned J M^-1 = I + C D^-1 (element blocks
// cancel with their inverses).
#include <cooperative_groups.h>

#include <cmath>

#include "eg_internal.h"
#include "eg_kernels.cuh"
#include "eg_krylov.cuh"
#include "eg_linalg.h"

namespace cg = cooperative_groups;

namespace {

enum { F_DONE = 0, F_JDONE = 1, F_ITS = 2, F_CONV = 3, F_ITERMAX = 4, F_REORTH = 5 };
enum { S_TOL = 0, S_RESID = 1, S_BETA = 2, S_BNORM = 3 };
constexpr int NT = 1024;  // one block per SM
constexpr int NB_MAX = 64;  // coupling-block rows handled by the face-side pass
constexpr int PSTRIDE = 33;  // partial slots per block

template <typename T>
struct CoopArgs {
  DevMesh md;
  const T* inv;      // [E][n][n] block inverses (column-major)
  const T* cpl;      // [I][2][nb][nb] coupling blocks (row-major)
  const int* spos;   // [F][Np]
  const int* fside;  // [E][F] coupling block of each element face, or -1
  T* cfs;            // [I][2][nb] coupling products of each face side
  T* V;              // [(m+1)][N]
  T* w;              // [N]
  T* z;              // [N]
  T* part;           // [4][gridDim][PSTRIDE]
  double* dH;        // H | cs | sn | g | y
  int* flags;
  double* scal;
  int m, n, E;
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

// One Arnoldi cycle.  Gram-Schmidt: classical, with the norm of the
// orthogonalised vector from the same reduction (|w'|^2 = w.w - |h|^2), and
// a second classical pass (whose reduction also yields w'.w') when
// |w'|^2 < |w|^2 / 2 (the DGKS criterion with eta = 1/sqrt 2).  The Givens
// rotations and the least-squares right-hand side are carried in T by one
// lane while the other warps form v_{j+1}.
template <int DIM, int NB, typename T>
__global__ void __launch_bounds__(NT, 1) k_arnoldi_coop(CoopArgs<T> a) {
  cg::grid_group grid = cg::this_grid();
  const int nblk = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int n = NB > 0 ? NB : a.n, m = a.m;
  const int64_t N = a.N;
  // contiguous element range of this block
  const int epb = (a.E + nblk - 1) / nblk;
  const int e0 = min(a.E, b * epb), e1 = min(a.E, e0 + epb);
  const int64_t r0 = (int64_t)e0 * n;
  const int nrow = (e1 - e0) * n;
  const bool vec = NB > 0 ? (NB % Vec<T>::W) == 0 : (a.n % Vec<T>::W) == 0;
  T* P0 = a.part;                               // first pass: dots and w.w
  T* P2 = a.part + 2 * (size_t)nblk * PSTRIDE;  // second pass: dots and w'.w'
  extern __shared__ __align__(16) unsigned char dsmem[];
  T* sZ = reinterpret_cast<T*>(dsmem);  // [ec][n] D^-1 v_j of a chunk of the block's elements
  __shared__ int sPerm[64], sSpos[128];
  __shared__ T sh1[33], sh2[33];
  __shared__ T scs[32], ssn[32], sg[33], sHc[33];
  __shared__ int s_done, s_its, s_reorth, s_jdone;
  __shared__ T s_inv;
  __shared__ double s_tol;
  double* Hg = a.dH;
  double* csg = a.dH + (size_t)(m + 1) * m;
  double* sng = csg + m;
  double* gg = sng + m;
  if (tid == 0) {
    s_done = a.flags[F_DONE];
    s_its = a.flags[F_ITS];
    s_tol = a.scal[S_TOL];
    s_jdone = 0;
  }
  for (int k = tid; k <= m; k += NT) sg[k] = T(gg[k]);
  for (int k = tid; k < a.F * a.S; k += NT) sPerm[k] = a.md.perm[k];
  for (int k = tid; k < a.F * a.md.Np; k += NT) sSpos[k] = a.spos[k];
  __syncthreads();
  for (int j = 0; j < m; ++j) {
    if (s_done) break;
    const T* vj = a.V + (size_t)j * N;
    T* vn = a.V + (size_t)(j + 1) * N;
    // (1) per chunk of the block's elements: z = D^-1 v_j into shared
    //     memory, then the push of C z to the neighbours' face sides
    for (int c0 = e0; c0 < e1; c0 += a.ec) {
      const int nl = min(a.ec, e1 - c0);
      for (int t = tid; t < nl * n; t += NT) {
        const int le = t / n, r = t - le * n;
        const int e = c0 + le;
        sZ[t] = block_row<NB, T>(a.inv + (size_t)e * n * n, vj + (size_t)e * n, r, n);
      }
      __syncthreads();
      face_push<DIM, T>(a, sZ, sPerm, c0, nl, a.cfs);
      __syncthreads();
    }
    grid.sync();
    // (2) w = v_j + sum over the faces whose stencil holds the row's node of
    //     the pushed product (own rows)
    {
      constexpr int NV = DIM + 2;
      for (int t = tid; t < nrow; t += NT) {
        const int le = t / n, r = t - le * n;
        const int j = r / NV, av = r - j * NV;
        const int e = e0 + le;
        const int64_t row = (int64_t)e * n + r;
        T acc = vj[row];
        for (int f = 0; f < a.F; ++f) {
          const int sp = sSpos[f * a.md.Np + j];
          if (sp < 0) continue;
          const int fs = a.fside[(int64_t)e * a.F + f];
          if (fs >= 0) acc += a.cfs[(size_t)fs * a.nb + sp * NV + av];
        }
        a.w[row] = acc;
      }
    }
    __syncthreads();
    // (3) first pass: h1 = V^T w and w.w in one reduction
    block_dots<T>(a.V, a.w, j + 1, 1, N, r0, nrow, vec, P0 + (size_t)b * PSTRIDE);
    grid.sync();
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
    T n2;
    if (s_reorth) {
      // (4) second pass on w' = w - V h1: h2 = V^T w' and w'.w' in one reduction
      block_sub_scale<T>(a.V, sh1, j + 1, N, a.w, T(1), a.w, r0, nrow, vec, 0);
      __syncthreads();
      block_dots<T>(a.V, a.w, j + 1, 1, N, r0, nrow, vec, P2 + (size_t)b * PSTRIDE);
      grid.sync();
      block_reduce_all<T>(P2, nblk, j + 2, sh2);
      __syncthreads();
      if (tid == 0) {
        T hh = T(0);
        for (int k = 0; k <= j; ++k) hh += sh2[k] * sh2[k];
        const T r = sh2[j + 1] - hh;
        sh2[32] = r > T(0) ? r : T(0);
      }
      __syncthreads();
      n2 = sh2[32];
    } else {
      n2 = sh2[32];
    }
    const T hn = sqrt(n2);
    const T inv = hn > T(0) ? T(1) / hn : T(0);
    // (5) lane 0 of warp 0: Hessenberg column j and its Givens rotation
    //     (identical in every block); warps 1.. : v_{j+1} = (w - V h) / hn
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
        const double resid = fabs(double(sg[j + 1]));
        if (resid <= s_tol || hn == T(0) || s_its >= a.flags[F_ITERMAX]) s_done = 1;
      }
      if (b == 0) {
        double* Hc = Hg + (size_t)j * (m + 1);
        for (int k = 0; k <= j + 1; ++k) Hc[k] = double(sHc[k]);
        a.scal[S_RESID] = fabs(double(sg[j + 1]));
      }
    } else if (tid >= 32) {
      if (s_reorth)
        block_sub_scale<T>(a.V, sh2, j + 1, N, a.w, inv, vn, r0, nrow, vec, 32);
      else
        block_sub_scale<T>(a.V, sh1, j + 1, N, a.w, inv, vn, r0, nrow, vec, 32);
    }
    __syncthreads();
  }
  if (b == 0 && tid == 0) {
    a.flags[F_ITS] = s_its;
    a.flags[F_JDONE] = s_jdone;
    a.flags[F_DONE] = s_done;
    for (int k = 0; k <= m; ++k) gg[k] = double(sg[k]);
    for (int k = 0; k < m; ++k) {
      csg[k] = double(scs[k]);
      sng[k] = double(ssn[k]);
    }
  }
}

template <typename T>
int launch_T(eg_ls* ls, int* max_blocks_cache) {
  eg_mesh* m = ls->lo->mesh;
  CoopArgs<T> a;
  a.md = dev_mesh(m);
  a.inv = (const T*)ls->pc->inv;
  a.cpl = (const T*)ls->lo->cpl;
  a.spos = ls->lo->spos;
  a.fside = ls->lo->fside;
  a.cfs = (T*)ls->cfs;
  a.nb = ls->lo->nb;
  a.S = m->S;
  a.F = m->F;
  a.nv = m->nv;
  a.V = (T*)ls->V;
  a.w = (T*)ls->w;
  a.z = (T*)ls->z;
  a.part = (T*)ls->part;
  a.dH = ls->dH;
  a.flags = ls->dflags;
  a.scal = ls->dscal;
  a.m = ls->m;
  a.n = ls->lo->n;
  a.E = m->E;
  a.N = m->ndof;
  void* fn = nullptr;
  switch (a.n) {
#define EG_CASE(NBV) \
  case NBV: fn = m->dim == 2 ? (void*)k_arnoldi_coop<2, NBV, T> : (void*)k_arnoldi_coop<3, NBV, T>; break;
    EG_CASE(12) EG_CASE(24) EG_CASE(28) EG_CASE(40) EG_CASE(48) EG_CASE(60) EG_CASE(72) EG_CASE(30)
#undef EG_CASE
    default: fn = m->dim == 2 ? (void*)k_arnoldi_coop<2, 0, T> : (void*)k_arnoldi_coop<3, 0, T>;
  }
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  (void)max_blocks_cache;
  // elements per block, and per shared-memory chunk of D^-1 v values
  const size_t side_bytes = (size_t)a.n * sizeof(T);
  int nblk = sms;
  if (nblk > m->E) nblk = m->E;
  if (nblk > EG_COOP_MAX_BLOCKS) nblk = EG_COOP_MAX_BLOCKS;
  const int epb = (m->E + nblk - 1) / nblk;
  int ec = (int)((40 * 1024) / side_bytes);
  if (ec < 1) ec = 1;
  if (ec > epb) ec = epb;
  a.ec = ec;
  const size_t smem = (size_t)ec * side_bytes;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, NT, smem);
  if (per_sm < 1) nblk = 0;
  if (nblk <= 0) {
    eg_set_error("persistent Arnoldi kernel cannot be resident");
    return EG_ERR_UNSUPPORTED;
  }
  void* args[] = {&a};
  EG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(nblk), dim3(NT), args, smem, m->stream));
  m->launches += 1;
  return EG_OK;
}

}  // namespace

// one Arnoldi cycle (up to ls->m iterations) of the right-preconditioned
// GMRES as one cooperative launch; partial sums need 4 * grid * 33 values of
// ls->part, which eg_ls_create sizes for up to 2 blocks per SM.
int eg_arnoldi_coop(eg_ls* ls) {
  static int cache_f = 0, cache_d = 0;
  return ls->lo->prec == EG_F64 ? launch_T<double>(ls, &cache_d) : launch_T<float>(ls, &cache_f);
}

bool eg_coop_usable(const eg_ls* ls) {
  const eg_mesh* m = ls->lo->mesh;
  return ls->lo->nb <= NB_MAX && m->F * m->S <= 64 && m->F * m->Np <= 128 && m->I > 0 &&
         eg_coop_supported();
}

bool eg_coop_supported() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess) return false;
  return v != 0;
}
