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
// Per iteration: 3 grid barriers (5 with the second Gram-Schmidt pass).
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
constexpr int NT = 512;
constexpr int PSTRIDE = 33;  // partial slots per block

template <typename T>
struct CoopArgs {
  DevMesh md;
  const T* inv;      // [E][n][n] block inverses (column-major)
  const T* cpl;      // [I][2][nb][nb] coupling blocks (row-major)
  const int* spos;   // [F][Np]
  T* V;              // [(m+1)][N]
  T* w;              // [N]
  T* z;              // [N]
  T* part;           // [4][gridDim][PSTRIDE]
  double* dH;        // H | cs | sn | g | y
  int* flags;
  double* scal;
  int m, n, E;
  int64_t N;
};

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

// partial dots of the block's rows: k < cnt against V[k], k == cnt: w.w
// (when with_ww); warp q owns k = q, q+8, q+16, q+24, q+32
template <typename T>
__device__ void block_dots(const T* __restrict__ V, const T* __restrict__ w, int cnt, int with_ww,
                           int64_t N, int64_t r0, int nrow, T* __restrict__ pb) {
  const int lane = threadIdx.x & 31, q = threadIdx.x >> 5;
  const int tot = cnt + (with_ww ? 1 : 0);
  for (int k = q; k < tot; k += NT / 32) {
    const T* v = (k < cnt) ? V + (size_t)k * N + r0 : w + r0;
    const T* x = w + r0;
    T acc = T(0);
    for (int i = lane; i < nrow; i += 32) acc += v[i] * x[i];
    acc = wsum(acc);
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

// w -= sum_k V[k] h[k] on the block's rows; returns the block's |w|^2 (thread 0)
template <typename T>
__device__ T block_sub_norm(const T* __restrict__ V, const T* __restrict__ h, int cnt, int64_t N,
                            T* __restrict__ w, int64_t r0, int nrow, T* sred) {
  T acc = T(0);
  for (int i = threadIdx.x; i < nrow; i += NT) {
    const int64_t row = r0 + i;
    T a = w[row];
    for (int k = 0; k < cnt; ++k) a -= V[(size_t)k * N + row] * h[k];
    w[row] = a;
    acc += a * a;
  }
  acc = wsum(acc);
  if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = acc;
  __syncthreads();
  T t = T(0);
  if (threadIdx.x == 0)
    for (int q = 0; q < NT / 32; ++q) t += sred[q];
  __syncthreads();
  return t;
}

template <int DIM, int NB, typename T>
__global__ void __launch_bounds__(NT, 2) k_arnoldi_coop(CoopArgs<T> a) {
  cg::grid_group grid = cg::this_grid();
  const int nblk = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int n = NB > 0 ? NB : a.n, m = a.m;
  const int64_t N = a.N;
  // contiguous element range of this block
  const int epb = (a.E + nblk - 1) / nblk;
  const int e0 = min(a.E, b * epb), e1 = min(a.E, e0 + epb);
  const int64_t r0 = (int64_t)e0 * n;
  const int nrow = (e1 - e0) * n;
  T* P0 = a.part;                               // dots, first pass
  T* P1 = a.part + (size_t)nblk * PSTRIDE;      // |w|^2, first pass
  T* P2 = a.part + 2 * (size_t)nblk * PSTRIDE;  // dots, second pass
  T* P3 = a.part + 3 * (size_t)nblk * PSTRIDE;  // |w|^2, second pass
  __shared__ T sh1[33], sh2[33], sred[NT / 32], s_n2[1];
  __shared__ double scs[32], ssn[32], sg[33], sHc[33];
  __shared__ int s_done, s_its, s_reorth, s_jdone;
  __shared__ T s_hn;
  __shared__ double s_tol;
  double* Hg = a.dH;
  double* csg = a.dH + (size_t)(m + 1) * m;
  double* sng = csg + m;
  double* gg = sng + m;
  if (tid == 0) {
    s_done = a.flags[F_DONE];
    s_its = a.flags[F_ITS];
    s_tol = a.scal[S_TOL];
  }
  for (int k = tid; k <= m; k += NT) sg[k] = gg[k];
  if (tid == 0) s_jdone = 0;
  __syncthreads();
  for (int j = 0; j < m; ++j) {
    if (s_done) break;
    const T* vj = a.V + (size_t)j * N;
    // (1) z = D^-1 v_j on the block's elements
    for (int t = tid; t < nrow; t += NT) {
      const int le = t / n, r = t - le * n;
      const int e = e0 + le;
      a.z[(size_t)e * n + r] = block_row<NB, T>(a.inv + (size_t)e * n * n, vj + (size_t)e * n, r, n);
    }
    grid.sync();
    // (2) w = v_j + C z on the block's rows
    for (int t = tid; t < nrow; t += NT) {
      const int le = t / n, r = t - le * n;
      const int e = e0 + le;
      const int64_t row = (int64_t)e * n + r;
      a.w[row] = vj[row] + coupling_row<DIM, T>(a.md, a.cpl, a.spos, a.z, e, r, n);
    }
    __syncthreads();
    // (3) first Gram-Schmidt pass: dots with v_0..v_j and w.w
    block_dots<T>(a.V, a.w, j + 1, 1, N, r0, nrow, P0 + (size_t)b * PSTRIDE);
    grid.sync();
    block_reduce_all<T>(P0, nblk, j + 2, sh1);
    __syncthreads();
    T bn = block_sub_norm<T>(a.V, sh1, j + 1, N, a.w, r0, nrow, sred);
    if (tid == 0) P1[b * PSTRIDE] = bn;
    grid.sync();
    block_reduce_all<T>(P1, nblk, 1, s_n2);
    __syncthreads();
    if (tid == 0) s_reorth = double(s_n2[0]) < 0.5 * double(sh1[j + 1]);
    __syncthreads();
    if (s_reorth) {
      block_dots<T>(a.V, a.w, j + 1, 0, N, r0, nrow, P2 + (size_t)b * PSTRIDE);
      grid.sync();
      block_reduce_all<T>(P2, nblk, j + 1, sh2);
      __syncthreads();
      bn = block_sub_norm<T>(a.V, sh2, j + 1, N, a.w, r0, nrow, sred);
      if (tid == 0) P3[b * PSTRIDE] = bn;
      grid.sync();
      block_reduce_all<T>(P3, nblk, 1, s_n2);
    } else {
      for (int k = tid; k <= j; k += NT) sh2[k] = T(0);
    }
    __syncthreads();
    // (4) Hessenberg column j and Givens rotation (identical in every block)
    if (tid == 0) {
      const double hn = sqrt(double(s_n2[0]));
      for (int k = 0; k <= j; ++k) sHc[k] = double(sh1[k]) + double(sh2[k]);
      sHc[j + 1] = hn;
      for (int k = 0; k < j; ++k) {
        const double t0 = scs[k] * sHc[k] + ssn[k] * sHc[k + 1];
        sHc[k + 1] = -ssn[k] * sHc[k] + scs[k] * sHc[k + 1];
        sHc[k] = t0;
      }
      const double den = hypot(sHc[j], sHc[j + 1]);
      s_its += 1;
      s_hn = T(hn);
      if (!(den > 0.0) || !isfinite(den)) {
        s_done = 1;  // breakdown: keep the j columns built so far
      } else {
        scs[j] = sHc[j] / den;
        ssn[j] = sHc[j + 1] / den;
        sHc[j] = den;
        sHc[j + 1] = 0.0;
        sg[j + 1] = -ssn[j] * sg[j];
        sg[j] = scs[j] * sg[j];
        s_jdone = j + 1;
        const double resid = fabs(sg[j + 1]);
        if (resid <= s_tol || hn == 0.0 || s_its >= a.flags[F_ITERMAX]) s_done = 1;
      }
      if (b == 0) {
        double* Hc = Hg + (size_t)j * (m + 1);
        for (int k = 0; k <= j + 1; ++k) Hc[k] = sHc[k];
        a.scal[S_RESID] = fabs(sg[j + 1]);
      }
    }
    __syncthreads();
    // (5) v_{j+1} = w / |w| on the block's rows
    {
      const T hn = s_hn;
      const T inv = hn > T(0) ? T(1) / hn : T(0);
      T* vn = a.V + (size_t)(j + 1) * N;
      for (int i = tid; i < nrow; i += NT) vn[r0 + i] = a.w[r0 + i] * inv;
    }
    __syncthreads();
  }
  if (b == 0 && tid == 0) {
    a.flags[F_ITS] = s_its;
    a.flags[F_JDONE] = s_jdone;
    a.flags[F_DONE] = s_done;
    for (int k = 0; k <= m; ++k) gg[k] = sg[k];
    for (int k = 0; k < m; ++k) {
      csg[k] = scs[k];
      sng[k] = ssn[k];
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
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, NT, 0);
  (void)max_blocks_cache;
  int nblk = sms * (per_sm < 2 ? per_sm : 2);
  if (nblk > m->E) nblk = m->E;
  if (nblk > EG_COOP_MAX_BLOCKS) nblk = EG_COOP_MAX_BLOCKS;
  if (nblk <= 0) {
    eg_set_error("persistent Arnoldi kernel cannot be resident");
    return EG_ERR_UNSUPPORTED;
  }
  void* args[] = {&a};
  EG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(nblk), dim3(NT), args, 0, m->stream));
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

bool eg_coop_supported() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess) return false;
  return v != 0;
}
