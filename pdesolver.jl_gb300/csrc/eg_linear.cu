// eg_linear.cu -- linear operator (explicit Jacobian), element block-Jacobi
// preconditioner and right-preconditioned GMRES(m).
//
// Reference: src/linearsolvers/LinearSolvers.jl:68-660 (calcLinearOperator,
// applyLinearOperator, calcPC, applyPC, linearSolve, setTolerances),
// ls_standard.jl:210-371 (PETSc KSP GMRES), NonlinearSolvers/preconditioning.jl
// (NewtonBDiagPC: getrf!/getrs per element block).
//
// All kernels are templated on the operator precision T (double: plain FP64
// path; float: the FP32 Jacobian / preconditioner / Krylov of the mixed
// path, FP32 accumulation).
#include <cmath>
#include <cstring>
#include <algorithm>
#include <vector>

#include "eg_internal.h"
#include "eg_kernels.cuh"
#include "eg_linalg.h"
#include "eg_krylov.cuh"

namespace {

// ---------------------------------------------------------------- SpMV
// y[e][r] = sum_c diag[e][c][r] x[e][c] + face couplings of row r.
// One CTA per `epb` elements, one thread per row; x of the CTA's elements in
// shared memory; coupling operands read from the neighbours (L2).
template <int DIM, int NB, typename T>
__global__ void k_spmv(DevMesh md, const T* __restrict__ diag, const T* __restrict__ cpl,
                       const int* __restrict__ spos, const T* __restrict__ x, T* __restrict__ y,
                       int epb, const int* __restrict__ done) {
  constexpr int NV = DIM + 2;
  if (done && *done) return;
  extern __shared__ unsigned char smraw[];
  T* sx = reinterpret_cast<T*>(smraw);
  const int n = NB > 0 ? NB : md.Np * NV;
  const int e0 = blockIdx.x * epb;
  const int nloc = min(epb, md.E - e0);
  for (int t = threadIdx.x; t < nloc * n; t += blockDim.x) sx[t] = x[(size_t)e0 * n + t];
  __syncthreads();
  const int le = threadIdx.x / n, r = threadIdx.x - le * n;
  if (le >= nloc) return;
  const int e = e0 + le;
  T acc = block_row<NB, T>(diag + (size_t)e * n * n, sx + (size_t)le * n, r, n);
  acc += coupling_row<DIM, T>(md, cpl, spos, x, e, r, n);
  y[(size_t)e * n + r] = acc;
}

// Right-preconditioned operator without the element blocks:
// (D + C) D^-1 v = v + C z with z = D^-1 v (z computed by k_block_apply).
// Inside the Arnoldi loop this replaces k_spmv + the diagonal-block read.
// v == nullptr: w = C z alone (the coupling part K v of I + K).
template <int DIM, typename T>
__global__ void k_cpl_apply(DevMesh md, const T* __restrict__ cpl, const int* __restrict__ spos,
                            const T* __restrict__ v, const T* __restrict__ z, T* __restrict__ w,
                            const int* __restrict__ done) {
  constexpr int NV = DIM + 2;
  if (done && *done) return;
  const int n = md.Np * NV;
  const int64_t N = (int64_t)md.E * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(t / n), r = (int)(t - (int64_t)e * n);
    w[t] = (v ? v[t] : T(0)) + coupling_row<DIM, T>(md, cpl, spos, z, e, r, n);
  }
}

// ---------------------------------------------------------------- block-Jacobi
// In-place Gauss-Jordan inversion with partial pivoting of one element block
// per CTA (column-major n x n in shared memory).  Rows are swapped during the
// elimination; the inverse's columns are swapped back at the end.
template <typename T>
__global__ void k_block_inverse(const T* __restrict__ blocks, T* __restrict__ inv, int n,
                                unsigned int* __restrict__ status) {
  extern __shared__ unsigned char smraw[];
  T* A = reinterpret_cast<T*>(smraw);                       // A[c*n + r]
  int* piv = reinterpret_cast<int*>(A + (size_t)n * n);
  __shared__ int s_p;
  __shared__ T s_d;
  __shared__ int s_bad;
  const int e = blockIdx.x;
  const T* src = blocks + (size_t)e * n * n;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) A[t] = src[t];
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      int p = k;
      T best = fabs(A[(size_t)k * n + k]);
      for (int i = k + 1; i < n; ++i) {
        const T v = fabs(A[(size_t)k * n + i]);
        if (v > best) { best = v; p = i; }
      }
      s_p = p;
      piv[k] = p;
      if (!(best > T(0))) s_bad = 1;
    }
    __syncthreads();
    const int p = s_p;
    if (p != k)
      for (int c = threadIdx.x; c < n; c += blockDim.x) {
        const T t0 = A[(size_t)c * n + k];
        A[(size_t)c * n + k] = A[(size_t)c * n + p];
        A[(size_t)c * n + p] = t0;
      }
    __syncthreads();
    if (threadIdx.x == 0) {
      const T piv_v = A[(size_t)k * n + k];
      s_d = s_bad ? T(0) : T(1) / piv_v;
      A[(size_t)k * n + k] = T(1);
    }
    __syncthreads();
    const T d = s_d;
    for (int c = threadIdx.x; c < n; c += blockDim.x) A[(size_t)c * n + k] *= d;  // row k
    __syncthreads();
    // eliminate column k from the other rows: A[i][c] -= A[i][k] * A[k][c]
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int c = t / n, i = t - c * n;
      if (i == k || c == k) continue;
      A[t] -= A[(size_t)k * n + i] * A[(size_t)c * n + k];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      if (i != k) A[(size_t)k * n + i] = -A[(size_t)k * n + i] * d;
    __syncthreads();
  }
  // undo the row interchanges as column interchanges, last first
  for (int k = n - 1; k >= 0; --k) {
    const int p = piv[k];
    if (p != k)
      for (int r = threadIdx.x; r < n; r += blockDim.x) {
        const T t0 = A[(size_t)k * n + r];
        A[(size_t)k * n + r] = A[(size_t)p * n + r];
        A[(size_t)p * n + r] = t0;
      }
    __syncthreads();
  }
  if (threadIdx.x == 0 && s_bad) atomicOr(status, EG_DEV_LU_PIVOT);
  T* dst = inv + (size_t)e * n * n;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) dst[t] = A[t];
}

// y_e = inv_e x_e (batched dense matrix-vector product, thread per row)
template <int NB, typename T>
__global__ void k_block_apply(const T* __restrict__ inv, const T* __restrict__ x, T* __restrict__ y,
                              int E, int nrt, int epb, const int* __restrict__ done) {
  if (done && *done) return;
  extern __shared__ unsigned char smraw[];
  T* sx = reinterpret_cast<T*>(smraw);
  const int n = NB > 0 ? NB : nrt;
  const int e0 = blockIdx.x * epb;
  const int nloc = min(epb, E - e0);
  for (int t = threadIdx.x; t < nloc * n; t += blockDim.x) sx[t] = x[(size_t)e0 * n + t];
  __syncthreads();
  const int le = threadIdx.x / n, r = threadIdx.x - le * n;
  if (le >= nloc) return;
  y[(size_t)(e0 + le) * n + r] =
      block_row<NB, T>(inv + (size_t)(e0 + le) * n * n, sx + (size_t)le * n, r, n);
}

// ---------------------------------------------------------------- vectors
template <typename T>
__global__ void k_to_T(const double* __restrict__ s, T* __restrict__ d, int64_t n, double scale) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = T(scale * s[i]);
}
template <typename T>
__global__ void k_from_T(const T* __restrict__ s, double* __restrict__ d, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = double(s[i]);
}

// partial[b][k] = sum over block b's rows of V[k][i] * w[i], k < cnt
template <typename T, int NT>
__global__ void k_multidot(const T* __restrict__ V, const T* __restrict__ w, int cnt, int64_t N,
                           T* __restrict__ part, int stride) {
  __shared__ T sh[NT];
  const int64_t chunk = (N + gridDim.x - 1) / gridDim.x;
  const int64_t lo = blockIdx.x * chunk;
  const int64_t hi = min(N, lo + chunk);
  for (int k = 0; k < cnt; ++k) {
    const T* v = V + (size_t)k * N;
    T s = T(0);
    for (int64_t i = lo + threadIdx.x; i < hi; i += NT) s += v[i] * w[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = NT / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[(size_t)blockIdx.x * stride + k] = sh[0];
    __syncthreads();
  }
}

// out[k] (+)= sum_b part[b][k]; mode 0: assign, 1: accumulate, 2: assign sqrt
template <typename T, int NT>
__global__ void k_reduce_parts(const T* __restrict__ part, int nblk, int cnt, int stride,
                               T* __restrict__ out, int mode) {
  __shared__ T sh[NT];
  for (int k = 0; k < cnt; ++k) {
    T s = T(0);
    for (int b = threadIdx.x; b < nblk; b += NT) s += part[(size_t)b * stride + k];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = NT / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      if (mode == 0) out[k] = sh[0];
      else if (mode == 1) out[k] += sh[0];
      else out[k] = sqrt(sh[0]);
    }
    __syncthreads();
  }
}

// w -= sum_k V[k] h[k]  (h on the device)
template <typename T>
__global__ void k_sub_Vh(const T* __restrict__ V, const T* __restrict__ h, int cnt, int64_t N,
                         T* __restrict__ w) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    T acc = w[i];
    for (int k = 0; k < cnt; ++k) acc -= V[(size_t)k * N + i] * h[k];
    w[i] = acc;
  }
}

// z = sum_k V[k] y[k]
template <typename T>
__global__ void k_Vy(const T* __restrict__ V, const T* __restrict__ yv, int cnt, int64_t N,
                     T* __restrict__ z) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    T acc = T(0);
    for (int k = 0; k < cnt; ++k) acc += V[(size_t)k * N + i] * yv[k];
    z[i] = acc;
  }
}

// dst = src * (1/nrm[0]) (nrm[0] == 0 leaves dst = 0)
template <typename T>
__global__ void k_scale_by_inv(const T* __restrict__ src, const T* __restrict__ nrm, int64_t N,
                               T* __restrict__ dst) {
  const T s = nrm[0];
  const T inv = (s > T(0)) ? T(1) / s : T(0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i] * inv;
}

// y = a*x + b*y
template <typename T>
__global__ void k_axpby(T a, const T* __restrict__ x, T b, T* __restrict__ y, int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b > 152 * 16 ? 152 * 16 : (b < 1 ? 1 : b));
}

// element-block sizes with a compiled specialisation (Np * nv of the tri
// Omega/Gamma operators p = 1..4 and the tet diagonal-E p = 1)
#define EG_NB_CASES(X) X(12) X(24) X(28) X(40) X(48) X(60) X(72) X(30)

template <int DIM, typename T>
void launch_spmv(eg_mesh* m, const DevMesh& md, const eg_lo* lo, const T* x, T* y, int blocks,
                 int threads, size_t smem, int epb, const int* done) {
  const T* D = (const T*)lo->diag;
  const T* Cp = (const T*)lo->cpl;
  switch (lo->n) {
#define EG_CASE(NBV) \
  case NBV: k_spmv<DIM, NBV, T><<<blocks, threads, smem, m->stream>>>(md, D, Cp, lo->spos, x, y, epb, done); return;
    EG_NB_CASES(EG_CASE)
#undef EG_CASE
    default:
      k_spmv<DIM, 0, T><<<blocks, threads, smem, m->stream>>>(md, D, Cp, lo->spos, x, y, epb, done);
  }
}

template <typename T>
int spmv_T(eg_lo* lo, const T* x, T* y, const int* done = nullptr) {
  eg_mesh* m = lo->mesh;
  DevMesh md = dev_mesh(m);
  const int n = lo->n;
  int epb = 256 / n;
  if (epb < 1) epb = 1;
  const int blocks = (m->E + epb - 1) / epb;
  const size_t smem = sizeof(T) * (size_t)epb * n;
  eg_phase_begin(m, EG_PHASE_OTHER);
  if (m->dim == 2)
    launch_spmv<2, T>(m, md, lo, x, y, blocks, epb * n, smem, epb, done);
  else
    launch_spmv<3, T>(m, md, lo, x, y, blocks, epb * n, smem, epb, done);
  eg_phase_end(m, EG_PHASE_OTHER, 1);
  return EG_OK;
}

template <typename T>
int cplapply_T(eg_lo* lo, const T* v, const T* z, T* w, const int* done) {
  eg_mesh* m = lo->mesh;
  DevMesh md = dev_mesh(m);
  const int64_t N = m->ndof;
  int blocks = (int)((N + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  eg_phase_begin(m, EG_PHASE_OTHER);
  if (m->dim == 2)
    k_cpl_apply<2, T><<<blocks, 256, 0, m->stream>>>(md, (const T*)lo->cpl, lo->spos, v, z, w, done);
  else
    k_cpl_apply<3, T><<<blocks, 256, 0, m->stream>>>(md, (const T*)lo->cpl, lo->spos, v, z, w, done);
  eg_phase_end(m, EG_PHASE_OTHER, 1);
  return EG_OK;
}

template <typename T>
int pcapply_T(eg_pc* pc, const T* x, T* y, const int* done = nullptr) {
  eg_lo* lo = pc->lo;
  eg_mesh* m = lo->mesh;
  const int n = lo->n;
  int epb = 256 / n;
  if (epb < 1) epb = 1;
  const int blocks = (m->E + epb - 1) / epb;
  const size_t smem = sizeof(T) * (size_t)epb * n;
  const T* A = (const T*)pc->inv;
  eg_phase_begin(m, EG_PHASE_OTHER);
  switch (n) {
#define EG_CASE(NBV) \
  case NBV: k_block_apply<NBV, T><<<blocks, epb * n, smem, m->stream>>>(A, x, y, m->E, n, epb, done); break;
    EG_NB_CASES(EG_CASE)
#undef EG_CASE
    default:
      k_block_apply<0, T><<<blocks, epb * n, smem, m->stream>>>(A, x, y, m->E, n, epb, done);
  }
  eg_phase_end(m, EG_PHASE_OTHER, 1);
  return EG_OK;
}

// ------------------------------------------------------------ transposes
// Coupling part of row (e, j, a) of J^T x: row (e, j, a) of J^T is column
// (e, j, a) of J; for each interface face of e whose stencil holds node j it
// takes column (s, a) of the neighbour's coupling block (the block whose rows
// are the neighbour's stencil and whose columns are e's).
template <int DIM, typename T>
__device__ __forceinline__ T coupling_col(const DevMesh& md, const T* __restrict__ cpl,
                                          const int* __restrict__ spos, const T* __restrict__ x, int e,
                                          int r, int n) {
  constexpr int NV = DIM + 2;
  constexpr int F = DIM + 1;
  const int Np = md.Np, S = md.S, nb = S * NV, Nf = md.Nf;
  const int j = r / NV, a = r - j * NV;
  T acc = T(0);
  for (int f = 0; f < F; ++f) {
    const int s = spos[f * Np + j];
    if (s < 0) continue;
    const EFace ef = md.eface[(size_t)e * F + f];
    if (ef.slot >= md.I) continue;
    const int* itf = md.ifaces + 5 * ef.slot;
    const int en = ef.side ? itf[0] : itf[1];
    const int fn = ef.side ? itf[2] : itf[3];
    const int o = itf[4];
    const int blk = ef.slot * 2 + (1 - ef.side);  // rows: the neighbour's stencil
    const T* xn = x + (size_t)en * n;
    if (md.sparse_face) {
      // the neighbour's row node facing e's node s
      const int sp = (1 - ef.side) == 0 ? md.nbrinv[o * Nf + s] : md.nbrperm[o * Nf + s];
      const T* C = cpl + ((size_t)blk * S + sp) * NV * NV;
      const T* xs = xn + md.perm[fn * S + sp] * NV;
      for (int b = 0; b < NV; ++b) acc += C[b * NV + a] * xs[b];
    } else {
      const T* C = cpl + (size_t)blk * nb * nb;  // row-major [row][col]
      for (int sp = 0; sp < S; ++sp) {
        const T* xs = xn + md.perm[fn * S + sp] * NV;
        for (int b = 0; b < NV; ++b) acc += C[(size_t)(sp * NV + b) * nb + s * NV + a] * xs[b];
      }
    }
  }
  return acc;
}

// y = J^T x (applyLinearOperatorTranspose, LinearSolvers.jl:533; the PETSc
// operator runs MatMultTranspose, lo_petscmat.jl:143-160), one thread per row
// of y: column r of e's element block, plus the coupling columns.  With
// `done` non-null the launch does nothing while *done != 0.
template <int DIM, typename T>
__global__ void k_spmv_t(DevMesh md, const T* __restrict__ diag, const T* __restrict__ cpl,
                         const int* __restrict__ spos, const T* __restrict__ x, T* __restrict__ y,
                         int n, const int* __restrict__ done) {
  if (done && *done) return;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)md.E * n) return;
  const int e = (int)(t / n), r = (int)(t - (int64_t)e * n);
  const T* col = diag + ((size_t)e * n + r) * n;  // column r of the element block
  const T* xe = x + (size_t)e * n;
  T acc = T(0);
  for (int i = 0; i < n; ++i) acc += col[i] * xe[i];
  y[t] = acc + coupling_col<DIM, T>(md, cpl, spos, x, e, r, n);
}

// w = v + C^T z: the transposed right-preconditioned operator
// J^T M^-T v = (M^-1 J)^T v = v + C^T D^-T v with z = D^-T v (the element
// blocks cancel with their inverses), coupling blocks only; v == nullptr:
// w = C^T z alone
template <int DIM, typename T>
__global__ void k_cpl_apply_t(DevMesh md, const T* __restrict__ cpl, const int* __restrict__ spos,
                              const T* __restrict__ v, const T* __restrict__ z, T* __restrict__ w, int n,
                              const int* __restrict__ done) {
  if (done && *done) return;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)md.E * n) return;
  const int e = (int)(t / n), r = (int)(t - (int64_t)e * n);
  w[t] = (v ? v[t] : T(0)) + coupling_col<DIM, T>(md, cpl, spos, z, e, r, n);
}

// y = M^-T x (applyPCTranspose, LinearSolvers.jl:277): the transposed element
// inverses, one thread per row
template <typename T>
__global__ void k_block_apply_t(const T* __restrict__ inv, const T* __restrict__ x, T* __restrict__ y,
                                int E, int n, const int* __restrict__ done) {
  if (done && *done) return;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)E * n) return;
  const int e = (int)(t / n), r = (int)(t - (int64_t)e * n);
  const T* col = inv + ((size_t)e * n + r) * n;
  const T* xe = x + (size_t)e * n;
  T acc = T(0);
  for (int i = 0; i < n; ++i) acc += col[i] * xe[i];
  y[t] = acc;
}

template <typename T>
void launch_transpose(eg_lo* lo, const T* inv, const T* x, T* y, const int* done = nullptr) {
  eg_mesh* m = lo->mesh;
  const int64_t rows = (int64_t)m->E * lo->n;
  const int blocks = (int)((rows + 255) / 256);
  eg_phase_begin(m, EG_PHASE_OTHER);
  if (inv)
    k_block_apply_t<T><<<blocks, 256, 0, m->stream>>>(inv, x, y, m->E, lo->n, done);
  else if (m->dim == 2)
    k_spmv_t<2, T><<<blocks, 256, 0, m->stream>>>(dev_mesh(m), (const T*)lo->diag, (const T*)lo->cpl,
                                                  lo->spos, x, y, lo->n, done);
  else
    k_spmv_t<3, T><<<blocks, 256, 0, m->stream>>>(dev_mesh(m), (const T*)lo->diag, (const T*)lo->cpl,
                                                  lo->spos, x, y, lo->n, done);
  eg_phase_end(m, EG_PHASE_OTHER, 1);
}

template <typename T>
void launch_cpl_transpose(eg_lo* lo, const T* v, const T* z, T* w, const int* done) {
  eg_mesh* m = lo->mesh;
  const int64_t rows = (int64_t)m->E * lo->n;
  const int blocks = (int)((rows + 255) / 256);
  eg_phase_begin(m, EG_PHASE_OTHER);
  if (m->dim == 2)
    k_cpl_apply_t<2, T><<<blocks, 256, 0, m->stream>>>(dev_mesh(m), (const T*)lo->cpl, lo->spos, v, z, w,
                                                       lo->n, done);
  else
    k_cpl_apply_t<3, T><<<blocks, 256, 0, m->stream>>>(dev_mesh(m), (const T*)lo->cpl, lo->spos, v, z, w,
                                                       lo->n, done);
  eg_phase_end(m, EG_PHASE_OTHER, 1);
}

// Register-tiled Gauss-Jordan inversion for blocks of 33..128 unknowns, one
// CTA of NW warps per element block.  Thread (lane, warp) keeps rows
// lane + 32 r (r < MR) and columns warp + NW c (c < MC) in registers.
// Partial pivoting is implicit: the pivot of column k is the unused row p of
// largest |A[p][k]| (ties: lowest row), found by one warp with shuffles; row p
// is scaled in place and eliminated from the others, so no rows move.  Row p
// is read by every warp from its own lane p % 32 (shuffles), column k goes
// through a double-buffered shared array, so one barrier per column suffices.
// With S the in-place result and perm[k] the pivot row of column k,
// A^-1[r][c] = S[perm[r]][q] where perm[q] = c.
// register row r (warp-uniform) of a thread's tile, through branches on the
// uniform index so that only one copy executes (no per-element selects)
template <typename T, int MR, int MC>
__device__ __forceinline__ void tile_row_shfl(const T (&a)[MR][MC], int r, int src_lane, T scale,
                                              T (&out)[MC]) {
#pragma unroll
  for (int rr = 0; rr < MR; ++rr)
    if (rr == r) {
#pragma unroll
      for (int c = 0; c < MC; ++c) out[c] = __shfl_sync(0xffffffffu, a[rr][c], src_lane) * scale;
    }
}

template <typename T, int MR, int MC, int NW>
__global__ void __launch_bounds__(32 * NW) k_block_inverse_reg(const T* __restrict__ blocks,
                                                                T* __restrict__ inv, int n,
                                                                unsigned int* __restrict__ status) {
  extern __shared__ unsigned char smraw[];
  T* S = reinterpret_cast<T*>(smraw);                      // [n][n] column-major, at the end
  T* colk = S + (size_t)n * n;                             // [2][32 MR] column k
  int* sp = reinterpret_cast<int*>(colk + 2 * 32 * MR);    // [2] pivot row
  int* perm = sp + 2;                                      // [n]
  int* iperm = perm + n;                                   // [n]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const T* src = blocks + (size_t)blockIdx.x * n * n;
  T a[MR][MC];
  unsigned used = 0;  // bit r: row lane + 32 r is a pivot row already (or beyond n)
#pragma unroll
  for (int r = 0; r < MR; ++r) {
    const int i = lane + 32 * r;
    if (i >= n) used |= 1u << r;
#pragma unroll
    for (int c = 0; c < MC; ++c) {
      const int col = warp + NW * c;
      a[r][c] = (i < n && col < n) ? src[(size_t)col * n + i] : T(0);
    }
  }
  bool bad = false;
  for (int k = 0; k < n; ++k) {
    const int buf = k & 1;
    T* ck = colk + buf * 32 * MR;
    const bool kwarp = warp == (k % NW);  // this warp holds column k, as its column kc
    const int kc = k / NW;
    if (kwarp) {
      T best = T(-1);
      int bi = n;
#pragma unroll
      for (int c = 0; c < MC; ++c)
        if (c == kc) {
#pragma unroll
          for (int r = 0; r < MR; ++r) {
            const T v = a[r][c];
            ck[lane + 32 * r] = v;
            // NaN ranks above every number, so some unused row (there are
            // n - k) is always chosen and the pivot check below flags it
            const T av = isnan(v) ? T(INFINITY) : fabs(v);
            if (!((used >> r) & 1u) && av > best) {
              best = av;
              bi = lane + 32 * r;
            }
          }
        }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const T ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (lane == 0) sp[buf] = bi;
    }
    __syncthreads();
    const int p = sp[buf];
    const T pv = ck[p];
    bad = bad || !(fabs(pv) > T(0));
    const T d = bad ? T(0) : T(1) / pv;
    T rc[MC];  // scaled pivot row, this thread's columns
    tile_row_shfl<T, MR, MC>(a, p >> 5, p & 31, d, rc);
    // rows: r_i -= f_i r_p (every column; column k is set below)
#pragma unroll
    for (int r = 0; r < MR; ++r) {
      const T f = ck[lane + 32 * r];
#pragma unroll
      for (int c = 0; c < MC; ++c) a[r][c] = fma(-f, rc[c], a[r][c]);
    }
    // the pivot row becomes the scaled row, column k becomes -f d (d in the
    // pivot row): the in-place inverse's new column
    if (lane == (p & 31)) {
#pragma unroll
      for (int r = 0; r < MR; ++r)
        if (r == (p >> 5)) {
#pragma unroll
          for (int c = 0; c < MC; ++c) a[r][c] = rc[c];
          used |= 1u << r;
        }
    }
    if (kwarp) {
#pragma unroll
      for (int c = 0; c < MC; ++c)
        if (c == kc) {
#pragma unroll
          for (int r = 0; r < MR; ++r)
            a[r][c] = (lane + 32 * r == p) ? d : -ck[lane + 32 * r] * d;
        }
    }
    if (threadIdx.x == 0) perm[k] = p;
  }
  // gather through shared memory into column-major A^-1
#pragma unroll
  for (int r = 0; r < MR; ++r)
#pragma unroll
    for (int c = 0; c < MC; ++c) {
      const int i = lane + 32 * r, col = warp + NW * c;
      if (i < n && col < n) S[(size_t)col * n + i] = a[r][c];
    }
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) iperm[perm[k]] = k;
  __syncthreads();
  T* dst = inv + (size_t)blockIdx.x * n * n;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    const int c = t / n, r = t - c * n;
    dst[t] = S[(size_t)iperm[c] * n + perm[r]];
  }
  if (bad && threadIdx.x == 0) atomicOr(status, EG_DEV_LU_PIVOT);
}

// dynamic shared memory of k_block_inverse_reg
template <typename T, int MR>
size_t block_inverse_reg_smem(int n) {
  return sizeof(T) * ((size_t)n * n + 2 * 32 * MR) + sizeof(int) * (2 + 2 * (size_t)n);
}

template <typename T>
int pccalc_T(eg_pc* pc) {
  eg_lo* lo = pc->lo;
  eg_mesh* m = lo->mesh;
  const int n = lo->n;
  eg_phase_begin(m, EG_PHASE_OTHER);
  const T* A = (const T*)lo->diag;
  T* X = (T*)pc->inv;
  // MC x NW columns cover the block: 8 warps of 8 or 12 columns up to 96
  // unknowns; up to 128, 16 warps of 8 columns in FP32 (4 x 8 values and 64
  // registers per thread, two blocks per SM: 18 % faster than 8 warps of 16
  // columns on 115-unknown blocks) and 8 warps of 16 columns in FP64 (the
  // 16-warp tile measured 0.7 % slower there)
#define EG_INV_REG(MR, MC, NW)                                                                  \
  {                                                                                           \
    const size_t smem = block_inverse_reg_smem<T, MR>(n);                                     \
    cudaFuncSetAttribute(k_block_inverse_reg<T, MR, MC, NW>,                                  \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);            \
    k_block_inverse_reg<T, MR, MC, NW><<<m->E, 32 * NW, smem, m->stream>>>(A, X, n, m->status); \
  }
  if (n <= 32) {
    const size_t smem = sizeof(T) * (size_t)n * n + sizeof(int) * n;
    cudaFuncSetAttribute(k_block_inverse<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    k_block_inverse<T><<<m->E, 256, smem, m->stream>>>(A, X, n, m->status);
  } else if (n <= 64) {
    EG_INV_REG(2, 8, 8)
  } else if (n <= 96) {
    EG_INV_REG(3, 12, 8)
  } else if (sizeof(T) == 4) {
    EG_INV_REG(4, 8, 16)
  } else {
    EG_INV_REG(4, 16, 8)
  }
#undef EG_INV_REG
  eg_phase_end(m, EG_PHASE_OTHER, 1);
  return EG_OK;
}

}  // namespace

size_t eg_lo_coupling_size(const eg_lo* lo) {
  const eg_mesh* m = lo->mesh;
  return lo->cpl_sparse ? (size_t)m->I * 2 * m->S * m->nv * m->nv
                        : (size_t)m->I * 2 * lo->nb * lo->nb;
}

// ====================================================================== C ABI
int eg_convert(eg_mesh* m, const double* src, void* dst, int prec, int64_t n, double scale) {
  const int g = grid_for(n);
  if (prec == EG_F64)
    k_to_T<double><<<g, 256, 0, m->stream>>>(src, (double*)dst, n, scale);
  else
    k_to_T<float><<<g, 256, 0, m->stream>>>(src, (float*)dst, n, scale);
  m->launches += 1;
  return EG_OK;
}

int eg_convert_back(eg_mesh* m, const void* src, double* dst, int prec, int64_t n) {
  const int g = grid_for(n);
  if (prec == EG_F64)
    k_from_T<double><<<g, 256, 0, m->stream>>>((const double*)src, dst, n);
  else
    k_from_T<float><<<g, 256, 0, m->stream>>>((const float*)src, dst, n);
  m->launches += 1;
  return EG_OK;
}

int eg_lo_apply_T(eg_lo* lo, const void* x, void* y, const int* done) {
  return lo->prec == EG_F64 ? spmv_T<double>(lo, (const double*)x, (double*)y, done)
                            : spmv_T<float>(lo, (const float*)x, (float*)y, done);
}

int eg_cpl_apply_T(eg_lo* lo, const void* v, const void* z, void* w, const int* done) {
  return lo->prec == EG_F64 ? cplapply_T<double>(lo, (const double*)v, (const double*)z, (double*)w, done)
                            : cplapply_T<float>(lo, (const float*)v, (const float*)z, (float*)w, done);
}

int eg_pc_apply_T(eg_pc* pc, const void* x, void* y, const int* done) {
  return pc->lo->prec == EG_F64 ? pcapply_T<double>(pc, (const double*)x, (double*)y, done)
                                : pcapply_T<float>(pc, (const float*)x, (float*)y, done);
}

int eg_lo_apply_t_T(eg_lo* lo, const void* x, void* y, const int* done) {
  if (lo->prec == EG_F64)
    launch_transpose<double>(lo, nullptr, (const double*)x, (double*)y, done);
  else
    launch_transpose<float>(lo, nullptr, (const float*)x, (float*)y, done);
  return EG_OK;
}

int eg_cpl_apply_t_T(eg_lo* lo, const void* v, const void* z, void* w, const int* done) {
  if (lo->prec == EG_F64)
    launch_cpl_transpose<double>(lo, (const double*)v, (const double*)z, (double*)w, done);
  else
    launch_cpl_transpose<float>(lo, (const float*)v, (const float*)z, (float*)w, done);
  return EG_OK;
}

int eg_pc_apply_t_T(eg_pc* pc, const void* x, void* y, const int* done) {
  if (pc->lo->prec == EG_F64)
    launch_transpose<double>(pc->lo, (const double*)pc->inv, (const double*)x, (double*)y, done);
  else
    launch_transpose<float>(pc->lo, (const float*)pc->inv, (const float*)x, (float*)y, done);
  return EG_OK;
}

static void lo_free(eg_lo* lo) {
  if (!lo) return;
  void* bufs[] = {lo->diag, lo->cpl, lo->dF, lo->spos, lo->fside, lo->xT, lo->yT, lo->xd, lo->yd};
  for (void* b : bufs)
    if (b) cudaFree(b);
  delete lo;
}

extern "C" int eg_lo_create(eg_mesh* m, int32_t precision, eg_lo** out) {
  if (!m || !out || (precision != EG_F64 && precision != EG_F32)) {
    eg_set_error("eg_lo_create: invalid argument");
    return EG_ERR_INVALID;
  }
  eg_lo* lo = new eg_lo();
  std::memset(lo, 0, sizeof(*lo));
  lo->mesh = m;
  lo->prec = precision;
  lo->n = m->Np * m->nv;
  lo->nb = m->S * m->nv;
  lo->cpl_sparse = m->sparse_face;
  const size_t es = precision == EG_F64 ? 8 : 4;
  const size_t nd = (size_t)m->E * lo->n * lo->n, nc = eg_lo_coupling_size(lo);
  const size_t nf = (size_t)(m->I + m->B) * m->Nf * 2 * m->nv * m->nv;
  cudaError_t e = cudaMalloc(&lo->diag, es * nd);
  if (e == cudaSuccess && nc) e = cudaMalloc(&lo->cpl, es * nc);
  if (e == cudaSuccess) e = cudaMalloc(&lo->dF, es * nf);
  if (e == cudaSuccess) e = cudaMalloc((void**)&lo->spos, sizeof(int32_t) * m->F * m->Np);
  if (e == cudaSuccess) e = cudaMalloc(&lo->xT, es * m->ndof);
  if (e == cudaSuccess) e = cudaMalloc(&lo->yT, es * m->ndof);
  if (e == cudaSuccess) e = cudaMalloc((void**)&lo->xd, 8 * m->ndof);
  if (e == cudaSuccess) e = cudaMalloc((void**)&lo->yd, 8 * m->ndof);
  if (e != cudaSuccess) {
    lo_free(lo);
    return eg_cuda_fail(e, "eg_lo_create");
  }
  // stencil positions from the device perm table
  std::vector<int32_t> perm((size_t)m->F * m->S), spos((size_t)m->F * m->Np, -1);
  cudaMemcpy(perm.data(), m->perm, sizeof(int32_t) * perm.size(), cudaMemcpyDeviceToHost);
  for (int f = 0; f < m->F; ++f)
    for (int s = 0; s < m->S; ++s) spos[(size_t)f * m->Np + perm[(size_t)f * m->S + s]] = s;
  e = cudaMemcpy(lo->spos, spos.data(), sizeof(int32_t) * spos.size(), cudaMemcpyHostToDevice);
  // coupling block (slot * 2 + side) of every element face, -1 on boundaries
  if (e == cudaSuccess) {
    std::vector<EFace> ef((size_t)m->E * m->F);
    e = cudaMemcpy(ef.data(), m->eface, sizeof(EFace) * ef.size(), cudaMemcpyDeviceToHost);
    std::vector<int32_t> fside(ef.size(), -1);
    for (size_t t = 0; t < ef.size(); ++t)
      if (ef[t].slot >= 0 && ef[t].slot < m->I) fside[t] = ef[t].slot * 2 + ef[t].side;
    if (e == cudaSuccess) e = cudaMalloc((void**)&lo->fside, sizeof(int32_t) * fside.size());
    if (e == cudaSuccess)
      e = cudaMemcpy(lo->fside, fside.data(), sizeof(int32_t) * fside.size(), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    lo_free(lo);
    return eg_cuda_fail(e, "eg_lo_create");
  }
  *out = lo;
  return EG_OK;
}

extern "C" int eg_lo_destroy(eg_lo* lo) {
  if (!lo) return EG_OK;
  cudaStreamSynchronize(lo->mesh->stream);
  lo_free(lo);
  return EG_OK;
}

extern "C" int eg_lo_calc(eg_lo* lo, const double* q, int32_t mem) {
  if (!lo || !q) {
    eg_set_error("eg_lo_calc: NULL argument");
    return EG_ERR_INVALID;
  }
  eg_mesh* m = lo->mesh;
  const double* qd = q;
  if (mem == EG_MEM_HOST) {
    EG_CUDA(cudaMemcpyAsync(lo->xd, q, 8 * m->ndof, cudaMemcpyHostToDevice, m->stream));
    qd = lo->xd;
  }
  int st = eg_jacobian_launch(lo, qd);
  if (st != EG_OK) return st;
  EG_CUDA(cudaGetLastError());
  if (mem == EG_MEM_HOST) EG_CUDA(cudaStreamSynchronize(m->stream));
  lo->valid = true;
  return EG_OK;
}

extern "C" int eg_lo_apply(eg_lo* lo, const double* x, double* y, int32_t mem) {
  if (!lo || !x || !y || !lo->valid) {
    eg_set_error("eg_lo_apply: invalid argument or operator not computed");
    return EG_ERR_INVALID;
  }
  eg_mesh* m = lo->mesh;
  const double* xd = x;
  if (mem == EG_MEM_HOST) {
    EG_CUDA(cudaMemcpyAsync(lo->xd, x, 8 * m->ndof, cudaMemcpyHostToDevice, m->stream));
    xd = lo->xd;
  }
  eg_convert(m, xd, lo->xT, lo->prec, m->ndof, 1.0);
  eg_lo_apply_T(lo, lo->xT, lo->yT);
  double* yd = mem == EG_MEM_HOST ? lo->yd : y;
  eg_convert_back(m, lo->yT, yd, lo->prec, m->ndof);
  EG_CUDA(cudaGetLastError());
  if (mem == EG_MEM_HOST) {
    EG_CUDA(cudaMemcpyAsync(y, yd, 8 * m->ndof, cudaMemcpyDeviceToHost, m->stream));
    EG_CUDA(cudaStreamSynchronize(m->stream));
  }
  return EG_OK;
}

// FP64 interface of the transposed applies: x -> operator precision, apply,
// back to FP64 (host or device arrays per mem)
static int apply_transpose(eg_lo* lo, const void* inv, const double* x, double* y, int32_t mem) {
  eg_mesh* m = lo->mesh;
  const double* xd = x;
  if (mem == EG_MEM_HOST) {
    EG_CUDA(cudaMemcpyAsync(lo->xd, x, 8 * m->ndof, cudaMemcpyHostToDevice, m->stream));
    xd = lo->xd;
  }
  eg_convert(m, xd, lo->xT, lo->prec, m->ndof, 1.0);
  if (lo->prec == EG_F64)
    launch_transpose<double>(lo, (const double*)inv, (const double*)lo->xT, (double*)lo->yT);
  else
    launch_transpose<float>(lo, (const float*)inv, (const float*)lo->xT, (float*)lo->yT);
  double* yd = mem == EG_MEM_HOST ? lo->yd : y;
  eg_convert_back(m, lo->yT, yd, lo->prec, m->ndof);
  EG_CUDA(cudaGetLastError());
  if (mem == EG_MEM_HOST) EG_CUDA(cudaMemcpyAsync(y, yd, 8 * m->ndof, cudaMemcpyDeviceToHost, m->stream));
  EG_CUDA(cudaStreamSynchronize(m->stream));
  return EG_OK;
}

extern "C" int eg_lo_apply_transpose(eg_lo* lo, const double* x, double* y, int32_t mem) {
  if (!lo || !x || !y || !lo->valid) {
    eg_set_error("eg_lo_apply_transpose: invalid argument or operator not computed");
    return EG_ERR_INVALID;
  }
  return apply_transpose(lo, nullptr, x, y, mem);
}

extern "C" int eg_pc_apply_transpose(eg_pc* pc, const double* x, double* y, int32_t mem) {
  if (!pc || !x || !y || !pc->valid) {
    eg_set_error("eg_pc_apply_transpose: invalid argument or preconditioner not computed");
    return EG_ERR_INVALID;
  }
  return apply_transpose(pc->lo, pc->inv, x, y, mem);
}

extern "C" int eg_lo_get_blocks(eg_lo* lo, double* diag, double* coupling) {
  if (!lo || !lo->valid) {
    eg_set_error("eg_lo_get_blocks: operator not computed");
    return EG_ERR_INVALID;
  }
  eg_mesh* m = lo->mesh;
  const size_t nd = (size_t)m->E * lo->n * lo->n, nc = eg_lo_coupling_size(lo);
  EG_CUDA(cudaStreamSynchronize(m->stream));
  auto copy = [&](const void* src, double* dst, size_t n) -> int {
    if (!dst || n == 0) return EG_OK;
    if (lo->prec == EG_F64) {
      EG_CUDA(cudaMemcpy(dst, src, 8 * n, cudaMemcpyDeviceToHost));
    } else {
      std::vector<float> tmp(n);
      EG_CUDA(cudaMemcpy(tmp.data(), src, 4 * n, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < n; ++i) dst[i] = tmp[i];
    }
    return EG_OK;
  };
  int st = copy(lo->diag, diag, nd);
  if (st == EG_OK && coupling && nc) {
    // device coupling blocks are row-major; the ABI exports them column-major
    std::vector<double> tmp(nc);
    st = copy(lo->cpl, tmp.data(), nc);
    const int nb = lo->nb;
    if (st == EG_OK && lo->cpl_sparse) {
      // face-diagonal storage [I][2][S][nv][nv] -> dense blocks
      const int S = m->S, nv = m->nv, Nf = m->Nf;
      std::vector<int32_t> itf((size_t)m->I * 5), nbp((size_t)m->norient * Nf),
          nbi((size_t)m->norient * Nf);
      EG_CUDA(cudaMemcpy(itf.data(), m->ifaces, sizeof(int32_t) * itf.size(), cudaMemcpyDeviceToHost));
      EG_CUDA(cudaMemcpy(nbp.data(), m->nbrperm, sizeof(int32_t) * nbp.size(), cudaMemcpyDeviceToHost));
      EG_CUDA(cudaMemcpy(nbi.data(), m->nbrinv, sizeof(int32_t) * nbi.size(), cudaMemcpyDeviceToHost));
      std::fill(coupling, coupling + (size_t)m->I * 2 * nb * nb, 0.0);
      for (size_t blk = 0; blk < (size_t)m->I * 2; ++blk) {
        const int o = itf[(blk / 2) * 5 + 4], side = (int)(blk & 1);
        for (int s = 0; s < S; ++s) {
          const int sp = side ? nbi[(size_t)o * Nf + s] : nbp[(size_t)o * Nf + s];
          for (int a = 0; a < nv; ++a)
            for (int b = 0; b < nv; ++b)
              coupling[blk * nb * nb + (size_t)(sp * nv + b) * nb + s * nv + a] =
                  tmp[((blk * S + s) * nv + a) * nv + b];
        }
      }
    } else if (st == EG_OK) {
      for (size_t blk = 0; blk < (size_t)m->I * 2; ++blk)
        for (int r = 0; r < nb; ++r)
          for (int c = 0; c < nb; ++c)
            coupling[blk * nb * nb + (size_t)c * nb + r] = tmp[blk * nb * nb + (size_t)r * nb + c];
    }
  }
  return st;
}

extern "C" int eg_pc_create(eg_lo* lo, eg_pc** out) {
  if (!lo || !out) {
    eg_set_error("eg_pc_create: NULL argument");
    return EG_ERR_INVALID;
  }
  eg_pc* pc = new eg_pc();
  pc->lo = lo;
  pc->valid = false;
  const size_t es = lo->prec == EG_F64 ? 8 : 4;
  cudaError_t e = cudaMalloc(&pc->inv, es * (size_t)lo->mesh->E * lo->n * lo->n);
  if (e != cudaSuccess) {
    delete pc;
    return eg_cuda_fail(e, "eg_pc_create");
  }
  *out = pc;
  return EG_OK;
}

extern "C" int eg_pc_destroy(eg_pc* pc) {
  if (!pc) return EG_OK;
  cudaStreamSynchronize(pc->lo->mesh->stream);
  cudaFree(pc->inv);
  delete pc;
  return EG_OK;
}

extern "C" int eg_pc_calc(eg_pc* pc) {
  if (!pc || !pc->lo->valid) {
    eg_set_error("eg_pc_calc: operator not computed");
    return EG_ERR_INVALID;
  }
  const int n = pc->lo->n;
  const size_t smem = (pc->lo->prec == EG_F64 ? 8 : 4) * ((size_t)n * n + 256) + sizeof(int) * (2 + 2 * (size_t)n);
  if (n > 128 || smem > 200 * 1024) {
    eg_set_error("eg_pc_calc: element block of %d unknowns exceeds shared memory", n);
    return EG_ERR_UNSUPPORTED;
  }
  int st = pc->lo->prec == EG_F64 ? pccalc_T<double>(pc) : pccalc_T<float>(pc);
  if (st != EG_OK) return st;
  EG_CUDA(cudaGetLastError());
  pc->valid = true;
  return EG_OK;
}

extern "C" int eg_pc_apply(eg_pc* pc, const double* x, double* y, int32_t mem) {
  if (!pc || !x || !y || !pc->valid) {
    eg_set_error("eg_pc_apply: invalid argument or preconditioner not computed");
    return EG_ERR_INVALID;
  }
  eg_lo* lo = pc->lo;
  eg_mesh* m = lo->mesh;
  const double* xd = x;
  if (mem == EG_MEM_HOST) {
    EG_CUDA(cudaMemcpyAsync(lo->xd, x, 8 * m->ndof, cudaMemcpyHostToDevice, m->stream));
    xd = lo->xd;
  }
  eg_convert(m, xd, lo->xT, lo->prec, m->ndof, 1.0);
  eg_pc_apply_T(pc, lo->xT, lo->yT);
  double* yd = mem == EG_MEM_HOST ? lo->yd : y;
  eg_convert_back(m, lo->yT, yd, lo->prec, m->ndof);
  EG_CUDA(cudaGetLastError());
  EG_CUDA(cudaMemcpyAsync(m->h_status, m->status, sizeof(unsigned int), cudaMemcpyDeviceToHost, m->stream));
  if (mem == EG_MEM_HOST) EG_CUDA(cudaMemcpyAsync(y, yd, 8 * m->ndof, cudaMemcpyDeviceToHost, m->stream));
  EG_CUDA(cudaStreamSynchronize(m->stream));
  EG_CUDA(cudaMemsetAsync(m->status, 0, sizeof(unsigned int), m->stream));
  return eg_check_status(m);
}

static void ls_free(eg_ls* ls) {
  if (!ls) return;
  eg_gmres_release(ls);
  void* bufs[] = {ls->V, ls->w, ls->z, ls->xT, ls->bT, ls->part, ls->h, ls->y, ls->xd, ls->bd,
                  ls->dH, ls->dflags, ls->dscal, ls->cfs, ls->dargs};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (ls->hh) cudaFreeHost(ls->hh);
  if (ls->hargs) cudaFreeHost(ls->hargs);
  if (ls->ev_in) cudaEventDestroy(ls->ev_in);
  delete ls;
}

extern "C" int eg_ls_create(eg_lo* lo, eg_pc* pc, int32_t restart, eg_ls** out) {
  if (!lo || !pc || !out || restart < 1 || restart > 31 || pc->lo != lo) {
    eg_set_error("eg_ls_create: invalid argument (restart must be 1..31, pc built on lo)");
    return EG_ERR_INVALID;
  }
  eg_ls* ls = new eg_ls();
  std::memset(ls, 0, sizeof(*ls));
  ls->lo = lo;
  ls->pc = pc;
  ls->m = restart;
  ls->reltol = 1e-2;     // read_input.jl:493 krylov_reltol
  ls->abstol = 1e-12;
  ls->dtol = 1e5;
  ls->itermax = 1000;    // read_input.jl:496 krylov_itermax
  ls->nblk = EG_GMRES_STREAM_BLOCKS;
  const int64_t N = lo->mesh->ndof;
  const size_t es = lo->prec == EG_F64 ? 8 : 4;
  cudaError_t e = cudaMalloc(&ls->V, es * (size_t)(restart + 1) * N);
  if (e == cudaSuccess) e = cudaMalloc(&ls->w, es * N);
  if (e == cudaSuccess) e = cudaMalloc(&ls->z, es * N);
  if (e == cudaSuccess && lo->mesh->I)
    e = cudaMalloc(&ls->cfs, es * (size_t)lo->mesh->I * 2 * lo->nb);
  if (e == cudaSuccess) e = cudaMalloc(&ls->xT, es * N);
  if (e == cudaSuccess) e = cudaMalloc(&ls->bT, es * N);
  if (e == cudaSuccess) e = cudaMalloc(&ls->part, es * eg_gmres_partials(restart));
  if (e == cudaSuccess) e = cudaMalloc(&ls->h, es * 4 * (restart + 2));
  if (e == cudaSuccess) e = cudaMalloc(&ls->y, es * (restart + 1));
  // Hessenberg, Givens and least-squares state in FP64: H[(m+1) m] | cs[m] |
  // sn[m] | g[m+1] | y[m]
  if (e == cudaSuccess)
    e = cudaMalloc((void**)&ls->dH, sizeof(double) * ((size_t)(restart + 1) * restart + 4 * (restart + 1)));
  // flags[0..7] + two arrival counters of the fused reductions (zeroed)
  if (e == cudaSuccess) e = cudaMalloc((void**)&ls->dflags, sizeof(int) * 16);
  if (e == cudaSuccess) e = cudaMemset(ls->dflags, 0, sizeof(int) * 16);
  if (e == cudaSuccess) e = cudaMalloc((void**)&ls->dscal, sizeof(double) * 8);
  if (e == cudaSuccess) e = cudaMalloc((void**)&ls->xd, 8 * N);
  if (e == cudaSuccess) e = cudaMalloc((void**)&ls->bd, 8 * N);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&ls->hh, 8 * (restart + 16));
  if (e != cudaSuccess) {
    ls_free(ls);
    return eg_cuda_fail(e, "eg_ls_create");
  }
  *out = ls;
  return EG_OK;
}

extern "C" int eg_ls_set_grid(eg_ls* ls, int32_t blocks) {
  if (!ls || blocks < 0) {
    eg_set_error("eg_ls_set_grid: invalid argument");
    return EG_ERR_INVALID;
  }
  ls->coop_grid = blocks;
  return EG_OK;
}

extern "C" int eg_ls_destroy(eg_ls* ls) {
  if (!ls) return EG_OK;
  cudaStreamSynchronize(ls->lo->mesh->stream);
  ls_free(ls);
  return EG_OK;
}

extern "C" int eg_ls_set_tolerances(eg_ls* ls, double reltol, double abstol, double dtol, int32_t itermax) {
  if (!ls) return EG_ERR_INVALID;
  if (reltol >= 0) ls->reltol = reltol;
  if (abstol >= 0) ls->abstol = abstol;
  if (dtol >= 0) ls->dtol = dtol;
  if (itermax >= 0) ls->itermax = itermax;
  return EG_OK;
}

static int ls_solve(eg_ls* ls, const double* b, double* x, int32_t mem, eg_ls_stats* stats, int transpose) {
  if (!ls || !b || !x || !ls->lo->valid || !ls->pc->valid || (mem != EG_MEM_HOST && mem != EG_MEM_DEVICE)) {
    eg_set_error("%s: invalid argument or operator/preconditioner not computed",
                 transpose ? "eg_ls_solve_transpose" : "eg_ls_solve");
    return EG_ERR_INVALID;
  }
  eg_mesh* m = ls->lo->mesh;
  const int64_t N = m->ndof;
  const double* bd = b;
  double* xd = x;
  if (mem == EG_MEM_HOST) {
    EG_CUDA(cudaMemcpyAsync(ls->bd, b, 8 * N, cudaMemcpyHostToDevice, m->stream));
    EG_CUDA(cudaMemcpyAsync(ls->xd, x, 8 * N, cudaMemcpyHostToDevice, m->stream));
    bd = ls->bd;
    xd = ls->xd;
  }
  eg_convert(m, bd, ls->bT, ls->lo->prec, N, 1.0);
  eg_convert(m, xd, ls->xT, ls->lo->prec, N, 1.0);
  int st = eg_gmres_T(ls, ls->bT, ls->xT, stats, transpose);
  if (st != EG_OK) return st;
  eg_convert_back(m, ls->xT, xd, ls->lo->prec, N);
  EG_CUDA(cudaGetLastError());
  if (mem == EG_MEM_HOST) EG_CUDA(cudaMemcpyAsync(x, xd, 8 * N, cudaMemcpyDeviceToHost, m->stream));
  EG_CUDA(cudaStreamSynchronize(m->stream));
  return EG_OK;
}

extern "C" int eg_ls_solve(eg_ls* ls, const double* b, double* x, int32_t mem, eg_ls_stats* stats) {
  return ls_solve(ls, b, x, mem, stats, 0);
}

extern "C" int eg_ls_solve_transpose(eg_ls* ls, const double* b, double* x, int32_t mem,
                                     eg_ls_stats* stats) {
  return ls_solve(ls, b, x, mem, stats, 1);
}

extern "C" int eg_lo_apply_native(eg_lo* lo, const void* x, void* y) {
  if (!lo || !x || !y || !lo->valid) {
    eg_set_error("eg_lo_apply_native: invalid argument or operator not computed");
    return EG_ERR_INVALID;
  }
  int st = eg_lo_apply_T(lo, x, y);
  if (st != EG_OK) return st;
  EG_CUDA(cudaGetLastError());
  return EG_OK;
}

extern "C" int eg_pc_apply_native(eg_pc* pc, const void* x, void* y) {
  if (!pc || !x || !y || !pc->valid) {
    eg_set_error("eg_pc_apply_native: invalid argument or preconditioner not computed");
    return EG_ERR_INVALID;
  }
  int st = eg_pc_apply_T(pc, x, y);
  if (st != EG_OK) return st;
  EG_CUDA(cudaGetLastError());
  return EG_OK;
}
