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
#include <vector>

#include "eg_internal.h"
#include "eg_kernels.cuh"
#include "eg_linalg.h"

namespace {

// ---------------------------------------------------------------- SpMV
// y[e][r] = sum_c diag[e][c][r] x[e][c] + face couplings of row r.
// One CTA per `epb` elements, one thread per row; x of the CTA's elements in
// shared memory; coupling operands read from the neighbours (L2).
template <int DIM, typename T>
__global__ void k_spmv(DevMesh md, const T* __restrict__ diag, const T* __restrict__ cpl,
                       const int* __restrict__ spos, const T* __restrict__ x, T* __restrict__ y,
                       int epb) {
  constexpr int NV = DIM + 2;
  constexpr int F = DIM + 1;
  extern __shared__ unsigned char smraw[];
  T* sx = reinterpret_cast<T*>(smraw);
  const int Np = md.Np, S = md.S, Nf = md.Nf;
  (void)Nf;
  const int n = Np * NV, nb = S * NV;
  const int e0 = blockIdx.x * epb;
  const int nloc = min(epb, md.E - e0);
  for (int t = threadIdx.x; t < nloc * n; t += blockDim.x) sx[t] = x[(size_t)e0 * n + t];
  __syncthreads();
  const int le = threadIdx.x / n, r = threadIdx.x - le * n;
  if (le >= nloc) return;
  const int e = e0 + le;
  const T* D = diag + (size_t)e * n * n;
  const T* xe = sx + (size_t)le * n;
  T acc = T(0);
  for (int c = 0; c < n; ++c) acc += D[(size_t)c * n + r] * xe[c];
  const int j = r / NV, a = r - j * NV;
#pragma unroll
  for (int f = 0; f < F; ++f) {
    const int s = spos[f * Np + j];
    if (s < 0) continue;
    const EFace ef = md.eface[(size_t)e * F + f];
    if (ef.slot >= md.I) continue;  // boundary face: no coupling
    const int* itf = md.ifaces + 5 * ef.slot;
    const int en = ef.side ? itf[0] : itf[1];
    const int fn = ef.side ? itf[2] : itf[3];
    const T* C = cpl + ((size_t)ef.slot * 2 + ef.side) * nb * nb;
    const T* xn = x + (size_t)en * n;
    for (int sp = 0; sp < S; ++sp) {
      const int mnode = md.perm[fn * S + sp];
#pragma unroll
      for (int b = 0; b < NV; ++b)
        acc += C[(size_t)(sp * NV + b) * nb + s * NV + a] * xn[mnode * NV + b];
    }
  }
  y[(size_t)e * n + r] = acc;
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
template <typename T>
__global__ void k_block_apply(const T* __restrict__ inv, const T* __restrict__ x, T* __restrict__ y,
                              int E, int n, int epb) {
  extern __shared__ unsigned char smraw[];
  T* sx = reinterpret_cast<T*>(smraw);
  const int e0 = blockIdx.x * epb;
  const int nloc = min(epb, E - e0);
  for (int t = threadIdx.x; t < nloc * n; t += blockDim.x) sx[t] = x[(size_t)e0 * n + t];
  __syncthreads();
  const int le = threadIdx.x / n, r = threadIdx.x - le * n;
  if (le >= nloc) return;
  const T* A = inv + (size_t)(e0 + le) * n * n;
  const T* xe = sx + (size_t)le * n;
  T acc = T(0);
  for (int c = 0; c < n; ++c) acc += A[(size_t)c * n + r] * xe[c];
  y[(size_t)(e0 + le) * n + r] = acc;
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

template <typename T>
int spmv_T(eg_lo* lo, const T* x, T* y) {
  eg_mesh* m = lo->mesh;
  DevMesh md = dev_mesh(m);
  const int n = lo->n;
  int epb = 256 / n;
  if (epb < 1) epb = 1;
  const int blocks = (m->E + epb - 1) / epb;
  const size_t smem = sizeof(T) * (size_t)epb * n;
  eg_phase_begin(m, EG_PHASE_OTHER);
  if (m->dim == 2)
    k_spmv<2, T><<<blocks, epb * n, smem, m->stream>>>(md, (const T*)lo->diag, (const T*)lo->cpl,
                                                      lo->spos, x, y, epb);
  else
    k_spmv<3, T><<<blocks, epb * n, smem, m->stream>>>(md, (const T*)lo->diag, (const T*)lo->cpl,
                                                      lo->spos, x, y, epb);
  eg_phase_end(m, EG_PHASE_OTHER, 1);
  return EG_OK;
}

template <typename T>
int pcapply_T(eg_pc* pc, const T* x, T* y) {
  eg_lo* lo = pc->lo;
  eg_mesh* m = lo->mesh;
  const int n = lo->n;
  int epb = 256 / n;
  if (epb < 1) epb = 1;
  const int blocks = (m->E + epb - 1) / epb;
  eg_phase_begin(m, EG_PHASE_OTHER);
  k_block_apply<T><<<blocks, epb * n, sizeof(T) * (size_t)epb * n, m->stream>>>(
      (const T*)pc->inv, x, y, m->E, n, epb);
  eg_phase_end(m, EG_PHASE_OTHER, 1);
  return EG_OK;
}

template <typename T>
int pccalc_T(eg_pc* pc) {
  eg_lo* lo = pc->lo;
  eg_mesh* m = lo->mesh;
  const int n = lo->n;
  const size_t smem = sizeof(T) * (size_t)n * n + sizeof(int) * n;
  cudaFuncSetAttribute(k_block_inverse<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  eg_phase_begin(m, EG_PHASE_OTHER);
  k_block_inverse<T><<<m->E, 256, smem, m->stream>>>((const T*)lo->diag, (T*)pc->inv, n, m->status);
  eg_phase_end(m, EG_PHASE_OTHER, 1);
  return EG_OK;
}

// ---------------------------------------------------------------- GMRES
template <typename T>
int gmres_T(eg_ls* ls, const T* b, T* x, eg_ls_stats* st) {
  eg_lo* lo = ls->lo;
  eg_mesh* m = lo->mesh;
  const int64_t N = m->ndof;
  const int mm = ls->m;
  const int nblk = ls->nblk;
  const int stride = mm + 2;
  T* V = (T*)ls->V;
  T* w = (T*)ls->w;
  T* z = (T*)ls->z;
  T* part = (T*)ls->part;
  T* h = (T*)ls->h;
  T* yv = (T*)ls->y;
  const int g = grid_for(N);
  std::vector<double> H((size_t)(mm + 1) * mm, 0.0), cs(mm), sn(mm), gvec(mm + 1), yh(mm);
  auto norm_into = [&](const T* v, T* out) {
    k_multidot<T, 256><<<nblk, 256, 0, m->stream>>>(v, v, 1, N, part, stride);
    k_reduce_parts<T, 256><<<1, 256, 0, m->stream>>>(part, nblk, 1, stride, out, 2);
    m->launches += 2;
  };
  auto fetch = [&](int cnt) -> int {
    T tmp[64];
    EG_CUDA(cudaMemcpyAsync(tmp, h, sizeof(T) * cnt, cudaMemcpyDeviceToHost, m->stream));
    EG_CUDA(cudaStreamSynchronize(m->stream));
    for (int k = 0; k < cnt; ++k) ls->hh[k] = double(tmp[k]);
    return EG_OK;
  };
  // r = b - A x  (into V[0])
  int its = 0, restarts = 0;
  double beta = 0.0, res0 = -1.0, bnorm = 0.0;
  norm_into(b, h);
  if (fetch(1) != EG_OK) return EG_ERR_CUDA;
  bnorm = ls->hh[0];
  bool converged = false;
  double resid = 0.0;
  while (true) {
    spmv_T<T>(lo, x, w);
    k_axpby<T><<<g, 256, 0, m->stream>>>(T(1), b, T(-1), w, N);  // w = b - A x
    m->launches += 1;
    norm_into(w, h);
    if (fetch(1) != EG_OK) return EG_ERR_CUDA;
    beta = ls->hh[0];
    if (res0 < 0) res0 = beta;
    resid = beta;
    const double tol = fmax(ls->reltol * bnorm, ls->abstol);
    if (!(beta > tol) || its >= ls->itermax) {
      converged = !(beta > tol);
      break;
    }
    if (!std::isfinite(beta)) {
      eg_set_error("GMRES: non-finite residual");
      return EG_ERR_NONFINITE;
    }
    k_scale_by_inv<T><<<g, 256, 0, m->stream>>>(w, h, N, V);  // v0 = r / beta
    m->launches += 1;
    std::fill(gvec.begin(), gvec.end(), 0.0);
    gvec[0] = beta;
    int j = 0;
    for (; j < mm && its < ls->itermax; ++j) {
      ++its;
      T* vj = V + (size_t)j * N;
      pcapply_T<T>(ls->pc, vj, z);
      spmv_T<T>(lo, z, w);
      // classical Gram-Schmidt, twice: pass-1 coefficients in h[0..j],
      // pass-2 coefficients in h2[0..j] (h2 = h + mm + 2), ||w|| in h[j+1]
      T* h2 = h + (mm + 2);
      for (int pass = 0; pass < 2; ++pass) {
        T* hp = pass ? h2 : h;
        k_multidot<T, 256><<<nblk, 256, 0, m->stream>>>(V, w, j + 1, N, part, stride);
        k_reduce_parts<T, 256><<<1, 256, 0, m->stream>>>(part, nblk, j + 1, stride, hp, 0);
        k_sub_Vh<T><<<g, 256, 0, m->stream>>>(V, hp, j + 1, N, w);
        m->launches += 3;
      }
      norm_into(w, h + j + 1);
      k_scale_by_inv<T><<<g, 256, 0, m->stream>>>(w, h + j + 1, N, V + (size_t)(j + 1) * N);
      m->launches += 1;
      // host: H[0..j, j] = pass1 + pass2, H[j+1, j] = ||w||
      T tmp[2 * 64];
      EG_CUDA(cudaMemcpyAsync(tmp, h, sizeof(T) * 2 * (mm + 2), cudaMemcpyDeviceToHost, m->stream));
      EG_CUDA(cudaStreamSynchronize(m->stream));
      double* Hc = &H[(size_t)j * (mm + 1)];
      for (int k = 0; k <= j; ++k) Hc[k] = double(tmp[k]) + double(tmp[mm + 2 + k]);
      Hc[j + 1] = double(tmp[j + 1]);
      // Givens rotations
      for (int k = 0; k < j; ++k) {
        const double t0 = cs[k] * Hc[k] + sn[k] * Hc[k + 1];
        Hc[k + 1] = -sn[k] * Hc[k] + cs[k] * Hc[k + 1];
        Hc[k] = t0;
      }
      const double den = std::hypot(Hc[j], Hc[j + 1]);
      if (den == 0.0) {
        eg_set_error("GMRES: breakdown (zero Hessenberg column)");
        return EG_ERR_KRYLOV;
      }
      cs[j] = Hc[j] / den;
      sn[j] = Hc[j + 1] / den;
      Hc[j] = den;
      Hc[j + 1] = 0.0;
      gvec[j + 1] = -sn[j] * gvec[j];
      gvec[j] = cs[j] * gvec[j];
      resid = std::fabs(gvec[j + 1]);
      if (!std::isfinite(resid)) {
        eg_set_error("GMRES: non-finite residual estimate");
        return EG_ERR_NONFINITE;
      }
      if (resid <= tol || tmp[j + 1] == T(0)) {
        ++j;
        break;
      }
    }
    // y = H^-1 g (upper triangular j x j), x += M^-1 V y
    for (int k = j - 1; k >= 0; --k) {
      double s = gvec[k];
      for (int c = k + 1; c < j; ++c) s -= H[(size_t)c * (mm + 1) + k] * yh[c];
      yh[k] = s / H[(size_t)k * (mm + 1) + k];
    }
    T ytmp[128];
    for (int k = 0; k < j; ++k) ytmp[k] = T(yh[k]);
    EG_CUDA(cudaMemcpyAsync(yv, ytmp, sizeof(T) * j, cudaMemcpyHostToDevice, m->stream));
    k_Vy<T><<<g, 256, 0, m->stream>>>(V, yv, j, N, w);
    m->launches += 1;
    pcapply_T<T>(ls->pc, w, z);
    k_axpby<T><<<g, 256, 0, m->stream>>>(T(1), z, T(1), x, N);
    m->launches += 1;
    EG_CUDA(cudaStreamSynchronize(m->stream));
    ++restarts;
    if (resid <= tol) {
      // recompute the true residual on the next pass of the loop
    }
  }
  if (st) {
    st->iters = its;
    st->restarts = restarts;
    st->converged = converged ? 1 : 0;
    st->res0 = res0;
    st->res_final = resid;
  }
  return EG_OK;
}

}  // namespace

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

int eg_lo_apply_T(eg_lo* lo, const void* x, void* y) {
  return lo->prec == EG_F64 ? spmv_T<double>(lo, (const double*)x, (double*)y)
                            : spmv_T<float>(lo, (const float*)x, (float*)y);
}

int eg_pc_apply_T(eg_pc* pc, const void* x, void* y) {
  return pc->lo->prec == EG_F64 ? pcapply_T<double>(pc, (const double*)x, (double*)y)
                                : pcapply_T<float>(pc, (const float*)x, (float*)y);
}

int eg_gmres_T(eg_ls* ls, const void* bT, void* xT, eg_ls_stats* st) {
  return ls->lo->prec == EG_F64 ? gmres_T<double>(ls, (const double*)bT, (double*)xT, st)
                                : gmres_T<float>(ls, (const float*)bT, (float*)xT, st);
}

static void lo_free(eg_lo* lo) {
  if (!lo) return;
  void* bufs[] = {lo->diag, lo->cpl, lo->dF, lo->spos, lo->xT, lo->yT, lo->xd, lo->yd};
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
  const size_t es = precision == EG_F64 ? 8 : 4;
  const size_t nd = (size_t)m->E * lo->n * lo->n, nc = (size_t)m->I * 2 * lo->nb * lo->nb;
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

extern "C" int eg_lo_get_blocks(eg_lo* lo, double* diag, double* coupling) {
  if (!lo || !lo->valid) {
    eg_set_error("eg_lo_get_blocks: operator not computed");
    return EG_ERR_INVALID;
  }
  eg_mesh* m = lo->mesh;
  const size_t nd = (size_t)m->E * lo->n * lo->n, nc = (size_t)m->I * 2 * lo->nb * lo->nb;
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
  if (st == EG_OK) st = copy(lo->cpl, coupling, nc);
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
  const size_t smem = (pc->lo->prec == EG_F64 ? 8 : 4) * (size_t)n * n + sizeof(int) * n;
  if (smem > 200 * 1024) {
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
  void* bufs[] = {ls->V, ls->w, ls->z, ls->xT, ls->bT, ls->part, ls->h, ls->y, ls->xd, ls->bd};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (ls->hh) cudaFreeHost(ls->hh);
  delete ls;
}

extern "C" int eg_ls_create(eg_lo* lo, eg_pc* pc, int32_t restart, eg_ls** out) {
  if (!lo || !pc || !out || restart < 1 || restart > 60 || pc->lo != lo) {
    eg_set_error("eg_ls_create: invalid argument (restart must be 1..60, pc built on lo)");
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
  ls->nblk = 304;
  const int64_t N = lo->mesh->ndof;
  const size_t es = lo->prec == EG_F64 ? 8 : 4;
  cudaError_t e = cudaMalloc(&ls->V, es * (size_t)(restart + 1) * N);
  if (e == cudaSuccess) e = cudaMalloc(&ls->w, es * N);
  if (e == cudaSuccess) e = cudaMalloc(&ls->z, es * N);
  if (e == cudaSuccess) e = cudaMalloc(&ls->xT, es * N);
  if (e == cudaSuccess) e = cudaMalloc(&ls->bT, es * N);
  if (e == cudaSuccess) e = cudaMalloc(&ls->part, es * (size_t)ls->nblk * (restart + 2));
  if (e == cudaSuccess) e = cudaMalloc(&ls->h, es * 2 * (restart + 2));
  if (e == cudaSuccess) e = cudaMalloc(&ls->y, es * (restart + 1));
  if (e == cudaSuccess) e = cudaMalloc((void**)&ls->xd, 8 * N);
  if (e == cudaSuccess) e = cudaMalloc((void**)&ls->bd, 8 * N);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&ls->hh, 8 * (restart + 2));
  if (e != cudaSuccess) {
    ls_free(ls);
    return eg_cuda_fail(e, "eg_ls_create");
  }
  *out = ls;
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

extern "C" int eg_ls_solve(eg_ls* ls, const double* b, double* x, int32_t mem, eg_ls_stats* stats) {
  if (!ls || !b || !x || !ls->lo->valid || !ls->pc->valid) {
    eg_set_error("eg_ls_solve: invalid argument or operator/preconditioner not computed");
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
  int st = eg_gmres_T(ls, ls->bT, ls->xT, stats);
  if (st != EG_OK) return st;
  eg_convert_back(m, ls->xT, xd, ls->lo->prec, N);
  EG_CUDA(cudaGetLastError());
  if (mem == EG_MEM_HOST) EG_CUDA(cudaMemcpyAsync(x, xd, 8 * N, cudaMemcpyDeviceToHost, m->stream));
  EG_CUDA(cudaStreamSynchronize(m->stream));
  return EG_OK;
}
