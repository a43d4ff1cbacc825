// eg_gmres.cu -- right-preconditioned restarted GMRES driven from the device.
//
// Reference: linearSolve -> PETSc KSPSolve with GMRES(30), right
// preconditioning (src/linearsolvers/ls_standard.jl:321-371,
// src/input/read_input.jl:559-569).  The algorithm is Saad's GMRES(m) with
// classical Gram-Schmidt and a second pass when the Daniel-Gragg-Kaufman-
// Stewart test asks for it (as stable as the reference's modified
// Gram-Schmidt, but each pass is one batched multi-dot kernel).
//
// GB300 design: the Hessenberg column, Givens rotations, convergence test and
// the small triangular solve all run on the device (FP64, one thread), so a
// restart cycle needs no host round trip.  A device flag `done` makes every
// remaining kernel of the cycle return immediately once the residual estimate
// meets the tolerance.  One cycle (m iterations, the update x += M^-1 V y,
// the true residual b - A x and the re-initialisation) is captured once as a
// CUDA graph and replayed; the host reads 2 ints and 2 doubles per cycle.
#include <cmath>
#include <cstring>

#include "eg_internal.h"
#include "eg_kernels.cuh"
#include "eg_linalg.h"

namespace {


// a cycle kernel runs unless the cycle is done, or its optional condition
// flag (need >= 0) is zero
__device__ __forceinline__ bool gm_skip(const int* flags, int need) {
  return flags && (flags[F_DONE] || (need >= 0 && !flags[need]));
}

// per-block partial sums of V[k] . w for k < cnt (skips when *done)
template <typename T, int NT>
__global__ void k_gm_multidot(const T* __restrict__ V, const T* __restrict__ w, int cnt, int64_t N,
                              T* __restrict__ part, int stride, const int* __restrict__ flags,
                              int need) {
  if (gm_skip(flags, need)) return;
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

// out[k] = sum_b part[b][k] (sqrt when take_sqrt)
template <typename T, int NT>
__global__ void k_gm_reduce(const T* __restrict__ part, int nblk, int cnt, int stride,
                            T* __restrict__ out, int take_sqrt, const int* __restrict__ flags,
                            int need) {
  if (gm_skip(flags, need)) return;
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
    if (threadIdx.x == 0) out[k] = take_sqrt ? sqrt(sh[0]) : sh[0];
    __syncthreads();
  }
}

// w -= sum_{k<cnt} V[k] h[k]
template <typename T>
__global__ void k_gm_sub(const T* __restrict__ V, const T* __restrict__ h, int cnt, int64_t N,
                         T* __restrict__ w, const int* __restrict__ flags, int need) {
  if (gm_skip(flags, need)) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    T acc = w[i];
    for (int k = 0; k < cnt; ++k) acc -= V[(size_t)k * N + i] * h[k];
    w[i] = acc;
  }
}

// dst = src / nrm[0] (zero when nrm[0] == 0); skipped when *done unless force
template <typename T>
__global__ void k_gm_scale(const T* __restrict__ src, const T* __restrict__ nrm, int64_t N,
                           T* __restrict__ dst, const int* __restrict__ flags, int force) {
  if (!force && flags[F_DONE]) return;
  const T s = nrm[0];
  const T inv = (s > T(0)) ? T(1) / s : T(0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i] * inv;
}

// w = b - w
template <typename T>
__global__ void k_gm_bminus(const T* __restrict__ b, T* __restrict__ w, int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    w[i] = b[i] - w[i];
}

// x += z
template <typename T>
__global__ void k_gm_add(const T* __restrict__ z, T* __restrict__ x, int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += z[i];
}

// w = sum_{k < jdone} V[k] y[k]
template <typename T>
__global__ void k_gm_Vy(const T* __restrict__ V, const double* __restrict__ y, int64_t N,
                        T* __restrict__ w, const int* __restrict__ flags) {
  const int cnt = flags[F_JDONE];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    T acc = T(0);
    for (int k = 0; k < cnt; ++k) acc += V[(size_t)k * N + i] * T(y[k]);
    w[i] = acc;
  }
}

// start of a cycle: beta = |b - A x|, g = (beta, 0, ...), decide done
template <typename T>
__global__ void k_gm_init(const T* __restrict__ beta, const T* __restrict__ bnorm, int first, int m,
                          double* __restrict__ dH, int* __restrict__ flags, double* __restrict__ scal) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double* g = dH + (size_t)(m + 1) * m + 2 * m;
  if (first) {
    scal[S_BNORM] = double(bnorm[0]);
    scal[S_TOL] = fmax(scal[S_RELTOL] * scal[S_BNORM], scal[S_ABSTOL]);
    flags[F_ITS] = 0;
  }
  const double b = double(beta[0]);
  scal[S_BETA] = b;
  scal[S_RESID] = b;
  for (int k = 0; k <= m; ++k) g[k] = 0.0;
  g[0] = b;
  const bool conv = !(b > scal[S_TOL]);
  flags[F_CONV] = conv ? 1 : 0;
  flags[F_DONE] = (conv || flags[F_ITS] >= flags[F_ITERMAX] || !isfinite(b)) ? 1 : 0;
  flags[F_JDONE] = 0;
}

// Hessenberg column j from the two CGS passes and |w|; Givens update
template <typename T>
__global__ void k_gm_givens(int j, int m, const T* __restrict__ h1, const T* __restrict__ h2,
                            const T* __restrict__ hn, double* __restrict__ dH,
                            int* __restrict__ flags, double* __restrict__ scal) {
  if (threadIdx.x != 0 || blockIdx.x != 0 || flags[F_DONE]) return;
  double* H = dH;
  double* cs = dH + (size_t)(m + 1) * m;
  double* sn = cs + m;
  double* g = sn + m;
  double* Hc = H + (size_t)j * (m + 1);
  for (int k = 0; k <= j; ++k) Hc[k] = double(h1[k]) + double(h2[k]);
  Hc[j + 1] = double(hn[0]);
  for (int k = 0; k < j; ++k) {
    const double t0 = cs[k] * Hc[k] + sn[k] * Hc[k + 1];
    Hc[k + 1] = -sn[k] * Hc[k] + cs[k] * Hc[k + 1];
    Hc[k] = t0;
  }
  const double den = hypot(Hc[j], Hc[j + 1]);
  flags[F_ITS] += 1;
  if (!(den > 0.0) || !isfinite(den)) {  // breakdown: stop with the current basis
    flags[F_DONE] = 1;
    flags[F_JDONE] = j;
    return;
  }
  cs[j] = Hc[j] / den;
  sn[j] = Hc[j + 1] / den;
  Hc[j] = den;
  Hc[j + 1] = 0.0;
  g[j + 1] = -sn[j] * g[j];
  g[j] = cs[j] * g[j];
  const double resid = fabs(g[j + 1]);
  scal[S_RESID] = resid;
  flags[F_JDONE] = j + 1;
  if (resid <= scal[S_TOL] || double(hn[0]) == 0.0 || flags[F_ITS] >= flags[F_ITERMAX])
    flags[F_DONE] = 1;
}

// selective re-orthogonalisation (Daniel-Gragg-Kaufman-Stewart test): after
// one classical Gram-Schmidt pass, |w|^2 before the pass is sum h1^2 + |w|^2
// after it; a second pass is needed only when |w| dropped below 1/sqrt(2) of
// that.  Without one, the second-pass coefficients h2 are zero.
template <typename T>
__global__ void k_gm_reorth_check(int j, const T* __restrict__ h1, const T* __restrict__ hn,
                                  T* __restrict__ h2, int* __restrict__ flags) {
  if (threadIdx.x != 0 || blockIdx.x != 0 || flags[F_DONE]) return;
  double before = double(hn[0]) * double(hn[0]);
  for (int k = 0; k <= j; ++k) before += double(h1[k]) * double(h1[k]);
  const int need = double(hn[0]) * double(hn[0]) < 0.5 * before;
  flags[F_REORTH] = need;
  flags[F_NREORTH] += need;
  if (!need)
    for (int k = 0; k <= j; ++k) h2[k] = T(0);
}

// y = H^-1 g on the leading jdone x jdone block (H staged in shared memory)
__global__ void k_gm_lsq(int m, double* __restrict__ dH, const int* __restrict__ flags) {
  __shared__ double sH[32 * 33];
  __shared__ double sg[33];
  const int n = flags[F_JDONE];
  const double* H = dH;
  const double* g = dH + (size_t)(m + 1) * m + 2 * m;
  double* y = dH + (size_t)(m + 1) * m + 3 * m + 1;
  for (int t = threadIdx.x; t < n * (m + 1); t += blockDim.x) sH[t] = H[t];
  for (int t = threadIdx.x; t < n; t += blockDim.x) sg[t] = g[t];
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int k = n - 1; k >= 0; --k) {
    double s = sg[k];
    for (int c = k + 1; c < n; ++c) s -= sH[(size_t)c * (m + 1) + k] * sg[c];
    sg[k] = s / sH[(size_t)k * (m + 1) + k];
  }
  for (int k = 0; k < n; ++k) y[k] = sg[k];
}

// ---- fused Arnoldi kernels --------------------------------------------------
// The basis has at most 32 vectors (restart <= 31).  Partial sums go to
// part[block][k]; the last block to finish (threadfence + counter) reduces
// them in block order, so the results are deterministic and no separate
// reduction launch is needed.

// Givens update of Hessenberg column j (h1 + h2 when a second pass ran)
template <typename T>
__device__ void gm_givens_core(int j, int m, const T* h1, const T* h2, double hn, double* dH,
                               int* flags, double* scal) {
  double* H = dH;
  double* cs = dH + (size_t)(m + 1) * m;
  double* sn = cs + m;
  double* g = sn + m;
  double* Hc = H + (size_t)j * (m + 1);
  for (int k = 0; k <= j; ++k) Hc[k] = double(h1[k]) + (h2 ? double(h2[k]) : 0.0);
  Hc[j] += 1.0;  // column j of H_K + I: the Arnoldi vectors come from K = C D^-1
  Hc[j + 1] = hn;
  for (int k = 0; k < j; ++k) {
    const double t0 = cs[k] * Hc[k] + sn[k] * Hc[k + 1];
    Hc[k + 1] = -sn[k] * Hc[k] + cs[k] * Hc[k + 1];
    Hc[k] = t0;
  }
  const double den = hypot(Hc[j], Hc[j + 1]);
  flags[F_ITS] += 1;
  if (!(den > 0.0) || !isfinite(den)) {  // breakdown: stop with the current basis
    flags[F_DONE] = 1;
    flags[F_JDONE] = j;
    return;
  }
  cs[j] = Hc[j] / den;
  sn[j] = Hc[j + 1] / den;
  Hc[j] = den;
  Hc[j + 1] = 0.0;
  g[j + 1] = -sn[j] * g[j];
  g[j] = cs[j] * g[j];
  const double resid = fabs(g[j + 1]);
  scal[S_RESID] = resid;
  flags[F_JDONE] = j + 1;
  if (resid <= scal[S_TOL] || hn == 0.0 || flags[F_ITS] >= flags[F_ITERMAX]) flags[F_DONE] = 1;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// true in every thread of the last block to arrive
__device__ __forceinline__ bool last_block(unsigned int* counter) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  return s_last;
}

// vector load of W consecutive values (16-byte aligned when W > 1)
template <typename T, int W> struct VecOf;
template <> struct VecOf<float, 4> { using type = float4; };
template <> struct VecOf<double, 2> { using type = double2; };
template <typename T, int W>
__device__ __forceinline__ void vload(const T* p, T (&v)[W]) {
  if constexpr (W == 1) {
    v[0] = p[0];
  } else {
    const auto t = *reinterpret_cast<const typename VecOf<T, W>::type*>(p);
    if constexpr (W == 4) { v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w; }
    else { v[0] = t.x; v[1] = t.y; }
  }
}
template <typename T, int W>
__device__ __forceinline__ void vstore(T* p, const T (&v)[W]) {
  if constexpr (W == 1) {
    p[0] = v[0];
  } else if constexpr (W == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  }
}

// h[k] = V[k] . w for k < cnt (and ww = w . w when with_ww).  Each thread
// owns groups of W consecutive rows and accumulates every coefficient in
// registers (W-wide vector loads of all basis vectors in flight at once);
// warp shuffles and shared memory combine the block's partials.
template <typename T, int W>
__global__ void __launch_bounds__(256) k_gm_dots2(const T* __restrict__ V, const T* __restrict__ w,
                                                  int cnt, int with_ww, int64_t N, T* __restrict__ part,
                                                  int stride, const int* __restrict__ flags, int need,
                                                  unsigned int* __restrict__ counter, T* __restrict__ h,
                                                  T* __restrict__ ww) {
  if (gm_skip(flags, need)) return;
  __shared__ T sred[8][33];
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  const int64_t ng = N / W;                         // row groups (N % W == 0)
  const int64_t chunk = (ng + gridDim.x - 1) / gridDim.x;
  const int64_t lo = blockIdx.x * chunk;
  const int64_t hi = min(ng, lo + chunk);
  T acc[33];
#pragma unroll
  for (int k = 0; k < 33; ++k) acc[k] = T(0);
  for (int64_t g = lo + threadIdx.x; g < hi; g += 256) {
    T wv[W];
    vload<T, W>(w + g * W, wv);
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      if (k < cnt) {
        T vv[W];
        vload<T, W>(V + (size_t)k * N + g * W, vv);
#pragma unroll
        for (int q = 0; q < W; ++q) acc[k] += vv[q] * wv[q];
      }
    }
#pragma unroll
    for (int q = 0; q < W; ++q) acc[32] += wv[q] * wv[q];
  }
#pragma unroll
  for (int k = 0; k < 33; ++k) {
    if (k < cnt || (k == 32 && with_ww)) {
      const T v = warp_sum(acc[k]);
      if (lane == 0) sred[wq][k] = v;
    }
  }
  __syncthreads();
  T* pb = part + (size_t)blockIdx.x * stride;
  for (int k = threadIdx.x; k < 33; k += 256) {
    if (k < cnt || (k == 32 && with_ww)) {
      T v = T(0);
#pragma unroll
      for (int q = 0; q < 8; ++q) v += sred[q][k];
      pb[k == 32 ? cnt : k] = v;
    }
  }
  if (!last_block(counter)) return;
  const int tot = cnt + (with_ww ? 1 : 0);
  for (int k = wq; k < tot; k += 8) {
    T v = T(0);
    for (int b = lane; b < (int)gridDim.x; b += 32) v += part[(size_t)b * stride + k];
    v = warp_sum(v);
    if (lane == 0) {
      if (k < cnt) h[k] = v;
      else ww[0] = v;
    }
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// w -= sum_k V[k] h[k]; then |w| and, in the last block, the DGKS test
// (pass 1) and/or the Givens update of column j
template <typename T, int W>
__global__ void __launch_bounds__(256) k_gm_sub2(const T* __restrict__ V, const T* __restrict__ h,
                                                 int cnt, int64_t N, T* __restrict__ w,
                                                 T* __restrict__ part, int stride, const int* __restrict__ flagsc,
                                                 int need, unsigned int* __restrict__ counter, int pass, int j,
                                                 int m, const T* __restrict__ h1, const T* __restrict__ h2,
                                                 const T* __restrict__ ww, T* __restrict__ hn,
                                                 double* __restrict__ dH, int* __restrict__ flags,
                                                 double* __restrict__ scal) {
  if (gm_skip(flagsc, need)) return;
  __shared__ T sh[32];
  __shared__ T sw[8];
  if (threadIdx.x < cnt) sh[threadIdx.x] = h[threadIdx.x];
  __syncthreads();
  const int64_t ng = N / W;
  const int64_t chunk = (ng + gridDim.x - 1) / gridDim.x;
  const int64_t lo = blockIdx.x * chunk;
  const int64_t hi = min(ng, lo + chunk);
  T acc = T(0);
  for (int64_t g = lo + threadIdx.x; g < hi; g += 256) {
    T a[W];
    vload<T, W>(w + g * W, a);
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      if (k < cnt) {
        T vv[W];
        vload<T, W>(V + (size_t)k * N + g * W, vv);
        const T hk = sh[k];
#pragma unroll
        for (int q = 0; q < W; ++q) a[q] -= vv[q] * hk;
      }
    }
    vstore<T, W>(w + g * W, a);
#pragma unroll
    for (int q = 0; q < W; ++q) acc += a[q] * a[q];
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    T t = T(0);
    for (int q = 0; q < 8; ++q) t += sw[q];
    part[(size_t)blockIdx.x * stride] = t;
  }
  if (!last_block(counter)) return;
  if (threadIdx.x < 32) {
    T v = T(0);
    for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) v += part[(size_t)b * stride];
    v = warp_sum(v);
    if (threadIdx.x == 0) {
      *counter = 0u;
      const double n2 = double(v);
      hn[0] = T(sqrt(n2));
      if (pass == 1) {
        const int need2 = n2 < 0.5 * double(ww[0]);
        flags[F_REORTH] = need2;
        flags[F_NREORTH] += need2;
        if (!need2) gm_givens_core<T>(j, m, h1, nullptr, sqrt(n2), dH, flags, scal);
      } else {
        gm_givens_core<T>(j, m, h1, h2, sqrt(n2), dH, flags, scal);
      }
    }
  }
}

int gridN(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b > 152 * 8 ? 152 * 8 : (b < 1 ? 1 : b));
}

// |v| into out[0] (two launches)
// |v| into out[0] (two launches)
template <typename T>
void norm_T(eg_ls* ls, const T* v, T* out, const int* flags, int need = -1) {
  eg_mesh* m = ls->lo->mesh;
  const int stride = ls->m + 2;
  k_gm_multidot<T, 256><<<ls->nblk, 256, 0, m->stream>>>(v, v, 1, m->ndof, (T*)ls->part, stride, flags, need);
  k_gm_reduce<T, 256><<<1, 256, 0, m->stream>>>((const T*)ls->part, ls->nblk, 1, stride, out, 1, flags, need);
}

// the launches of the initial residual + cycle set-up (the k_gm_* kernels
// take flags == nullptr to run unconditionally)
template <typename T>
void enqueue_init(eg_ls* ls, int first) {
  eg_mesh* m = ls->lo->mesh;
  const int64_t N = m->ndof;
  T* V = (T*)ls->V;
  T* w = (T*)ls->w;
  T* h = (T*)ls->h;  // h: [0..m+1] pass 1 | [m+2 ..] pass 2 | [2(m+2)] |w| | [2(m+2)+1] beta | +2 bnorm
  T* beta = h + 2 * (ls->m + 2) + 1;
  T* bnorm = h + 2 * (ls->m + 2) + 2;
  const T* b = (const T*)ls->bT;
  const T* x = (const T*)ls->xT;
  if (first) norm_T<T>(ls, b, bnorm, nullptr);
  if (ls->trans)
    eg_lo_apply_t_T(ls->lo, x, w);
  else
    eg_lo_apply_T(ls->lo, x, w);
  k_gm_bminus<T><<<gridN(N), 256, 0, m->stream>>>(b, w, N);
  norm_T<T>(ls, w, beta, nullptr);
  k_gm_init<T><<<1, 32, 0, m->stream>>>(beta, bnorm, first, ls->m, ls->dH, ls->dflags, ls->dscal);
  k_gm_scale<T><<<gridN(N), 256, 0, m->stream>>>(w, beta, N, V, ls->dflags, 0);
}

// vector width of the Arnoldi kernels: 16-byte loads when the vector length
// allows (every 2-D problem: nv = 4)
template <typename T>
int vec_width(int64_t N) {
  const int W = sizeof(T) == 4 ? 4 : 2;
  return (N % W == 0) ? W : 1;
}

template <typename T>
void launch_dots(eg_ls* ls, const T* V, const T* w, int cnt, int with_ww, const int* fl, int need,
                 unsigned int* counter, T* h, T* ww) {
  eg_mesh* m = ls->lo->mesh;
  const int stride = ls->m + 2;
  const int64_t N = m->ndof;
  T* part = (T*)ls->part;
  if (vec_width<T>(N) > 1)
    k_gm_dots2<T, (sizeof(T) == 4 ? 4 : 2)><<<ls->nblk, 256, 0, m->stream>>>(
        V, w, cnt, with_ww, N, part, stride, fl, need, counter, h, ww);
  else
    k_gm_dots2<T, 1><<<ls->nblk, 256, 0, m->stream>>>(V, w, cnt, with_ww, N, part, stride, fl, need,
                                                      counter, h, ww);
}

template <typename T>
void launch_sub(eg_ls* ls, const T* V, const T* h, int cnt, T* w, const int* fl, int need,
                unsigned int* counter, int pass, int j, const T* h1, const T* h2, const T* ww, T* hn) {
  eg_mesh* m = ls->lo->mesh;
  const int stride = ls->m + 2;
  const int64_t N = m->ndof;
  T* part = (T*)ls->part;
  if (vec_width<T>(N) > 1)
    k_gm_sub2<T, (sizeof(T) == 4 ? 4 : 2)><<<ls->nblk, 256, 0, m->stream>>>(
        V, h, cnt, N, w, part, stride, fl, need, counter, pass, j, ls->m, h1, h2, ww, hn, ls->dH,
        ls->dflags, ls->dscal);
  else
    k_gm_sub2<T, 1><<<ls->nblk, 256, 0, m->stream>>>(V, h, cnt, N, w, part, stride, fl, need, counter,
                                                     pass, j, ls->m, h1, h2, ww, hn, ls->dH, ls->dflags,
                                                     ls->dscal);
}

// the Arnoldi loop of one restart cycle as stream launches
template <typename T>
void enqueue_arnoldi(eg_ls* ls) {
  eg_mesh* m = ls->lo->mesh;
  const int64_t N = m->ndof;
  const int mm = ls->m;
  T* V = (T*)ls->V;
  T* w = (T*)ls->w;
  T* z = (T*)ls->z;
  T* h = (T*)ls->h;
  T* h1 = h;
  T* h2 = h + (mm + 2);
  T* hn = h + 2 * (mm + 2);
  const int* fl = ls->dflags;
  for (int j = 0; j < mm; ++j) {
    T* vj = V + (size_t)j * N;
    // J M^-1 = I + K with K = C D^-1: the element blocks cancel with their
    // inverses.  Arnoldi runs on K (same Krylov space; (I + K) V_j =
    // V_{j+1} (H_K + I), the identity added in the Givens step), so
    // w = K v_j = C (D^-1 v_j) without the v_j term (transposed:
    // w = C^T (D^-T v_j))
    if (ls->trans) {
      eg_pc_apply_t_T(ls->pc, vj, z, fl);
      eg_cpl_apply_t_T(ls->lo, nullptr, z, w, fl);
    } else {
      eg_pc_apply_T(ls->pc, vj, z, fl);
      eg_cpl_apply_T(ls->lo, nullptr, z, w, fl);
    }
    // classical Gram-Schmidt (with |w|^2 before, for the DGKS test), a second
    // pass only when the test asks, Givens on the device
    T* ww = hn + 3;  // slots hn+1, hn+2 hold beta and |b| (enqueue_init)
    unsigned int* cnt = (unsigned int*)(ls->dflags + 8);
    launch_dots<T>(ls, V, w, j + 1, 1, fl, -1, cnt, h1, ww);
    launch_sub<T>(ls, V, h1, j + 1, w, fl, -1, cnt + 1, 1, j, h1, h2, ww, hn);
    launch_dots<T>(ls, V, w, j + 1, 0, fl, F_REORTH, cnt, h2, ww);
    launch_sub<T>(ls, V, h2, j + 1, w, fl, F_REORTH, cnt + 1, 2, j, h1, h2, ww, hn);
    k_gm_scale<T><<<gridN(N), 256, 0, m->stream>>>(w, hn, N, V + (size_t)(j + 1) * N, ls->dflags, 0);
  }
}

// end of a cycle: y = H^-1 g, x += M^-1 V y, true residual, next set-up
template <typename T>
void enqueue_tail(eg_ls* ls) {
  eg_mesh* m = ls->lo->mesh;
  const int64_t N = m->ndof;
  const int mm = ls->m;
  T* V = (T*)ls->V;
  T* w = (T*)ls->w;
  T* z = (T*)ls->z;
  k_gm_lsq<<<1, 256, 0, m->stream>>>(mm, ls->dH, ls->dflags);
  k_gm_Vy<T><<<gridN(N), 256, 0, m->stream>>>(V, ls->dH + (size_t)(mm + 1) * mm + 3 * mm + 1, N, w,
                                              ls->dflags);
  if (ls->trans)
    eg_pc_apply_t_T(ls->pc, w, z);
  else
    eg_pc_apply_T(ls->pc, w, z);
  k_gm_add<T><<<gridN(N), 256, 0, m->stream>>>(z, (T*)ls->xT, N);
  enqueue_init<T>(ls, 0);
}

// one restart cycle, the update, and the set-up of the next cycle
template <typename T>
void enqueue_cycle(eg_ls* ls) {
  enqueue_arnoldi<T>(ls);
  enqueue_tail<T>(ls);
}

// capture fn into a graph; on failure fall back to eager launches
template <typename F>
bool capture(eg_mesh* m, F fn, cudaGraphExec_t* exec, int64_t* nodes) {
  if (m->stream == 0 || m->stream == cudaStreamLegacy || m->stream == cudaStreamPerThread) return false;
  cudaGraph_t graph = nullptr;
  m->capturing = true;
  cudaError_t e = cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    m->capturing = false;
    cudaGetLastError();
    return false;
  }
  fn();
  e = cudaStreamEndCapture(m->stream, &graph);
  m->capturing = false;
  if (e != cudaSuccess || !graph) {
    cudaGetLastError();
    return false;
  }
  size_t n = 0;
  cudaGraphGetNodes(graph, nullptr, &n);
  e = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  *nodes = (int64_t)n;
  return true;
}

template <typename T>
int gmres_T(eg_ls* ls, eg_ls_stats* st, int transpose) {
  eg_mesh* m = ls->lo->mesh;
  ls->trans = transpose ? 1 : 0;
  // tolerances into device memory (graphs read them there)
  double sc[8] = {0, 0, 0, 0, ls->reltol, ls->abstol, 0, 0};
  int fl[8] = {0, 0, 0, 0, ls->itermax, 0, 0, 0};
  EG_CUDA(cudaMemcpyAsync(ls->dscal, sc, sizeof(sc), cudaMemcpyHostToDevice, m->stream));
  EG_CUDA(cudaMemcpyAsync(ls->dflags, fl, sizeof(fl), cudaMemcpyHostToDevice, m->stream));
  const bool coop = !transpose && eg_coop_usable(ls) && !m->capturing;
  if (coop) {
    // the whole solve in one persistent launch
    const int rc = eg_gmres_coop(ls);
    if (rc != EG_OK) return rc;
    int flags[8];
    double scal[8];
    EG_CUDA(cudaMemcpyAsync(ls->hh, ls->dscal, sizeof(scal), cudaMemcpyDeviceToHost, m->stream));
    EG_CUDA(cudaMemcpyAsync(ls->hh + 8, ls->dflags, sizeof(flags), cudaMemcpyDeviceToHost, m->stream));
    EG_CUDA(cudaStreamSynchronize(m->stream));
    std::memcpy(scal, ls->hh, sizeof(scal));
    std::memcpy(flags, ls->hh + 8, sizeof(flags));
    if (!std::isfinite(scal[S_BETA])) {
      eg_set_error("GMRES: non-finite residual");
      return EG_ERR_NONFINITE;
    }
    if (st) {
      st->iters = flags[F_ITS];
      st->restarts = flags[F_CYCLES];
      st->converged = flags[F_CONV];
      st->reorth = flags[F_NREORTH];
      st->res0 = scal[S_BETA0];
      st->res_final = scal[S_BETA];
    }
    return EG_OK;
  }
  // the graphs of this mode (forward or transposed), captured on first use
  void*& g_init = transpose ? ls->g_init_t : ls->g_init;
  void*& g_cycle = transpose ? ls->g_cycle_t : ls->g_cycle;
  int64_t& init_nodes = transpose ? ls->g_init_t_nodes : ls->g_init_nodes;
  int64_t& cycle_nodes = transpose ? ls->g_cycle_t_nodes : ls->g_cycle_nodes;
  bool& graphs_ok = transpose ? ls->graphs_t_ok : ls->graphs_ok;
  if (!g_init && !g_cycle && !graphs_ok) {
    cudaGraphExec_t gi = nullptr, gc = nullptr;
    bool ok = capture(m, [&]() { enqueue_init<T>(ls, 1); }, &gi, &init_nodes);
    ok = ok && capture(m, [&]() { enqueue_cycle<T>(ls); }, &gc, &cycle_nodes);
    if (ok) {
      g_init = (void*)gi;
      g_cycle = (void*)gc;
      graphs_ok = true;
    } else {
      if (gi) cudaGraphExecDestroy(gi);
      if (gc) cudaGraphExecDestroy(gc);
    }
  }
  auto run_init = [&]() -> int {
    if (graphs_ok) {
      EG_CUDA(cudaGraphLaunch((cudaGraphExec_t)g_init, m->stream));
      m->launches += init_nodes;
    } else {
      enqueue_init<T>(ls, 1);
      m->launches += 8;
    }
    return EG_OK;
  };
  auto run_cycle = [&]() -> int {
    if (graphs_ok) {
      EG_CUDA(cudaGraphLaunch((cudaGraphExec_t)g_cycle, m->stream));
      m->launches += cycle_nodes;
    } else {
      enqueue_cycle<T>(ls);
      m->launches += 12 * ls->m + 12;
    }
    return EG_OK;
  };
  int rc = run_init();
  if (rc != EG_OK) return rc;
  int flags[8];
  double scal[8];
  int restarts = 0;
  double res0 = -1.0;
  for (;;) {
    EG_CUDA(cudaMemcpyAsync(ls->hh, ls->dscal, sizeof(scal), cudaMemcpyDeviceToHost, m->stream));
    EG_CUDA(cudaMemcpyAsync(ls->hh + 8, ls->dflags, sizeof(flags), cudaMemcpyDeviceToHost, m->stream));
    EG_CUDA(cudaStreamSynchronize(m->stream));
    std::memcpy(scal, ls->hh, sizeof(scal));
    std::memcpy(flags, ls->hh + 8, sizeof(flags));
    if (res0 < 0) res0 = scal[S_BETA];
    if (!std::isfinite(scal[S_BETA])) {
      eg_set_error("GMRES: non-finite residual");
      return EG_ERR_NONFINITE;
    }
    if (flags[F_DONE]) break;
    rc = run_cycle();
    if (rc != EG_OK) return rc;
    ++restarts;
  }
  EG_CUDA(cudaGetLastError());
  if (st) {
    st->iters = flags[F_ITS];
    st->restarts = restarts;
    st->converged = flags[F_CONV];
    st->reorth = flags[F_NREORTH];
    st->res0 = res0;
    st->res_final = scal[S_BETA];
  }
  return EG_OK;
}

}  // namespace

void eg_gmres_release(eg_ls* ls) {
  if (ls->g_init) cudaGraphExecDestroy((cudaGraphExec_t)ls->g_init);
  if (ls->g_cycle) cudaGraphExecDestroy((cudaGraphExec_t)ls->g_cycle);
  ls->g_init = ls->g_cycle = nullptr;
  ls->graphs_ok = false;
  if (ls->g_init_t) cudaGraphExecDestroy((cudaGraphExec_t)ls->g_init_t);
  if (ls->g_cycle_t) cudaGraphExecDestroy((cudaGraphExec_t)ls->g_cycle_t);
  ls->g_init_t = ls->g_cycle_t = nullptr;
  ls->graphs_t_ok = false;
}

// x_T <- GMRES(J, b_T) from the initial guess in x_T; the graphs are bound to
// ls->bT / ls->xT, so callers stage their vectors there.
int eg_gmres_T(eg_ls* ls, const void* bT, void* xT, eg_ls_stats* st, int transpose) {
  if (bT != ls->bT || xT != ls->xT) {
    eg_set_error("GMRES: right-hand side and solution must be the solver's staging vectors");
    return EG_ERR_INVALID;
  }
  return ls->lo->prec == EG_F64 ? gmres_T<double>(ls, st, transpose) : gmres_T<float>(ls, st, transpose);
}
