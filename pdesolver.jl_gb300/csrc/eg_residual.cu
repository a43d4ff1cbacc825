// eg_residual.cu -- evalResidual on the device.
//
// Reference: src/solver/euler/euler.jl:111-175 (evalResidual), with the fused
// per-element / per-face forms of euler_funcs.jl:158-205
// (calcVolumeIntegrals_nopre), flux.jl:79-123 (calcFaceIntegral_nopre) and
// bc.jl:290-329 (calcBoundaryFlux_nopre).
//
// Two launches per evaluation:
//   k_face_flux   one thread per (face, face node): interpolate both sides
//                 from the stencil (SBP interp/perm/nbrperm), numerical flux
//                 (Roe / Ismail-Roe; boundary: Roe against the precomputed
//                 Dirichlet state).  Each interface flux is computed once.
//   k_element     one thread per (element, node): Euler flux in the
//                 parametric directions into shared memory, then
//                 res_j = sum_k sum_i Q_k(i,j) F_k,i (weak form Q^T F) and the
//                 face terms -(+) sum_i lift_f(j,i) F_face,i for the elementL
//                 (elementR) side.  No atomics: every residual entry is written
//                 by exactly one thread, so results are deterministic.
// The split-form (Hadamard) volume term of volume_integral_type 2 lives in
// eg_split.cu.
#include <cstdio>

#include "eg_internal.h"
#include "eg_kernels.cuh"
#include "eg_physics.cuh"

using eg::Gas;

namespace {

template <int DIM>
__global__ void k_face_flux(DevMesh md, const double* __restrict__ q, double* __restrict__ fflux) {
  constexpr int NV = DIM + 2;
  const int Nf = md.Nf, S = md.S, Np = md.Np;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (md.I + md.B) * Nf) return;
  const int slot = t / Nf, i = t - slot * Nf;
  const Gas g{md.gamma, md.gamma_1};
  double qL[NV], qR[NV], fl[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) { qL[c] = 0.0; qR[c] = 0.0; }
  if (slot < md.I) {
    const int* itf = md.ifaces + 5 * slot;
    const int eL = itf[0], eR = itf[1], fL = itf[2], fR = itf[3], o = itf[4];
    const int iR = md.nbrperm[o * Nf + i];
    const double* cL = md.interp + ((size_t)fL * Nf + i) * S;
    const double* cR = md.interp + ((size_t)fR * Nf + iR) * S;
    const int* pL = md.perm + fL * S;
    const int* pR = md.perm + fR * S;
    for (int s = 0; s < S; ++s) {
      const double a = cL[s], b = cR[s];
      const double* xa = q + ((size_t)eL * Np + pL[s]) * NV;
      const double* xb = q + ((size_t)eR * Np + pR[s]) * NV;
#pragma unroll
      for (int c = 0; c < NV; ++c) {
        qL[c] = fma(a, xa[c], qL[c]);
        qR[c] = fma(b, xb[c], qR[c]);
      }
    }
    double nrm[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) nrm[k] = md.nrm_face[((size_t)slot * Nf + i) * DIM + k];
    if (md.face_flux == EG_FLUX_ROE) {
      eg::roe_flux<DIM>(g, qL, qR, nrm, fl);
    } else {
      // per-side square roots from one rsqrt each, logarithms only on the
      // log-mean branch
      const auto nL = eg::ir_node<DIM, false>(g, qL);
      const auto nR = eg::ir_node<DIM, false>(g, qR);
      const auto av = eg::ir_average_pre<DIM, false>(g, nL, nR);
      eg::ir_dir<DIM>(av, nrm, fl);
    }
  } else {
    const int b = slot - md.I;
    const int e = md.bfaces[2 * b], f = md.bfaces[2 * b + 1];
    const double* cL = md.interp + ((size_t)f * Nf + i) * S;
    const int* pL = md.perm + f * S;
    for (int s = 0; s < S; ++s) {
      const double a = cL[s];
      const double* xa = q + ((size_t)e * Np + pL[s]) * NV;
#pragma unroll
      for (int c = 0; c < NV; ++c) qL[c] = fma(a, xa[c], qL[c]);
    }
    double nrm[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) nrm[k] = md.nrm_bndry[((size_t)b * Nf + i) * DIM + k];
    if (md.bc_of_b[b] == EG_BC_NOPENETRATION_ES) {
      eg::wall_es_flux<DIM>(g, qL, nrm, fl);
    } else {
#pragma unroll
      for (int c = 0; c < NV; ++c) qR[c] = md.qg_bndry[((size_t)b * Nf + i) * NV + c];
      eg::roe_flux<DIM>(g, qL, qR, nrm, fl);
    }
  }
  double* out = fflux + (size_t)t * NV;
#pragma unroll
  for (int c = 0; c < NV; ++c) out[c] = fl[c];
}

// Weak-form volume contraction of the CTA's elements on the FP64 tensor
// cores: R[j][(le, c)] = sum_kk A[j][kk] B[kk][(le, c)] with
// A = [Q_1^T | ... | Q_DIM^T] (Np x DIM Np, A[j][k Np + i] = Q_k(i, j)) and B
// the parametric fluxes of the elements stacked by column (B[k Np + i][le NV
// + c] = F_k,i,c of element le).  Each warp owns 8 x 8 output tiles and runs
// mma.sync m8n8k4 (FP64) over K in steps of 4; rows, columns and K beyond
// the problem are zero padding.  Fragment layout of m8n8k4 .f64 (PTX ISA):
// lane l holds A[l / 4][l % 4], B[l % 4][l / 4] and C[l / 4][2 (l % 4) + {0,1}].
template <int DIM>
__device__ __forceinline__ void volume_mma(const double* sQ, const double* sF, double* sres,
                                           int Np, int nloc) {
  constexpr int NV = DIM + 2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int K = DIM * Np, Kp = (K + 3) & ~3;
  const int ncol = nloc * NV;
  const int mt = (Np + 7) >> 3, nt = (ncol + 7) >> 3;
  const int gq = lane >> 2, t4 = lane & 3;
  for (int tile = warp; tile < mt * nt; tile += nwarp) {
    const int tm = tile % mt, tn = tile / mt;
    const int row = tm * 8 + gq;          // A row of this lane, C row
    const int bcol = tn * 8 + gq;         // B column of this lane
    const bool brow_ok = bcol < ncol;
    const int ble = brow_ok ? bcol / NV : 0, bc = bcol - ble * NV;
    const double* Bp = sF + (size_t)ble * DIM * Np * NV + bc;   // + kk * NV
    const double* Ap = sQ + (size_t)row * Np;                    // + k Np Np + i
    double c0 = 0.0, c1 = 0.0;
    for (int k0 = 0; k0 < Kp; k0 += 4) {
      const int kk = k0 + t4;             // A column / B row of this lane
      double a = 0.0, b = 0.0;
      if (kk < K) {
        const int k = kk / Np, i = kk - k * Np;
        if (row < Np) a = Ap[(size_t)k * Np * Np + i];
        if (brow_ok) b = Bp[(size_t)kk * NV];
      }
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(c0), "+d"(c1)
                   : "d"(a), "d"(b));
    }
    const int col0 = tn * 8 + t4 * 2;
    if (row < Np) {
      if (col0 < ncol) {
        const int le = col0 / NV, c = col0 - le * NV;
        sres[((size_t)le * Np + row) * NV + c] = c0;
      }
      if (col0 + 1 < ncol) {
        const int le = (col0 + 1) / NV, c = col0 + 1 - le * NV;
        sres[((size_t)le * Np + row) * NV + c] = c1;
      }
    }
  }
}

// Shared-memory layout of k_element:
//   Q[dim][Np][Np] | liftS[F][Nf][S] | perm[F][S] (ints, padded) | Fbuf[epb][dim][Np][NV]
//   | sres[epb][Np][NV]
// MMA: the volume contraction runs on the FP64 tensor cores (volume_mma);
// the block is then a whole number of warps.
template <int DIM, bool MMA>
__global__ void k_element(DevMesh md, const double* __restrict__ q,
                          const double* __restrict__ fflux, double* __restrict__ res,
                          unsigned int* __restrict__ status, int epb) {
  constexpr int NV = DIM + 2;
  constexpr int F = DIM + 1;
  extern __shared__ double smem[];
  const int Np = md.Np, Nf = md.Nf, S = md.S;
  double* sQ = smem;
  double* sL = sQ + DIM * Np * Np;
  int* sPerm = reinterpret_cast<int*>(sL + F * Nf * S);
  double* sF = sL + F * Nf * S + (F * S + 1) / 2;
  double* sres = sF + (size_t)epb * DIM * Np * NV;
  for (int k = threadIdx.x; k < DIM * Np * Np; k += blockDim.x) sQ[k] = md.Q[k];
  for (int k = threadIdx.x; k < F * Nf * S; k += blockDim.x) sL[k] = md.liftS[k];
  for (int k = threadIdx.x; k < F * S; k += blockDim.x) sPerm[k] = md.perm[k];
  const int e0 = blockIdx.x * epb;
  const int nloc = min(epb, md.E - e0);
  const int le = threadIdx.x / Np, j = threadIdx.x - le * Np;
  const int e = e0 + le;
  const bool active = le < nloc;
  const Gas g{md.gamma, md.gamma_1};
  double* Fe = sF + (size_t)le * DIM * Np * NV;  // [k][i][c]
  if (active) {
    double qj[NV];
    const double* src = q + ((size_t)e * Np + j) * NV;
#pragma unroll
    for (int c = 0; c < NV; ++c) qj[c] = src[c];
    const double p = eg::pressure<DIM>(g, qj);
    if (!(qj[0] > 0.0)) atomicOr(status, EG_DEV_NEG_DENSITY);
    if (!(p > 0.0)) atomicOr(status, EG_DEV_NEG_PRESSURE);
    const double* dx = md.dxidx + ((size_t)e * Np + j) * DIM * DIM;  // [p(x)][k(xi)]
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      double dir[DIM];
#pragma unroll
      for (int pp = 0; pp < DIM; ++pp) dir[pp] = dx[pp * DIM + k];
      eg::euler_flux<DIM>(g, qj, dir, Fe + ((size_t)k * Np + j) * NV);
    }
  }
  __syncthreads();
  if (MMA) {
    volume_mma<DIM>(sQ, sF, sres, Np, nloc);
  } else if (active) {
    double acc[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) acc[c] = 0.0;
    // volume: (Q_k^T F_k)_j = sum_i Q_k(i, j) F_k,i ; sQ[k][j][i] = Q_k(i, j)
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const double* qrow = sQ + ((size_t)k * Np + j) * Np;
      const double* Fk = Fe + (size_t)k * Np * NV;
      for (int i = 0; i < Np; ++i) {
        const double a = qrow[i];
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] = fma(a, Fk[i * NV + c], acc[c]);
      }
    }
    double* r = sres + ((size_t)le * Np + j) * NV;
#pragma unroll
    for (int c = 0; c < NV; ++c) r[c] = acc[c];
  }
  __syncthreads();
  face_lift_smem<DIM>(md, fflux, sres, sL, sPerm, e0, nloc);
  // coalesced copy of the CTA's residual block
  for (int t = threadIdx.x; t < nloc * Np * NV; t += blockDim.x)
    res[(size_t)e0 * Np * NV + t] = sres[t];
}

// sum of r^2 * M^{+-1} per block, then one block reduces the partials in a
// fixed order (deterministic).
template <int NT>
__global__ void k_norm_partial(const double* __restrict__ r, const double* __restrict__ Minv,
                               int64_t nnode, int nv, int strongres, double* __restrict__ part) {
  __shared__ double sh[NT];
  double s = 0.0;
  for (int64_t n = blockIdx.x * (int64_t)NT + threadIdx.x; n < nnode; n += (int64_t)gridDim.x * NT) {
    const double mi = Minv[n];
    const double fac = strongres == 2 ? 1.0 : (strongres ? mi : 1.0 / mi);
    double t = 0.0;
    for (int c = 0; c < nv; ++c) {
      const double x = r[n * nv + c];
      t = fma(x, x, t);
    }
    s = fma(t, fac, s);
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = NT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

template <int NT>
__global__ void k_norm_final(const double* __restrict__ part, int n, double* __restrict__ out) {
  __shared__ double sh[NT];
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += NT) s += part[k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = NT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sqrt(sh[0]);
}

// boundary functional: partial sums of w_i p(q_face,i) |nrm_i| over the
// faces b0 <= b < b1 (one thread per face node), then k_norm_final-style sum.
template <int DIM, int NT>
__global__ void k_functional_pressure(DevMesh md, const double* __restrict__ q, int b0, int b1,
                                      double* __restrict__ part) {
  constexpr int NV = DIM + 2;
  __shared__ double sh[NT];
  const int Nf = md.Nf, S = md.S, Np = md.Np;
  const Gas g{md.gamma, md.gamma_1};
  double acc = 0.0;
  for (int t = blockIdx.x * NT + threadIdx.x; t < (b1 - b0) * Nf; t += gridDim.x * NT) {
    const int b = b0 + t / Nf, i = t % Nf;
    const int e = md.bfaces[2 * b], f = md.bfaces[2 * b + 1];
    double qf[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) qf[c] = 0.0;
    for (int s = 0; s < S; ++s) {
      const double a = md.interp[((size_t)f * Nf + i) * S + s];
      const double* x = q + ((size_t)e * Np + md.perm[f * S + s]) * NV;
#pragma unroll
      for (int c = 0; c < NV; ++c) qf[c] = fma(a, x[c], qf[c]);
    }
    const double* nr = md.nrm_bndry + ((size_t)b * Nf + i) * DIM;
    double a2 = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) a2 = fma(nr[k], nr[k], a2);
    acc += md.wface[i] * eg::pressure<DIM>(g, qf) * sqrt(a2);
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = NT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// calcMaxWaveSpeed (reference euler_funcs.jl:1810-1834): max over the nodes
// of a + |u|, a = sqrt(gamma p / rho); per-block maxima, then one block
template <int DIM, int NT>
__global__ void k_wave_speed_partial(const double* __restrict__ q, int64_t nnode, double gamma,
                                     double gamma_1, double* __restrict__ part) {
  constexpr int NV = DIM + 2;
  __shared__ double sh[NT];
  const Gas g{gamma, gamma_1};
  double mx = 0.0;
  for (int64_t k = blockIdx.x * (int64_t)NT + threadIdx.x; k < nnode; k += (int64_t)gridDim.x * NT) {
    const double* qk = q + k * NV;
    const double p = eg::pressure<DIM>(g, qk);
    double u2 = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const double u = qk[d + 1] / qk[0];
      u2 = fma(u, u, u2);
    }
    mx = fmax(mx, sqrt(gamma * p / qk[0]) + sqrt(u2));
  }
  sh[threadIdx.x] = mx;
  __syncthreads();
  for (int w = NT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

template <int NT>
__global__ void k_max_final(const double* __restrict__ part, int n, double* __restrict__ out) {
  __shared__ double sh[NT];
  double mx = 0.0;
  for (int k = threadIdx.x; k < n; k += NT) mx = fmax(mx, part[k]);
  sh[threadIdx.x] = mx;
  __syncthreads();
  for (int w = NT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

template <int NT>
__global__ void k_sum_final(const double* __restrict__ part, int n, double* __restrict__ out) {
  __shared__ double sh[NT];
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += NT) s += part[k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = NT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

}  // namespace

DevMesh dev_mesh(const eg_mesh* m) {
  DevMesh d;
  d.E = m->E; d.Np = m->Np; d.Nf = m->Nf; d.S = m->S; d.I = m->I; d.B = m->B;
  d.gamma = m->dp.gamma; d.gamma_1 = m->dp.gamma_1;
  d.face_flux = m->params.face_flux;
  d.Q = m->Q; d.interp = m->interp; d.perm = m->perm; d.nbrperm = m->nbrperm;
  d.lift = m->lift; d.dxidx = m->dxidx; d.ifaces = m->ifaces; d.nrm_face = m->nrm_face;
  d.bfaces = m->bfaces; d.nrm_bndry = m->nrm_bndry; d.qg_bndry = m->qg_bndry; d.bc_of_b = m->bc_of_b;
  d.eface = m->eface; d.Minv = m->Minv; d.w = m->w; d.jac = m->jac;
  d.liftS = m->liftS; d.nbrinv = m->nbrinv; d.wface = m->wface; d.sparse_face = m->sparse_face;
  return d;
}

// Launch shape of the element kernel with `epb` elements per CTA (0: the
// built-in choice, 256 / Np weak form; the split form as many as fit 160 KB).
// Weak form: one thread per (element, node), rounded up to whole warps with
// the tensor-core contraction.  Split form: the pair table of every element
// in shared memory.
int eg_element_shape(const eg_mesh* m, int epb, int mma, int* threads, size_t* smem) {
  const int nv = m->nv, Np = m->Np;
  const size_t common = sizeof(double) * ((size_t)m->dim * Np * Np + (size_t)m->F * m->Nf * m->S +
                                          (size_t)(m->F * m->S + 1) / 2);
  if (m->params.volume_integral_type == 2) {
    if (mma) {
      eg_set_error("launch config: the split form has no tensor-core contraction");
      return EG_ERR_INVALID;
    }
    const int P = Np * (Np - 1) / 2;
    auto smem_of = [&](int e) {
      return common + sizeof(double) * ((size_t)e * Np * nv + (size_t)e * P * nv +
                                        (size_t)e * Np * nv + (size_t)e * Np * 7) +
             sizeof(short2) * (size_t)P;
    };
    if (epb <= 0) {
      epb = 256 / Np;
      if (epb < 1) epb = 1;
      while (epb > 1 && smem_of(epb) > 160 * 1024) --epb;
    }
    *smem = smem_of(epb);
    *threads = epb * Np;
  } else {
    if (epb <= 0) {
      epb = 256 / Np;
      if (epb < 1) epb = 1;
    }
    *smem = common + sizeof(double) * ((size_t)epb * m->dim * Np * nv + (size_t)epb * Np * nv);
    *threads = mma ? (epb * Np + 31) / 32 * 32 : epb * Np;
  }
  if (*threads > 1024 || *smem > 200 * 1024) {
    eg_set_error("launch config: %d elements per CTA need %d threads and %zu B of shared memory",
                 epb, *threads, *smem);
    return EG_ERR_INVALID;
  }
  return EG_OK;
}

static int effective_epb(const eg_mesh* m) {
  if (m->elem_epb > 0) return m->elem_epb;
  int e = 256 / m->Np;
  if (e < 1) e = 1;
  if (m->params.volume_integral_type == 2) {
    int threads;
    size_t smem;
    while (e > 1 && (eg_element_shape(m, e, 0, &threads, &smem) != EG_OK || smem > 160 * 1024)) --e;
  }
  return e;
}

int eg_launch_element(eg_mesh* m, const double* q, double* res) {
  if (m->params.volume_integral_type == 2) return eg_launch_split_element(m, q, res, effective_epb(m));
  DevMesh md = dev_mesh(m);
  const int epb = effective_epb(m);
  const bool mma = m->vol_mma != 0;
  int threads;
  size_t smem;
  int st = eg_element_shape(m, epb, mma, &threads, &smem);
  if (st != EG_OK) return st;
  const int blocks = (m->E + epb - 1) / epb;
  // once per process (thread-safe static initialisation)
  static const bool attr_set = [] {
    cudaFuncSetAttribute(k_element<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_element<3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_element<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_element<3, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    return true;
  }();
  (void)attr_set;
  if (m->dim == 2) {
    if (mma)
      k_element<2, true><<<blocks, threads, smem, m->stream>>>(md, q, m->fflux, res, m->status, epb);
    else
      k_element<2, false><<<blocks, threads, smem, m->stream>>>(md, q, m->fflux, res, m->status, epb);
  } else {
    if (mma)
      k_element<3, true><<<blocks, threads, smem, m->stream>>>(md, q, m->fflux, res, m->status, epb);
    else
      k_element<3, false><<<blocks, threads, smem, m->stream>>>(md, q, m->fflux, res, m->status, epb);
  }
  return EG_OK;
}

int eg_launch_residual(eg_mesh* m, const double* q, double* res) {
  DevMesh md = dev_mesh(m);
  const int nf_threads = (m->I + m->B) * m->Nf;
  if (nf_threads > 0) {
    const int nt = 128;
    eg_phase_begin(m, EG_PHASE_FACE);
    if (m->dim == 2)
      k_face_flux<2><<<(nf_threads + nt - 1) / nt, nt, 0, m->stream>>>(md, q, m->fflux);
    else
      k_face_flux<3><<<(nf_threads + nt - 1) / nt, nt, 0, m->stream>>>(md, q, m->fflux);
    eg_phase_end(m, EG_PHASE_FACE, 1);
  }
  eg_phase_begin(m, EG_PHASE_ELEMENT);
  const int st = eg_launch_element(m, q, res);
  eg_phase_end(m, EG_PHASE_ELEMENT, 1);
  return st;
}

int eg_launch_norm(eg_mesh* m, const double* r, int strongres, double* out_dev) {
  const int64_t nnode = (int64_t)m->E * m->Np;
  int blocks = (int)((nnode + 255) / 256);
  if (blocks > 1024) blocks = 1024;
  eg_phase_begin(m, EG_PHASE_NORM);
  k_norm_partial<256><<<blocks, 256, 0, m->stream>>>(r, m->Minv, nnode, m->nv, strongres, m->red);
  k_norm_final<256><<<1, 256, 0, m->stream>>>(m->red, blocks, out_dev);
  eg_phase_end(m, EG_PHASE_NORM, 2);
  return EG_OK;
}

int eg_check_status(eg_mesh* m) {
  unsigned int s = *m->h_status;
  if (s & EG_DEV_NEG_DENSITY) {
    eg_set_error("negative density");
    return EG_ERR_NEG_DENSITY;
  }
  if (s & EG_DEV_NEG_PRESSURE) {
    eg_set_error("negative pressure");
    return EG_ERR_NEG_PRESSURE;
  }
  if (s & EG_DEV_NONFINITE) {
    eg_set_error("non-finite value");
    return EG_ERR_NONFINITE;
  }
  if (s & EG_DEV_LU_PIVOT) {
    eg_set_error("zero pivot in block LU");
    return EG_ERR_LU_PIVOT;
  }
  return EG_OK;
}

extern "C" int eg_eval_residual(eg_mesh* m, const double* q, double* res, double t, int32_t mem) {
  (void)t;  // the implemented boundary states are time-independent
  if (!m || !q || !res) {
    eg_set_error("eg_eval_residual: NULL argument");
    return EG_ERR_INVALID;
  }
  const size_t bytes = sizeof(double) * (size_t)m->ndof;
  const double* qd = q;
  double* rd = res;
  if (mem == EG_MEM_HOST) {
    EG_CUDA(cudaMemcpyAsync(m->q_dev, q, bytes, cudaMemcpyHostToDevice, m->stream));
    qd = m->q_dev;
    rd = m->res_dev;
  }
  EG_CUDA(cudaMemsetAsync(m->status, 0, sizeof(unsigned int), m->stream));
  int st = eg_launch_residual(m, qd, rd);
  if (st != EG_OK) return st;
  EG_CUDA(cudaGetLastError());
  EG_CUDA(cudaMemcpyAsync(m->h_status, m->status, sizeof(unsigned int), cudaMemcpyDeviceToHost, m->stream));
  if (mem == EG_MEM_HOST)
    EG_CUDA(cudaMemcpyAsync(res, rd, bytes, cudaMemcpyDeviceToHost, m->stream));
  EG_CUDA(cudaStreamSynchronize(m->stream));
  return eg_check_status(m);
}

extern "C" int eg_calc_norm(eg_mesh* m, const double* r, int32_t strongres, int32_t mem, double* out) {
  if (!m || !r || !out) {
    eg_set_error("eg_calc_norm: NULL argument");
    return EG_ERR_INVALID;
  }
  const double* rd = r;
  if (mem == EG_MEM_HOST) {
    EG_CUDA(cudaMemcpyAsync(m->res_dev, r, sizeof(double) * (size_t)m->ndof, cudaMemcpyHostToDevice, m->stream));
    rd = m->res_dev;
  }
  eg_launch_norm(m, rd, strongres, m->red + 2048);
  EG_CUDA(cudaGetLastError());
  EG_CUDA(cudaMemcpyAsync(m->h_red, m->red + 2048, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  EG_CUDA(cudaStreamSynchronize(m->stream));
  *out = m->h_red[0];
  return EG_OK;
}

extern "C" int eg_calc_max_wave_speed(eg_mesh* m, const double* q, int32_t mem, double* out) {
  if (!m || !q || !out) {
    eg_set_error("eg_calc_max_wave_speed: NULL argument");
    return EG_ERR_INVALID;
  }
  const double* qd = q;
  if (mem == EG_MEM_HOST) {
    EG_CUDA(cudaMemcpyAsync(m->q_dev, q, sizeof(double) * (size_t)m->ndof, cudaMemcpyHostToDevice, m->stream));
    qd = m->q_dev;
  }
  const int64_t nnode = (int64_t)m->E * m->Np;
  int blocks = (int)((nnode + 255) / 256);
  if (blocks > 1024) blocks = 1024;
  if (m->dim == 2)
    k_wave_speed_partial<2, 256><<<blocks, 256, 0, m->stream>>>(qd, nnode, m->dp.gamma, m->dp.gamma_1, m->red);
  else
    k_wave_speed_partial<3, 256><<<blocks, 256, 0, m->stream>>>(qd, nnode, m->dp.gamma, m->dp.gamma_1, m->red);
  k_max_final<256><<<1, 256, 0, m->stream>>>(m->red, blocks, m->red + 2051);
  m->launches += 2;
  EG_CUDA(cudaGetLastError());
  EG_CUDA(cudaMemcpyAsync(m->h_red, m->red + 2051, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  EG_CUDA(cudaStreamSynchronize(m->stream));
  *out = m->h_red[0];
  return EG_OK;
}

extern "C" int eg_calc_functional(eg_mesh* m, const double* q, int32_t bc_group, int32_t mem,
                                  double* out) {
  if (!m || !q || !out || bc_group < 0 || bc_group >= m->nbc) {
    eg_set_error("eg_calc_functional: invalid argument (bc_group %d of %d)", bc_group, m ? m->nbc : 0);
    return EG_ERR_INVALID;
  }
  const double* qd = q;
  if (mem == EG_MEM_HOST) {
    EG_CUDA(cudaMemcpyAsync(m->q_dev, q, sizeof(double) * (size_t)m->ndof, cudaMemcpyHostToDevice, m->stream));
    qd = m->q_dev;
  }
  const int b0 = m->h_bndry_offsets[bc_group], b1 = m->h_bndry_offsets[bc_group + 1];
  DevMesh md = dev_mesh(m);
  int blocks = ((b1 - b0) * m->Nf + 255) / 256;
  if (blocks < 1) blocks = 1;
  if (blocks > 1024) blocks = 1024;
  eg_phase_begin(m, EG_PHASE_OTHER);
  if (m->dim == 2)
    k_functional_pressure<2, 256><<<blocks, 256, 0, m->stream>>>(md, qd, b0, b1, m->red);
  else
    k_functional_pressure<3, 256><<<blocks, 256, 0, m->stream>>>(md, qd, b0, b1, m->red);
  k_sum_final<256><<<1, 256, 0, m->stream>>>(m->red, blocks, m->red + 2048);
  eg_phase_end(m, EG_PHASE_OTHER, 2);
  EG_CUDA(cudaGetLastError());
  EG_CUDA(cudaMemcpyAsync(m->h_red, m->red + 2048, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  EG_CUDA(cudaStreamSynchronize(m->stream));
  *out = m->h_red[0];
  return EG_OK;
}
