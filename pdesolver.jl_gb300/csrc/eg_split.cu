// eg_split.cu -- entropy-conservative Hadamard split-form volume integral.
//
// Reference: calcVolumeIntegralsSplitFormCurvilinear
// (src/solver/euler/euler_funcs.jl:295-362) with calcSCurvilinear
// (src/Utils/curvilinear.jl:17-41):
//   S_x[j,k,d] = 1/2 sum_m (dxidx[m,d,j] Q_m(j,k) - dxidx[m,d,k] Q_m(k,j))
//   res_j -= 2 sum_d S_x[j,k,d] F_IR,d(q_j, q_k),  res_k += same   (k < j)
// The IR flux is linear in its direction, so sum_d S_x[j,k,d] F_IR,d equals
// one IR flux in the direction n_jk = S_x[j,k,:]; each pair (j,k) costs one
// Ismail-Roe average and one projection.  The square roots and logarithms of
// the averages are per-node quantities, computed once per node (FP64 is the
// scarce resource on GB300); a pair costs divisions and multiply-adds only.
//
// k_split_element: a CTA owns `epb` elements.  Phase 1: all threads walk the
// element pairs, writing G_jk = 2 F_IR(q_j, q_k; n_jk) to shared memory.
// Phase 2: thread (element, j) sums its row with the antisymmetry signs, adds
// the face terms (same lift as the weak form) and writes res_j once.
#include "eg_internal.h"
#include "eg_kernels.cuh"
#include "eg_physics.cuh"

using eg::Gas;

namespace {

template <int DIM>
__global__ void k_split_element(DevMesh md, const double* __restrict__ q,
                                const double* __restrict__ fflux, double* __restrict__ res,
                                unsigned int* __restrict__ status, int epb) {
  constexpr int NV = DIM + 2;
  constexpr int F = DIM + 1;
  extern __shared__ double smem[];
  const int Np = md.Np, Nf = md.Nf;
  const int P = Np * (Np - 1) / 2;
  const int S = md.S;
  double* sQ = smem;                          // [DIM][Np][Np]
  double* sL = sQ + DIM * Np * Np;            // [F][Nf][S]
  int* sPerm = reinterpret_cast<int*>(sL + F * Nf * S);
  double* sq = sL + F * Nf * S + (F * S + 1) / 2;  // [epb][Np][NV]
  double* sG = sq + (size_t)epb * Np * NV;    // [epb][P][NV]
  double* sres = sG + (size_t)epb * P * NV;   // [epb][Np][NV]
  double* sN = sres + (size_t)epb * Np * NV;  // [epb][Np][7] per-node IR quantities
  short2* sPair = reinterpret_cast<short2*>(sN + (size_t)epb * Np * 7);  // [P]
  for (int k = threadIdx.x; k < DIM * Np * Np; k += blockDim.x) sQ[k] = md.Q[k];
  for (int k = threadIdx.x; k < F * Nf * S; k += blockDim.x) sL[k] = md.liftS[k];
  for (int k = threadIdx.x; k < F * S; k += blockDim.x) sPerm[k] = md.perm[k];
  for (int j = threadIdx.x; j < Np; j += blockDim.x)
    for (int k = 0; k < j; ++k) sPair[j * (j - 1) / 2 + k] = make_short2((short)j, (short)k);
  const int e0 = blockIdx.x * epb;
  const int nloc = min(epb, md.E - e0);
  for (int t = threadIdx.x; t < nloc * Np * NV; t += blockDim.x)
    sq[t] = q[(size_t)e0 * Np * NV + t];
  __syncthreads();
  const Gas g{md.gamma, md.gamma_1};
  // per-node IR quantities (square roots and logarithms once per node)
  for (int t = threadIdx.x; t < nloc * Np; t += blockDim.x) {
    const eg::IRNode<DIM> nd = eg::ir_node<DIM>(g, sq + (size_t)t * NV);
    double* o = sN + (size_t)t * 7;
    o[0] = nd.z1; o[1] = nd.zp; o[2] = nd.lz1; o[3] = nd.lzp; o[4] = nd.u; o[5] = nd.v; o[6] = nd.w;
  }
  __syncthreads();
  // ---- phase 1: pair fluxes
  for (int t = threadIdx.x; t < nloc * P; t += blockDim.x) {
    const int le = t / P, pidx = t - le * P;
    const short2 jk = sPair[pidx];
    const int j = jk.x, k = jk.y;
    const int e = e0 + le;
    const double* dxj = md.dxidx + ((size_t)e * Np + j) * DIM * DIM;  // [x][xi]
    const double* dxk = md.dxidx + ((size_t)e * Np + k) * DIM * DIM;
    double n[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      double s = 0.0;
#pragma unroll
      for (int m = 0; m < DIM; ++m) {
        // Q_m(j,k) = sQ[m][k][j]; Q_m(k,j) = sQ[m][j][k]
        s = fma(dxj[d * DIM + m], sQ[((size_t)m * Np + k) * Np + j], s);
        s = fma(-dxk[d * DIM + m], sQ[((size_t)m * Np + j) * Np + k], s);
      }
      n[d] = s;  // 2 * S_x[j,k,d]
    }
    const double* nj = sN + ((size_t)le * Np + j) * 7;
    const double* nk = sN + ((size_t)le * Np + k) * 7;
    const eg::IRNode<DIM> Lj{nj[0], nj[1], nj[2], nj[3], nj[4], nj[5], nj[6]};
    const eg::IRNode<DIM> Lk{nk[0], nk[1], nk[2], nk[3], nk[4], nk[5], nk[6]};
    auto av = eg::ir_average_pre<DIM>(g, Lj, Lk);
    double Fp[NV];
    eg::ir_dir<DIM>(av, n, Fp);
    double* G = sG + ((size_t)le * P + pidx) * NV;
#pragma unroll
    for (int c = 0; c < NV; ++c) G[c] = Fp[c];
  }
  __syncthreads();
  // ---- phase 2: rows, then faces, then one coalesced store
  {
    const int le = threadIdx.x / Np, j = threadIdx.x - le * Np;
    if (le < nloc) {
      const double* qj = sq + ((size_t)le * Np + j) * NV;
      const double pj = eg::pressure<DIM>(g, qj);
      if (!(qj[0] > 0.0)) atomicOr(status, EG_DEV_NEG_DENSITY);
      if (!(pj > 0.0)) atomicOr(status, EG_DEV_NEG_PRESSURE);
      double acc[NV];
#pragma unroll
      for (int c = 0; c < NV; ++c) acc[c] = 0.0;
      const double* Ge = sG + (size_t)le * P * NV;
      for (int k = 0; k < j; ++k) {          // pair (j, k): res_j -= G
        const double* G = Ge + (size_t)(j * (j - 1) / 2 + k) * NV;
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] -= G[c];
      }
      for (int k = j + 1; k < Np; ++k) {     // pair (k, j): res_j += G
        const double* G = Ge + (size_t)(k * (k - 1) / 2 + j) * NV;
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] += G[c];
      }
      double* r = sres + ((size_t)le * Np + j) * NV;
#pragma unroll
      for (int c = 0; c < NV; ++c) r[c] = acc[c];
    }
  }
  __syncthreads();
  face_lift_smem<DIM>(md, fflux, sres, sL, sPerm, e0, nloc);
  for (int t = threadIdx.x; t < nloc * Np * NV; t += blockDim.x)
    res[(size_t)e0 * Np * NV + t] = sres[t];
}

}  // namespace

int eg_launch_split_element(eg_mesh* m, const double* q, double* res, int epb) {
  DevMesh md = dev_mesh(m);
  int threads;
  size_t smem;
  const int st = eg_element_shape(m, epb, 0, &threads, &smem);
  if (st != EG_OK) return st;
  const int blocks = (m->E + epb - 1) / epb;
  // once per process (thread-safe static initialisation)
  static const bool attr_set = [] {
    cudaFuncSetAttribute(k_split_element<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_split_element<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    return true;
  }();
  (void)attr_set;
  if (m->dim == 2)
    k_split_element<2><<<blocks, threads, smem, m->stream>>>(md, q, m->fflux, res, m->status, epb);
  else
    k_split_element<3><<<blocks, threads, smem, m->stream>>>(md, q, m->fflux, res, m->status, epb);
  return EG_OK;
}
