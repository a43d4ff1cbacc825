// eg_jacobian.cu -- explicit Jacobian dR/dq of the weak-form Euler residual.
//
// Reference: evalJacobian (src/solver/euler/evalJacobian.jl:6-72) with
//   calcVolumeIntegrals_nopre_diff  euler_funcs_diff.jl:54-103
//   calcFaceIntegral_nopre_diff     flux_diff.jl:6-100 (interiorFaceCombined_jac!)
//   getBCFluxes_diff                bc_diff.jl:16-212 (boundary: the Dirichlet
//                                   state does not depend on q)
//   assembleElement/Interface/Boundary  src/jacobian/jacobian.jl:822-1135, 1715-1800
// The point flux Jacobians (dF/dq of calcEulerFlux, dF/dqL and dF/dqR of the
// Roe / IR flux) are forward-mode derivatives of the device flux routines of
// eg_physics.cuh (the reference differentiates the same routines by hand).
//
// Storage (element-block sparse, column-major blocks, see eulergpu.h):
//   diag[E][Np*nv][Np*nv]          element blocks (volume + own face terms)
//   cpl[I][2][S*nv][S*nv]          interface coupling blocks LR, RL (row-major)
// Kernels (templated on the precision T of the Jacobian: double or float):
//   k_elem_jac_split  the element block of the entropy-stable split form
//   k_face_jac     one thread per (face slot, face node): dF/dqL, dF/dqR
//   k_elem_jac     one CTA per element: sum_k Q_k(m,j) A_k(q_m) into a shared
//                  block, then the element's own face terms, coalesced store
//   k_couple_jac   one thread per coupling-block entry
#include <vector>

#include "eg_internal.h"
#include "eg_kernels.cuh"
#include "eg_linalg.h"
#include "eg_physics.cuh"

using eg::Fwd;
using eg::Gas;

namespace {

// dF/dqL (and dF/dqR for interfaces) at every face node; dF[slot][i][side][a][b]
template <int DIM, typename T>
__global__ void k_face_jac(DevMesh md, const double* __restrict__ q, T* __restrict__ dF) {
  constexpr int NV = DIM + 2;
  using D2 = Fwd<T, 2 * NV>;
  const int Nf = md.Nf, S = md.S, Np = md.Np;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (md.I + md.B) * Nf) return;
  const int slot = t / Nf, i = t - slot * Nf;
  const Gas g{md.gamma, md.gamma_1};
  T qLr[NV], qRr[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) { qLr[c] = T(0); qRr[c] = T(0); }
  T nrm[DIM];
  const bool interior = slot < md.I;
  const bool wall = !interior && md.bc_of_b[slot - md.I] == EG_BC_NOPENETRATION_ES;
  if (interior) {
    const int* itf = md.ifaces + 5 * slot;
    const int eL = itf[0], eR = itf[1], fL = itf[2], fR = itf[3], o = itf[4];
    const int iR = md.nbrperm[o * Nf + i];
    const double* cL = md.interp + ((size_t)fL * Nf + i) * S;
    const double* cR = md.interp + ((size_t)fR * Nf + iR) * S;
    for (int s = 0; s < S; ++s) {
      const T a = T(cL[s]), b = T(cR[s]);
      const double* xa = q + ((size_t)eL * Np + md.perm[fL * S + s]) * NV;
      const double* xb = q + ((size_t)eR * Np + md.perm[fR * S + s]) * NV;
#pragma unroll
      for (int c = 0; c < NV; ++c) {
        qLr[c] += a * T(xa[c]);
        qRr[c] += b * T(xb[c]);
      }
    }
#pragma unroll
    for (int k = 0; k < DIM; ++k) nrm[k] = T(md.nrm_face[((size_t)slot * Nf + i) * DIM + k]);
  } else {
    const int b = slot - md.I;
    const int e = md.bfaces[2 * b], f = md.bfaces[2 * b + 1];
    const double* cL = md.interp + ((size_t)f * Nf + i) * S;
    for (int s = 0; s < S; ++s) {
      const T a = T(cL[s]);
      const double* xa = q + ((size_t)e * Np + md.perm[f * S + s]) * NV;
#pragma unroll
      for (int c = 0; c < NV; ++c) qLr[c] += a * T(xa[c]);
    }
#pragma unroll
    for (int k = 0; k < DIM; ++k) nrm[k] = T(md.nrm_bndry[((size_t)b * Nf + i) * DIM + k]);
#pragma unroll
    for (int c = 0; c < NV; ++c) qRr[c] = T(md.qg_bndry[((size_t)b * Nf + i) * NV + c]);
  }
  D2 qL[NV], qR[NV], fl[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    qL[c] = D2(qLr[c]);
    qR[c] = D2(qRr[c]);
    qL[c].d[c] = T(1);
    if (interior) qR[c].d[NV + c] = T(1);
  }
  if (wall) {
    // the mirror state depends on q: its derivative runs through the flux
    eg::wall_es_flux<DIM>(g, qL, nrm, fl);
  } else if (!interior || md.face_flux == EG_FLUX_ROE) {
    eg::roe_flux<DIM>(g, qL, qR, nrm, fl);
  } else {
    auto av = eg::ir_average<DIM>(g, qL, qR);
    eg::ir_dir<DIM>(av, nrm, fl);
  }
  T* out = dF + (size_t)t * 2 * NV * NV;
#pragma unroll
  for (int a = 0; a < NV; ++a)
#pragma unroll
    for (int b = 0; b < NV; ++b) {
      out[a * NV + b] = fl[a].d[b];
      out[NV * NV + a * NV + b] = fl[a].d[NV + b];
    }
}

// The element's own face terms (LL for elementL / boundary, RR for
// elementR) added into the shared block sB of element e, then stored.
template <int DIM, typename T>
__device__ void elem_face_terms(const DevMesh& md, const T* __restrict__ dF, T* sB, int e) {
  constexpr int NV = DIM + 2;
  constexpr int F = DIM + 1;
  const int Np = md.Np, Nf = md.Nf, S = md.S;
  const int n = Np * NV;
  for (int f = 0; f < F; ++f) {
    const EFace ef = md.eface[(size_t)e * F + f];
    const T* dFs = dF + (size_t)ef.slot * Nf * 2 * NV * NV;
    const int sideoff = ef.side ? NV * NV : 0;  // dF/dq of this element's state
    const T sgn = ef.side ? T(1) : T(-1);
    const int* nb = md.nbrperm + ef.orient * Nf;
    if (md.sparse_face) {
      // interp = identity: only stencil node s with itself, through the face
      // node i that sees it, acc = wface[s] dF_i (the dense sum's one term)
      for (int t = threadIdx.x; t < S * NV * NV; t += blockDim.x) {
        const int ab = t % (NV * NV), s = t / (NV * NV);
        const int a = ab / NV, b = ab - a * NV;
        const int i = ef.side ? md.nbrinv[ef.orient * Nf + s] : s;
        const T acc = T(md.wface[s]) * dFs[(size_t)i * 2 * NV * NV + sideoff + a * NV + b];
        const int node = md.perm[f * S + s] * NV;
        sB[(size_t)(node + b) * n + node + a] += sgn * acc;
      }
      __syncthreads();
      continue;
    }
    for (int t = threadIdx.x; t < S * S * NV * NV; t += blockDim.x) {
      const int ab = t % (NV * NV), ss = t / (NV * NV);
      const int s = ss / S, sp = ss - s * S;        // row stencil s, column stencil s'
      const int a = ab / NV, b = ab - a * NV;
      T acc = T(0);
      for (int i = 0; i < Nf; ++i) {
        const int ii = ef.side ? nb[i] : i;         // this element's face-node index
        const T l = T(md.liftS[((size_t)f * Nf + ii) * S + s]);
        const T r = T(md.interp[((size_t)f * Nf + ii) * S + sp]);
        acc += l * r * dFs[(size_t)i * 2 * NV * NV + sideoff + a * NV + b];
      }
      const int row = md.perm[f * S + s] * NV + a;
      const int col = md.perm[f * S + sp] * NV + b;
      sB[(size_t)col * n + row] += sgn * acc;
    }
    __syncthreads();
  }
}

// Element block: one CTA per element.  Shared: A[k][m][a][b] (flux
// Jacobians at the nodes), the block blk[col][row] and face tables.  With
// block_in_global (blocks too large for shared memory, e.g. 225 unknowns of
// the p=3 diagonal-E tetrahedron) the block is accumulated in place in the
// output: every entry has one writer per pass, passes are separated by
// __syncthreads, which orders the CTA's global accesses as well.
template <int DIM, typename T>
__global__ void k_elem_jac(DevMesh md, const double* __restrict__ q, const T* __restrict__ dF,
                           T* __restrict__ diag, int block_in_global) {
  constexpr int NV = DIM + 2;
  using D1 = Fwd<T, NV>;
  extern __shared__ unsigned char smraw[];
  const int Np = md.Np;
  const int n = Np * NV;
  const int e = blockIdx.x;
  T* sA = reinterpret_cast<T*>(smraw);               // [DIM][Np][NV][NV]
  T* sQ = sA + (size_t)DIM * Np * NV * NV;            // [DIM][Np][Np] = Q
  T* sB = block_in_global ? diag + (size_t)e * n * n  // [n][n] col-major
                          : sQ + (size_t)DIM * Np * Np;
  for (int t = threadIdx.x; t < DIM * Np * Np; t += blockDim.x) sQ[t] = T(md.Q[t]);
  const Gas g{md.gamma, md.gamma_1};
  // flux Jacobians A_k(q_m) = dF_k/dq at node m, direction dxidx[.][k]
  for (int t = threadIdx.x; t < Np * DIM; t += blockDim.x) {
    const int m = t / DIM, k = t - m * DIM;
    const double* src = q + ((size_t)e * Np + m) * NV;
    D1 qm[NV], Fk[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      qm[c] = D1(T(src[c]));
      qm[c].d[c] = T(1);
    }
    const double* dx = md.dxidx + ((size_t)e * Np + m) * DIM * DIM;
    T dir[DIM];
#pragma unroll
    for (int pp = 0; pp < DIM; ++pp) dir[pp] = T(dx[pp * DIM + k]);
    eg::euler_flux<DIM>(g, qm, dir, Fk);
    T* A = sA + (((size_t)k * Np + m) * NV) * NV;
#pragma unroll
    for (int a = 0; a < NV; ++a)
#pragma unroll
      for (int b = 0; b < NV; ++b) A[a * NV + b] = Fk[a].d[b];
  }
  __syncthreads();
  // volume: blk[(m,b)][(j,a)] = sum_k Q_k(m, j) A_k(m)[a][b];  Q[k][j][m] = Q_k(m, j)
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    const int col = t / n, row = t - col * n;
    const int m = col / NV, b = col - m * NV;
    const int j = row / NV, a = row - j * NV;
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < DIM; ++k)
      acc += sQ[((size_t)k * Np + j) * Np + m] * sA[(((size_t)k * Np + m) * NV + a) * NV + b];
    sB[t] = acc;
  }
  __syncthreads();
  elem_face_terms<DIM, T>(md, dF, sB, e);
  if (block_in_global) return;
  T* dst = diag + (size_t)e * n * n;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) dst[t] = sB[t];
}

// d/dq of the pair term of the split form for the pair (first, second),
// first > second (residual: res_first -= G, res_second += G with
// G = F_IR(q_first, q_second; n), n = 2 S_x[first, second, :]), with respect
// to q_first (wrt_first) or q_second, times sign, added into blk[a][b].
template <int DIM, typename T>
__device__ void split_pair_jac(const DevMesh& md, const Gas& g, const double* __restrict__ qe,
                               const double* __restrict__ dxe, const T* sQ, int first, int second,
                               bool wrt_first, T sign, T (&blk)[DIM + 2][DIM + 2]) {
  constexpr int NV = DIM + 2;
  using D1 = Fwd<T, NV>;
  const int Np = md.Np;
  const double* d1 = dxe + (size_t)first * DIM * DIM;
  const double* d2 = dxe + (size_t)second * DIM * DIM;
  T nrm[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    T acc = T(0);
#pragma unroll
    for (int m = 0; m < DIM; ++m) {
      // Q_m(first, second) = sQ[m][second][first]; Q_m(second, first) = sQ[m][first][second]
      acc += T(d1[d * DIM + m]) * sQ[((size_t)m * Np + second) * Np + first];
      acc -= T(d2[d * DIM + m]) * sQ[((size_t)m * Np + first) * Np + second];
    }
    nrm[d] = acc;
  }
  D1 qa[NV], qb[NV], G[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    qa[c] = D1(T(qe[(size_t)first * NV + c]));
    qb[c] = D1(T(qe[(size_t)second * NV + c]));
    if (wrt_first)
      qa[c].d[c] = T(1);
    else
      qb[c].d[c] = T(1);
  }
  auto av = eg::ir_average<DIM>(g, qa, qb);
  eg::ir_dir<DIM>(av, nrm, G);
#pragma unroll
  for (int a = 0; a < NV; ++a)
#pragma unroll
    for (int b = 0; b < NV; ++b) blk[a][b] += sign * G[a].d[b];
}

// Element block of the entropy-stable split form (volume_integral_type 2):
// the Hadamard pair terms differentiated pair by pair (reference
// calcVolumeIntegralsSplitFormCurvilinear_diff, euler_funcs_diff.jl:330-430),
// then the same face terms as the weak form.  One thread per (row node j,
// column node m) block of the element: an off-diagonal block is the one pair
// (j, m); a diagonal block sums the pairs of node j, in a fixed order.
template <int DIM, typename T>
__global__ void k_elem_jac_split(DevMesh md, const double* __restrict__ q, const T* __restrict__ dF,
                                 T* __restrict__ diag, int block_in_global) {
  constexpr int NV = DIM + 2;
  extern __shared__ unsigned char smraw[];
  const int Np = md.Np;
  const int n = Np * NV;
  const int e = blockIdx.x;
  T* sQ = reinterpret_cast<T*>(smraw);                // [DIM][Np][Np] = Q
  T* sB = block_in_global ? diag + (size_t)e * n * n  // [n][n] col-major (see k_elem_jac)
                          : sQ + (size_t)DIM * Np * Np;
  for (int t = threadIdx.x; t < DIM * Np * Np; t += blockDim.x) sQ[t] = T(md.Q[t]);
  __syncthreads();
  const Gas g{md.gamma, md.gamma_1};
  const double* qe = q + (size_t)e * Np * NV;
  const double* dxe = md.dxidx + (size_t)e * Np * DIM * DIM;
  for (int t = threadIdx.x; t < Np * Np; t += blockDim.x) {
    const int j = t / Np, m = t - j * Np;  // row node j, column node m
    T blk[NV][NV];
#pragma unroll
    for (int a = 0; a < NV; ++a)
#pragma unroll
      for (int b = 0; b < NV; ++b) blk[a][b] = T(0);
    if (m < j) {
      split_pair_jac<DIM, T>(md, g, qe, dxe, sQ, j, m, false, T(-1), blk);  // res_j -= G(q_j, q_m)
    } else if (m > j) {
      split_pair_jac<DIM, T>(md, g, qe, dxe, sQ, m, j, true, T(1), blk);   // res_j += G(q_m, q_j)
    } else {
      for (int k = 0; k < Np; ++k) {
        if (k < j) split_pair_jac<DIM, T>(md, g, qe, dxe, sQ, j, k, true, T(-1), blk);
        else if (k > j) split_pair_jac<DIM, T>(md, g, qe, dxe, sQ, k, j, false, T(1), blk);
      }
    }
#pragma unroll
    for (int a = 0; a < NV; ++a)
#pragma unroll
      for (int b = 0; b < NV; ++b) sB[(size_t)(m * NV + b) * n + j * NV + a] = blk[a][b];
  }
  __syncthreads();
  elem_face_terms<DIM, T>(md, dF, sB, e);
  if (block_in_global) return;
  T* dst = diag + (size_t)e * n * n;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) dst[t] = sB[t];
}

// Interface coupling blocks, stored row-major so an operator row is one
// contiguous read: cpl[nI][side][row = s*NV+a][col = s'*NV+b]:
//   side 0: rows elementL stencil, cols elementR stencil, from dF/dqR, sign -
//   side 1: rows elementR stencil, cols elementL stencil, from dF/dqL, sign +
// Face-diagonal operators (face nodes are volume nodes) keep only the
// nonzero NV x NV block of each row stencil node: cpl[nI][side][s][a][b];
// row node s of side 0 couples to elementR's node nbrperm[o][s], row node s
// of side 1 to elementL's node nbrinv[o][s] (the one face node joining them).
template <int DIM, typename T>
__global__ void k_couple_jac_diag(DevMesh md, const T* __restrict__ dF, T* __restrict__ cpl) {
  constexpr int NV = DIM + 2;
  const int Nf = md.Nf, S = md.S;
  const int64_t per = 2LL * S * NV * NV;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= per * md.I) return;
  const int nI = (int)(t / per);
  const int rem = (int)(t - (int64_t)nI * per);
  const int side = rem / (S * NV * NV);
  const int sab = rem - side * S * NV * NV;
  const int s = sab / (NV * NV), ab = sab - s * NV * NV;
  const int o = md.ifaces[5 * nI + 4];
  const T* dFs = dF + (size_t)nI * Nf * 2 * NV * NV;
  // the dense sum over face nodes has one nonzero term: wface[s] dF at the
  // face node i that sees row node s (side 0: i = s; side 1: i = nbrinv[s])
  if (side == 0) {
    cpl[t] = -(T(md.wface[s]) * dFs[(size_t)s * 2 * NV * NV + NV * NV + ab]);
  } else {
    const int i = md.nbrinv[o * Nf + s];
    cpl[t] = T(md.wface[s]) * dFs[(size_t)i * 2 * NV * NV + ab];
  }
}

template <int DIM, typename T>
__global__ void k_couple_jac(DevMesh md, const T* __restrict__ dF, T* __restrict__ cpl) {
  constexpr int NV = DIM + 2;
  const int Nf = md.Nf, S = md.S;
  const int nb = S * NV;
  const int64_t per = 2LL * nb * nb;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= per * md.I) return;
  const int nI = (int)(t / per);
  const int rem = (int)(t - (int64_t)nI * per);
  const int side = rem / (nb * nb);
  const int cr = rem - side * nb * nb;
  const int row = cr / nb, col = cr - row * nb;
  const int sp = col / NV, b = col - sp * NV;
  const int s = row / NV, a = row - s * NV;
  const int* itf = md.ifaces + 5 * nI;
  const int fL = itf[2], fR = itf[3], o = itf[4];
  const int* nbp = md.nbrperm + o * Nf;
  const T* dFs = dF + (size_t)nI * Nf * 2 * NV * NV;
  T acc = T(0);
  for (int i = 0; i < Nf; ++i) {
    const int iR = nbp[i];
    T l, r;
    int off;
    if (side == 0) {
      l = T(md.liftS[((size_t)fL * Nf + i) * S + s]);
      r = T(md.interp[((size_t)fR * Nf + iR) * S + sp]);
      off = NV * NV;
    } else {
      l = T(md.liftS[((size_t)fR * Nf + iR) * S + s]);
      r = T(md.interp[((size_t)fL * Nf + i) * S + sp]);
      off = 0;
    }
    acc += l * r * dFs[(size_t)i * 2 * NV * NV + off + a * NV + b];
  }
  cpl[t] = side == 0 ? -acc : acc;
}

template <typename T>
int launch_jac(eg_lo* lo, const double* q) {
  eg_mesh* m = lo->mesh;
  DevMesh md = dev_mesh(m);
  T* dF = reinterpret_cast<T*>(lo->dF);
  T* diag = reinterpret_cast<T*>(lo->diag);
  T* cpl = reinterpret_cast<T*>(lo->cpl);
  const int nslot = (m->I + m->B) * m->Nf;
  const int n = m->Np * m->nv;
  // the block in shared memory when it fits, else accumulated in place
  const size_t fixed = sizeof(T) * ((size_t)m->dim * m->Np * m->nv * m->nv + (size_t)m->dim * m->Np * m->Np);
  const int gblk = fixed + sizeof(T) * (size_t)n * n > 200 * 1024 ? 1 : 0;
  const size_t smem = fixed + (gblk ? 0 : sizeof(T) * (size_t)n * n);
  eg_phase_begin(m, EG_PHASE_OTHER);
  const bool split = m->params.volume_integral_type == 2;
  if (m->dim == 2) {
    k_face_jac<2, T><<<(nslot + 127) / 128, 128, 0, m->stream>>>(md, q, dF);
    if (split) {
      cudaFuncSetAttribute(k_elem_jac_split<2, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      k_elem_jac_split<2, T><<<m->E, 256, smem, m->stream>>>(md, q, dF, diag, gblk);
    } else {
      cudaFuncSetAttribute(k_elem_jac<2, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      k_elem_jac<2, T><<<m->E, 256, smem, m->stream>>>(md, q, dF, diag, gblk);
    }
  } else {
    k_face_jac<3, T><<<(nslot + 127) / 128, 128, 0, m->stream>>>(md, q, dF);
    if (split) {
      cudaFuncSetAttribute(k_elem_jac_split<3, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      k_elem_jac_split<3, T><<<m->E, 256, smem, m->stream>>>(md, q, dF, diag, gblk);
    } else {
      cudaFuncSetAttribute(k_elem_jac<3, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      k_elem_jac<3, T><<<m->E, 256, smem, m->stream>>>(md, q, dF, diag, gblk);
    }
  }
  const int64_t ncpl = (int64_t)eg_lo_coupling_size(lo);
  if (ncpl > 0) {
    const int blocks = (int)((ncpl + 255) / 256);
    if (lo->cpl_sparse) {
      if (m->dim == 2)
        k_couple_jac_diag<2, T><<<blocks, 256, 0, m->stream>>>(md, dF, cpl);
      else
        k_couple_jac_diag<3, T><<<blocks, 256, 0, m->stream>>>(md, dF, cpl);
    } else if (m->dim == 2) {
      k_couple_jac<2, T><<<blocks, 256, 0, m->stream>>>(md, dF, cpl);
    } else {
      k_couple_jac<3, T><<<blocks, 256, 0, m->stream>>>(md, dF, cpl);
    }
  }
  eg_phase_end(m, EG_PHASE_OTHER, ncpl > 0 ? 3 : 2);
  return EG_OK;
}

}  // namespace

int eg_jacobian_launch(eg_lo* lo, const double* q) {
  const size_t smem_needed = (lo->prec == EG_F64 ? 8 : 4) *
                             ((size_t)lo->mesh->dim * lo->mesh->Np * lo->mesh->nv * lo->mesh->nv +
                              (size_t)lo->mesh->dim * lo->mesh->Np * lo->mesh->Np);
  if (smem_needed > 200 * 1024) {
    eg_set_error("evalJacobian: element tables of %d nodes exceed shared memory", lo->mesh->Np);
    return EG_ERR_UNSUPPORTED;
  }
  return lo->prec == EG_F64 ? launch_jac<double>(lo, q) : launch_jac<float>(lo, q);
}
