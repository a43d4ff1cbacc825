// eg_kernels.cuh -- kernel-side view of an eg_mesh and launch helpers shared
// by the translation units of libeulergpu.
#pragma once
#include "eg_internal.h"

// Plain-pointer view passed to kernels by value.
struct DevMesh {
  int E, Np, Nf, S, I, B;
  int face_flux;
  double gamma, gamma_1;
  const double* Q;        // [dim][Np][Np], Q[k][j][i] = Q_k(i, j)
  const double* interp;   // [F][Nf][S]
  const int* perm;        // [F][S]
  const int* nbrperm;     // [norient][Nf]
  const double* lift;     // [F][Np][Nf]
  const double* dxidx;    // [E][Np][dim][dim]
  const int* ifaces;      // [I][5]
  const double* nrm_face; // [I][Nf][dim]
  const int* bfaces;      // [B][2]
  const double* nrm_bndry;// [B][Nf][dim]
  const double* qg_bndry; // [B][Nf][nv]
  const int* bc_of_b;     // [B] boundary condition (eg_bc) of each boundary face
  const EFace* eface;     // [E][F]
  const double* Minv;     // [E][Np]
  const double* w;        // [Np]
  const double* jac;      // [E][Np]
  const double* liftS;    // [F][Nf][S]: interp[f][i][s] * wface[i]
  const int* nbrinv;      // [norient][Nf]: inverse of nbrperm
  const double* wface;    // [Nf]
  int sparse_face;        // face nodes are volume nodes (interp = identity)
};

// Face terms of the SBP weak form added into a shared-memory residual
// sres[epb][Np][NV] of the CTA's elements e0 .. e0+nloc-1 (reference
// interiorfaceintegrate! / boundaryintegrate! with Subtract: elementL and
// boundary faces subtract, elementR adds).  One pass per local face; in a
// pass thread t handles (element, stencil node) so only stencil nodes do
// work, and no two threads touch the same entry (deterministic, no atomics).
template <int DIM>
__device__ __forceinline__ void face_lift_smem(const DevMesh& md, const double* __restrict__ fflux,
                                               double* sres, const double* sLift, const int* sPerm,
                                               int e0, int nloc) {
  constexpr int NV = DIM + 2;
  constexpr int F = DIM + 1;
  const int Np = md.Np, Nf = md.Nf, S = md.S;
#pragma unroll 1
  for (int f = 0; f < F; ++f) {
    for (int t = threadIdx.x; t < nloc * S; t += blockDim.x) {
      const int le = t / S, s = t - le * S;
      const EFace ef = md.eface[(size_t)(e0 + le) * F + f];
      const double* fl = fflux + (size_t)ef.slot * Nf * NV;
      double acc[NV];
#pragma unroll
      for (int c = 0; c < NV; ++c) acc[c] = 0.0;
      if (md.sparse_face) {
        const int i = ef.side ? md.nbrinv[ef.orient * Nf + s] : s;
        const double a = md.wface[s];
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] = a * fl[i * NV + c];
      } else if (ef.side == 0) {
        for (int i = 0; i < Nf; ++i) {
          const double a = sLift[(f * Nf + i) * S + s];
#pragma unroll
          for (int c = 0; c < NV; ++c) acc[c] = fma(a, fl[i * NV + c], acc[c]);
        }
      } else {
        const int* nb = md.nbrperm + ef.orient * Nf;
        for (int i = 0; i < Nf; ++i) {
          const double a = sLift[(f * Nf + nb[i]) * S + s];
#pragma unroll
          for (int c = 0; c < NV; ++c) acc[c] = fma(a, fl[i * NV + c], acc[c]);
        }
      }
      double* r = sres + ((size_t)le * Np + sPerm[f * S + s]) * NV;
      if (ef.side == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) r[c] -= acc[c];
      } else {
#pragma unroll
        for (int c = 0; c < NV; ++c) r[c] += acc[c];
      }
    }
    __syncthreads();
  }
}

DevMesh dev_mesh(const eg_mesh* m);
int eg_launch_residual(eg_mesh* m, const double* q, double* res);
int eg_launch_split_element(eg_mesh* m, const double* q, double* res, int epb);
int eg_launch_norm(eg_mesh* m, const double* r, int strongres, double* out_dev);
