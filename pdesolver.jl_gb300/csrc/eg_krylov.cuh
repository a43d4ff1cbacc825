// eg_krylov.cuh -- device helpers shared by the operator / preconditioner
// kernels and the persistent Arnoldi kernel.
#pragma once
#include "eg_kernels.cuh"

// Face-coupling part of row r of element e: sum over the element's interface
// faces whose stencil holds row r's node of C (coupling block) x (neighbour's
// stencil values).
// With a face-diagonal operator (md.sparse_face) the coupling storage is
// [I][2][S][NV][NV]: row stencil node s of a side couples only to the
// neighbour's stencil node facing it, nbrperm[o][s] from side 0 (elementL)
// and nbrinv[o][s] from side 1.
template <int DIM, typename T>
__device__ __forceinline__ T coupling_row(const DevMesh& md, const T* __restrict__ cpl,
                                          const int* __restrict__ spos, const T* __restrict__ x,
                                          int e, int r, int n) {
  constexpr int NV = DIM + 2;
  constexpr int F = DIM + 1;
  const int Np = md.Np, S = md.S, nb = S * NV;
  const int j = r / NV, a = r - j * NV;
  T acc = T(0);
#pragma unroll
  for (int f = 0; f < F; ++f) {
    const int s = spos[f * Np + j];
    if (s < 0) continue;
    const EFace ef = md.eface[(size_t)e * F + f];
    if (ef.slot >= md.I) continue;  // boundary face: no coupling
    const int* itf = md.ifaces + 5 * ef.slot;
    const int en = ef.side ? itf[0] : itf[1];
    const int fn = ef.side ? itf[2] : itf[3];
    const T* xn = x + (size_t)en * n;
    if (md.sparse_face) {
      const int o = itf[4];
      const int sp = ef.side ? md.nbrinv[o * md.Nf + s] : md.nbrperm[o * md.Nf + s];
      const T* C = cpl + ((((size_t)ef.slot * 2 + ef.side) * S + s) * NV + a) * NV;
      const T* xs = xn + md.perm[fn * S + sp] * NV;
#pragma unroll
      for (int b = 0; b < NV; ++b) acc += C[b] * xs[b];
      continue;
    }
    // row (s, a) of the row-major coupling block: nb contiguous values
    const T* C = cpl + (((size_t)ef.slot * 2 + ef.side) * nb + s * NV + a) * nb;
    for (int sp = 0; sp < S; ++sp) {
      const T* xs = xn + md.perm[fn * S + sp] * NV;
#pragma unroll
      for (int b = 0; b < NV; ++b) acc += C[sp * NV + b] * xs[b];
    }
  }
  return acc;
}

// dense element-block row: sum_c A[c*n + r] xe[c]; NB > 0 fixes n at compile
// time so the loads of a row are all in flight at once
template <int NB, typename T>
__device__ __forceinline__ T block_row(const T* __restrict__ A, const T* __restrict__ xe, int r, int n) {
  T acc0 = T(0), acc1 = T(0), acc2 = T(0), acc3 = T(0);
  if (NB > 0) {
#pragma unroll
    for (int c = 0; c < NB; c += 4) {
      acc0 += A[(size_t)c * NB + r] * xe[c];
      if (c + 1 < NB) acc1 += A[(size_t)(c + 1) * NB + r] * xe[c + 1];
      if (c + 2 < NB) acc2 += A[(size_t)(c + 2) * NB + r] * xe[c + 2];
      if (c + 3 < NB) acc3 += A[(size_t)(c + 3) * NB + r] * xe[c + 3];
    }
  } else {
#pragma unroll 4
    for (int c = 0; c < n; ++c) acc0 += A[(size_t)c * n + r] * xe[c];
  }
  return (acc0 + acc1) + (acc2 + acc3);
}

