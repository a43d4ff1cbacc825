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
  const EFace* eface;     // [E][F]
  const double* Minv;     // [E][Np]
  const double* w;        // [Np]
  const double* jac;      // [E][Np]
};

DevMesh dev_mesh(const eg_mesh* m);
int eg_launch_residual(eg_mesh* m, const double* q, double* res);
int eg_launch_split_element(eg_mesh* m, const double* q, double* res);
int eg_launch_norm(eg_mesh* m, const double* r, int strongres, double* out_dev);
