// euler_oracle.cpp -- CPU oracle for the Euler SBP hot path (FP64).
//
// TEST INFRASTRUCTURE: a plain restatement of PDESolver.jl's algorithm used to
// check libeulergpu.so.  Only tests/, __graft_entry__.smoke() and the CPU
// baseline leg of bench.py load it.
//
// Pin status: the point functions, split form, entropy identities, Jacobian
// and RK4 are pinned to the known answers and properties of the reference's
// own tests (tests/test_oracle.py cites each one).  The SBP operator entries
// come from SummationByParts.jl, which is absent: they are pinned by their
// defining properties only, so entry-wise parity with that package is
// unpinned.
//
// Residual: src/solver/euler/euler.jl:111-175 (evalResidual), 441-519
// (dataPrep), 628-690 (volume + boundary integrals), 770-802 (face integrals);
// src/solver/euler/euler_funcs.jl:23-66 (getEulerFlux), 240-362 (split form);
// src/solver/euler/flux.jl:37-64, 613-646 (face interpolation + flux);
// src/solver/euler/bc.jl:49-96, 162-288 (boundary fluxes);
// src/Utils/curvilinear.jl:17-41 (calcSCurvilinear).
// The SBP operator calls (weakdifferentiate!, interiorfaceinterpolate!,
// interiorfaceintegrate!, boundaryinterpolate!, boundaryintegrate!) belong to
// SummationByParts.jl, which is not vendored; they are restated from their
// call sites with the operator fields interp / perm / nbrperm / wface.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../include/eulergpu.h"
#include "euler_oracle.hpp"

using namespace oracle;

namespace {

Params make_params(const eg_params* ep) {
  Params p;
  p.gamma = ep->gamma;
  p.gamma_1 = ep->gamma - 1;
  p.Ma = ep->Ma;
  p.aoa = ep->aoa;
  p.rho_free = ep->rho_free;
  p.p_free = ep->p_free;
  p.E_free = ep->p_free / p.gamma_1 + 0.5 * ep->rho_free * ep->Ma * ep->Ma;
  p.r_in = ep->vortex_r_in;
  p.rho_in = ep->vortex_rho_in;
  p.M_in = ep->vortex_M_in;
  p.R = 287.058;  // read_input.jl:141 default
  p.cv = p.R / p.gamma_1;
  return p;
}

struct View {
  const eg_mesh_desc* m;
  int dim, E, Np, Nf, S, F, nv;
  explicit View(const eg_mesh_desc* d)
      : m(d), dim(d->dim), E(d->num_el), Np(d->nodes_per_el), Nf(d->nodes_per_face),
        S(d->stencil_size), F(d->dim + 1), nv(d->dim + 2) {}
  double Q(int k, int i, int j) const { return m->Q[((size_t)k * Np + j) * Np + i]; }
  double interp(int f, int i, int s) const { return m->interp[((size_t)f * Nf + i) * S + s]; }
  int perm(int f, int s) const { return m->perm[f * S + s]; }
  int nbrperm(int o, int i) const { return m->nbrperm[o * Nf + i]; }
  double dxidx(int e, int j, int p, int k) const {
    return m->dxidx[(((size_t)e * Np + j) * dim + p) * dim + k];
  }
};

template <int DIM>
void boundary_state(const Params& p, int bc, const double* x, double* qg) {
  if (bc == EG_BC_VORTEX) {
    isentropic_vortex(p, x, qg);
  } else {
    free_stream<DIM>(p, qg);
  }
}

template <int DIM, typename T>
int eval_residual(const eg_mesh_desc* d, const eg_params* ep, const T* q, T* res) {
  View v(d);
  Params p = make_params(ep);
  const int nv = DIM + 2, Np = v.Np, Nf = v.Nf, S = v.S;
  const size_t ndof = (size_t)v.E * Np * nv;
  // dataPrep: fill!(res, 0) (euler.jl:455)
  for (size_t i = 0; i < ndof; ++i) res[i] = T(0.0);
  // checkDensity / checkPressure (euler.jl:543-611)
  for (int e = 0; e < v.E; ++e)
    for (int j = 0; j < Np; ++j) {
      const T* qj = q + ((size_t)e * Np + j) * nv;
      if (!(real(qj[0]) > 0)) return EG_ERR_NEG_DENSITY;
      if (!(real(pressure<DIM>(p, qj)) > 0)) return EG_ERR_NEG_PRESSURE;
    }
  // ---------------------------------------------------------------- volume
  if (ep->volume_integral_type == 1) {
    // getEulerFlux + weakdifferentiate!(trans=true): res_e += sum_k Q_k^T F_k
#pragma omp parallel for schedule(static)
    for (int e = 0; e < v.E; ++e) {
      std::vector<T> flux((size_t)DIM * Np * nv);
      for (int j = 0; j < Np; ++j) {
        const T* qj = q + ((size_t)e * Np + j) * nv;
        for (int k = 0; k < DIM; ++k) {
          double nrm[3];
          for (int pp = 0; pp < DIM; ++pp) nrm[pp] = v.dxidx(e, j, pp, k);
          euler_flux<DIM>(p, qj, nrm, &flux[((size_t)k * Np + j) * nv]);
        }
      }
      T* re = res + (size_t)e * Np * nv;
      for (int k = 0; k < DIM; ++k)
        for (int i = 0; i < Np; ++i)
          for (int j = 0; j < Np; ++j) {
            double qji = v.Q(k, j, i);
            for (int c = 0; c < nv; ++c) re[i * nv + c] += qji * flux[((size_t)k * Np + j) * nv + c];
          }
    }
  } else {
    // calcVolumeIntegralsSplitFormCurvilinear (euler_funcs.jl:295-362)
    double nrmD[9] = {0};
    for (int dd = 0; dd < DIM; ++dd) nrmD[dd * DIM + dd] = 1.0;
#pragma omp parallel for schedule(static)
    for (int e = 0; e < v.E; ++e) {
      std::vector<double> Sx((size_t)DIM * Np * Np);
      // calcSCurvilinear (curvilinear.jl:17-41)
      std::fill(Sx.begin(), Sx.end(), 0.0);
      for (int d1 = 0; d1 < DIM; ++d1)
        for (int d2 = 0; d2 < DIM; ++d2)
          for (int i = 0; i < Np; ++i)
            for (int j = 0; j < i; ++j) {
              double& sji = Sx[((size_t)d1 * Np + j) * Np + i];
              sji += 0.5 * v.dxidx(e, j, d1, d2) * v.Q(d2, j, i) - 0.5 * v.dxidx(e, i, d1, d2) * v.Q(d2, i, j);
              Sx[((size_t)d1 * Np + i) * Np + j] = -sji;
            }
      T* re = res + (size_t)e * Np * nv;
      for (int j = 0; j < Np; ++j) {
        const T* qj = q + ((size_t)e * Np + j) * nv;
        for (int k = 0; k < j; ++k) {
          const T* qk = q + ((size_t)e * Np + k) * nv;
          T Fd[3 * 5];
          ir_flux<DIM>(p, qj, qk, nrmD, DIM, Fd);
          for (int dd = 0; dd < DIM; ++dd) {
            double s = Sx[((size_t)dd * Np + j) * Np + k];
            for (int c = 0; c < nv; ++c) {
              re[j * nv + c] -= 2 * s * Fd[dd * nv + c];
              re[k * nv + c] += 2 * s * Fd[dd * nv + c];
            }
          }
        }
      }
    }
  }
  // ---------------------------------------------------------------- boundary
  // interpolateBoundary + calcBoundaryFlux + boundaryintegrate!(Subtract)
  for (int g = 0; g < d->num_bc; ++g) {
    int bc = d->bc_types[g];
    for (int b = d->bndry_offsets[g]; b < d->bndry_offsets[g + 1]; ++b) {
      int e = d->bndryfaces[2 * b], f = d->bndryfaces[2 * b + 1];
      T fl[16][5];
      for (int i = 0; i < Nf; ++i) {
        T qf[5] = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)}, qgT[5];
        double qg[5];
        for (int s = 0; s < S; ++s) {
          const T* qs = q + ((size_t)e * Np + v.perm(f, s)) * nv;
          for (int c = 0; c < nv; ++c) qf[c] += v.interp(f, i, s) * qs[c];
        }
        const double* x = d->coords_bndry + ((size_t)b * Nf + i) * DIM;
        const double* nrm = d->nrm_bndry + ((size_t)b * Nf + i) * DIM;
        if (bc == EG_BC_NOPENETRATION_ES) {
          nopenetration_es_flux<DIM>(p, qf, nrm, fl[i]);
          continue;
        }
        boundary_state<DIM>(p, bc, x, qg);
        for (int c = 0; c < nv; ++c) qgT[c] = T(qg[c]);
        roe_solver<DIM>(p, qf, qgT, nrm, fl[i]);
      }
      T* re = res + (size_t)e * Np * nv;
      for (int i = 0; i < Nf; ++i)
        for (int s = 0; s < S; ++s) {
          double c0 = v.interp(f, i, s) * d->wface[i];
          for (int c = 0; c < nv; ++c) re[v.perm(f, s) * nv + c] -= c0 * fl[i][c];
        }
    }
  }
  // ---------------------------------------------------------------- faces
  // interiorfaceinterpolate! + calcFaceFlux + interiorfaceintegrate!(Subtract)
  std::vector<T> fbuf((size_t)d->num_interfaces * Nf * nv);
#pragma omp parallel for schedule(static)
  for (int n = 0; n < d->num_interfaces; ++n) {
    const int32_t* itf = d->interfaces + 5 * n;
    int eL = itf[0], eR = itf[1], fL = itf[2], fR = itf[3], o = itf[4];
    T* fl = &fbuf[(size_t)n * Nf * nv];
    for (int i = 0; i < Nf; ++i) {
      int iR = v.nbrperm(o, i);
      T qL[5] = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)}, qR[5] = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)};
      for (int s = 0; s < S; ++s) {
        const T* a = q + ((size_t)eL * Np + v.perm(fL, s)) * nv;
        const T* b = q + ((size_t)eR * Np + v.perm(fR, s)) * nv;
        for (int c = 0; c < nv; ++c) {
          qL[c] += v.interp(fL, i, s) * a[c];
          qR[c] += v.interp(fR, iR, s) * b[c];
        }
      }
      const double* nrm = d->nrm_face + ((size_t)n * Nf + i) * DIM;
      if (ep->face_flux == EG_FLUX_ROE)
        roe_solver<DIM>(p, qL, qR, nrm, fl + i * nv);
      else
        ir_flux<DIM>(p, qL, qR, nrm, 1, fl + i * nv);
    }
  }
  for (int n = 0; n < d->num_interfaces; ++n) {
    const int32_t* itf = d->interfaces + 5 * n;
    int eL = itf[0], eR = itf[1], fL = itf[2], fR = itf[3], o = itf[4];
    const T* fl = &fbuf[(size_t)n * Nf * nv];
    T* rL = res + (size_t)eL * Np * nv;
    T* rR = res + (size_t)eR * Np * nv;
    for (int i = 0; i < Nf; ++i) {
      int iR = v.nbrperm(o, i);
      for (int s = 0; s < S; ++s) {
        double cL = v.interp(fL, i, s) * d->wface[i];
        double cR = v.interp(fR, iR, s) * d->wface[i];
        for (int c = 0; c < nv; ++c) {
          rL[v.perm(fL, s) * nv + c] -= cL * fl[i * nv + c];
          rR[v.perm(fR, s) * nv + c] += cR * fl[i * nv + c];
        }
      }
    }
  }
  return EG_OK;
}

}  // namespace

extern "C" {

#ifdef _OPENMP
#include <omp.h>
#endif
// number of host threads the oracle uses (OpenMP); n <= 0 leaves the default
int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int oracle_eval_residual(const eg_mesh_desc* d, const eg_params* p, const double* q, double* res) {
  if (d->nodes_per_face > 16) return EG_ERR_UNSUPPORTED;
  return d->dim == 2 ? eval_residual<2, double>(d, p, q, res) : eval_residual<3, double>(d, p, q, res);
}

// directional derivative of the residual: jv = (dR/dq) v, via dual numbers
int oracle_residual_jvp(const eg_mesh_desc* d, const eg_params* p, const double* q,
                        const double* vdir, double* res, double* jv) {
  if (d->nodes_per_face > 16) return EG_ERR_UNSUPPORTED;
  const size_t n = (size_t)d->num_el * d->nodes_per_el * (d->dim + 2);
  std::vector<Dual<1>> qd(n), rd(n);
  for (size_t i = 0; i < n; ++i) {
    qd[i].v = q[i];
    qd[i].d[0] = vdir[i];
  }
  int st = d->dim == 2 ? eval_residual<2, Dual<1>>(d, p, qd.data(), rd.data())
                       : eval_residual<3, Dual<1>>(d, p, qd.data(), rd.data());
  for (size_t i = 0; i < n; ++i) {
    if (res) res[i] = rd[i].v;
    jv[i] = rd[i].d[0];
  }
  return st;
}

// ---- point functions for the known-answer tests ---------------------------
double oracle_pressure(const eg_params* ep, int dim, const double* q) {
  Params p = make_params(ep);
  return dim == 2 ? pressure<2>(p, q) : pressure<3>(p, q);
}

void oracle_euler_flux(const eg_params* ep, int dim, const double* q, const double* dir, double* F) {
  Params p = make_params(ep);
  if (dim == 2) euler_flux<2>(p, q, dir, F); else euler_flux<3>(p, q, dir, F);
}

void oracle_roe_flux(const eg_params* ep, int dim, const double* qL, const double* qR,
                     const double* nrm, double* F) {
  Params p = make_params(ep);
  if (dim == 2) roe_solver<2>(p, qL, qR, nrm, F); else roe_solver<3>(p, qL, qR, nrm, F);
}

void oracle_ir_flux(const eg_params* ep, int dim, const double* qL, const double* qR,
                    const double* dirs, int ndir, double* F) {
  Params p = make_params(ep);
  if (dim == 2) ir_flux<2>(p, qL, qR, dirs, ndir, F); else ir_flux<3>(p, qL, qR, dirs, ndir, F);
}

double oracle_logavg(double a, double b) { return logavg(a, b); }

// boundary flux of noPenetrationESBC at one face node (bc.jl:767-795)
void oracle_wall_es_flux(const eg_params* ep, int dim, const double* q, const double* nrm, double* F) {
  Params p = make_params(ep);
  if (dim == 2) nopenetration_es_flux<2>(p, q, nrm, F); else nopenetration_es_flux<3>(p, q, nrm, F);
}

void oracle_lf_flux(const eg_params* ep, int dim, const double* qL, const double* qR, const double* nrm,
                    double* F) {
  Params p = make_params(ep);
  if (dim == 2) lf_flux<2>(p, qL, qR, nrm, F); else lf_flux<3>(p, qL, qR, nrm, F);
}

// d logavg / d(aL, aR) by forward-mode dual numbers (the derivative that the
// Jacobian assembly uses; logavg_diff, bc_solvers_diff.jl:5644-5716)
void oracle_logavg_diff(double a, double b, double* dL_da, double* dL_db) {
  Dual<2> x(a), y(b);
  x.d[0] = 1.0;
  y.d[1] = 1.0;
  Dual<2> L = logavg(x, y);
  *dL_da = L.d[0];
  *dL_db = L.d[1];
}

void oracle_vortex(const eg_params* ep, const double* x, double* q) {
  Params p = make_params(ep);
  isentropic_vortex(p, x, q);
}

void oracle_free_stream(const eg_params* ep, int dim, double* q) {
  Params p = make_params(ep);
  if (dim == 2) free_stream<2>(p, q); else free_stream<3>(p, q);
}

// calcNorm (Utils.jl:427-449) over a [E][Np][nv] vector with M = w/jac
double oracle_calc_norm(const eg_mesh_desc* d, const double* r, int strongres) {
  const int nv = d->dim + 2, Np = d->nodes_per_el;
  double val = 0;
  for (int e = 0; e < d->num_el; ++e)
    for (int j = 0; j < Np; ++j) {
      double M = d->w[j] / d->jac[(size_t)e * Np + j];
      double fac = strongres ? 1.0 / M : M;
      for (int c = 0; c < nv; ++c) {
        double x = r[((size_t)e * Np + j) * nv + c];
        val += x * fac * x;
      }
    }
  return std::sqrt(val);
}

}  // extern "C"

// ===========================================================================
// Explicit Jacobian, block-Jacobi + GMRES, Newton, RK4, boundary functional.
// ===========================================================================
namespace {

// Element-block Jacobian (same storage as the GPU library, see eulergpu.h):
// volume blocks from calcVolumeIntegrals_nopre_diff (euler_funcs_diff.jl:54-103),
// face blocks from calcFaceIntegral_nopre_diff / interiorFaceCombined_jac!
// (flux_diff.jl:6-100), boundary blocks from getBCFluxes_diff (bc_diff.jl:16-212).
// Point flux Jacobians use forward-mode dual numbers.
template <int DIM>
int eval_jacobian(const eg_mesh_desc* d, const eg_params* ep, const double* q, double* diag,
                  double* cpl) {
  constexpr int NV = DIM + 2;
  View v(d);
  Params p = make_params(ep);
  const int Np = v.Np, Nf = v.Nf, S = v.S, n = Np * NV, nb = S * NV;
  std::memset(diag, 0, sizeof(double) * (size_t)v.E * n * n);
  if (cpl) std::memset(cpl, 0, sizeof(double) * (size_t)d->num_interfaces * 2 * nb * nb);
  if (ep->volume_integral_type == 2) {
    // split form: the pair terms of calcVolumeIntegralsSplitFormCurvilinear
    // (euler_funcs.jl:295-362) differentiated pair by pair, as
    // calcVolumeIntegralsSplitFormCurvilinear_diff does (euler_funcs_diff.jl:
    // 330-430): res_j -= 2 S_x[j,k,:] F_IR(q_j, q_k), res_k += the same
    double nrmD[9] = {0};
    for (int dd = 0; dd < DIM; ++dd) nrmD[dd * DIM + dd] = 1.0;
#pragma omp parallel for schedule(static)
    for (int e = 0; e < v.E; ++e) {
      std::vector<double> Sx((size_t)DIM * Np * Np, 0.0);
      for (int d1 = 0; d1 < DIM; ++d1)
        for (int d2 = 0; d2 < DIM; ++d2)
          for (int i = 0; i < Np; ++i)
            for (int j = 0; j < i; ++j) {
              double& sji = Sx[((size_t)d1 * Np + j) * Np + i];
              sji += 0.5 * v.dxidx(e, j, d1, d2) * v.Q(d2, j, i) - 0.5 * v.dxidx(e, i, d1, d2) * v.Q(d2, i, j);
              Sx[((size_t)d1 * Np + i) * Np + j] = -sji;
            }
      double* D = diag + (size_t)e * n * n;
      for (int j = 0; j < Np; ++j)
        for (int k = 0; k < j; ++k) {
          Dual<2 * NV> qj[NV], qk[NV], Fd[3 * NV];
          for (int c = 0; c < NV; ++c) {
            qj[c] = Dual<2 * NV>(q[((size_t)e * Np + j) * NV + c]);
            qk[c] = Dual<2 * NV>(q[((size_t)e * Np + k) * NV + c]);
            qj[c].d[c] = 1.0;
            qk[c].d[NV + c] = 1.0;
          }
          ir_flux<DIM>(p, qj, qk, nrmD, DIM, Fd);
          for (int dd = 0; dd < DIM; ++dd) {
            const double s2 = 2 * Sx[((size_t)dd * Np + j) * Np + k];
            for (int a = 0; a < NV; ++a)
              for (int b = 0; b < NV; ++b) {
                const double gj = s2 * Fd[dd * NV + a].d[b], gk = s2 * Fd[dd * NV + a].d[NV + b];
                D[(size_t)(j * NV + b) * n + j * NV + a] -= gj;
                D[(size_t)(k * NV + b) * n + j * NV + a] -= gk;
                D[(size_t)(j * NV + b) * n + k * NV + a] += gj;
                D[(size_t)(k * NV + b) * n + k * NV + a] += gk;
              }
          }
        }
    }
  }
  // volume (weak form)
#pragma omp parallel for schedule(static)
  for (int e = 0; e < v.E; ++e) {
    if (ep->volume_integral_type == 2) continue;
    std::vector<double> A((size_t)DIM * Np * NV * NV);
    for (int m = 0; m < Np; ++m)
      for (int k = 0; k < DIM; ++k) {
        Dual<NV> qm[NV], F[NV];
        for (int c = 0; c < NV; ++c) {
          qm[c] = Dual<NV>(q[((size_t)e * Np + m) * NV + c]);
          qm[c].d[c] = 1.0;
        }
        double dir[3];
        for (int pp = 0; pp < DIM; ++pp) dir[pp] = v.dxidx(e, m, pp, k);
        euler_flux<DIM>(p, qm, dir, F);
        for (int a = 0; a < NV; ++a)
          for (int b = 0; b < NV; ++b) A[(((size_t)k * Np + m) * NV + a) * NV + b] = F[a].d[b];
      }
    double* D = diag + (size_t)e * n * n;
    for (int j = 0; j < Np; ++j)
      for (int m = 0; m < Np; ++m)
        for (int k = 0; k < DIM; ++k) {
          const double qmj = v.Q(k, m, j);
          for (int a = 0; a < NV; ++a)
            for (int b = 0; b < NV; ++b)
              D[(size_t)(m * NV + b) * n + j * NV + a] += qmj * A[(((size_t)k * Np + m) * NV + a) * NV + b];
        }
  }
  // boundary faces: rows/cols on the face stencil, -R^T W dF/dq R
  for (int b = 0; b < d->num_bndry; ++b) {
    int g = 0;
    while (b >= d->bndry_offsets[g + 1]) ++g;
    const int bc = d->bc_types[g];
    const int e = d->bndryfaces[2 * b], f = d->bndryfaces[2 * b + 1];
    double* D = diag + (size_t)e * n * n;
    for (int i = 0; i < Nf; ++i) {
      Dual<NV> qf[NV], qgD[NV], fl[NV];
      for (int c = 0; c < NV; ++c) qf[c] = Dual<NV>(0.0);
      for (int s = 0; s < S; ++s)
        for (int c = 0; c < NV; ++c) qf[c].v += v.interp(f, i, s) * q[((size_t)e * Np + v.perm(f, s)) * NV + c];
      for (int c = 0; c < NV; ++c) qf[c].d[c] = 1.0;
      if (bc == EG_BC_NOPENETRATION_ES) {
        // the mirror state follows q: differentiated through it
        nopenetration_es_flux<DIM>(p, qf, d->nrm_bndry + ((size_t)b * Nf + i) * DIM, fl);
      } else {
        double qg[5];
        boundary_state<DIM>(p, bc, d->coords_bndry + ((size_t)b * Nf + i) * DIM, qg);
        for (int c = 0; c < NV; ++c) qgD[c] = Dual<NV>(qg[c]);
        roe_solver<DIM>(p, qf, qgD, d->nrm_bndry + ((size_t)b * Nf + i) * DIM, fl);
      }
      for (int s = 0; s < S; ++s)
        for (int sp = 0; sp < S; ++sp) {
          const double c0 = v.interp(f, i, s) * d->wface[i] * v.interp(f, i, sp);
          const int jr = v.perm(f, s), mc = v.perm(f, sp);
          for (int a = 0; a < NV; ++a)
            for (int bb = 0; bb < NV; ++bb) D[(size_t)(mc * NV + bb) * n + jr * NV + a] -= c0 * fl[a].d[bb];
        }
    }
  }
  // interfaces
  for (int nI = 0; nI < d->num_interfaces; ++nI) {
    const int32_t* itf = d->interfaces + 5 * nI;
    const int eL = itf[0], eR = itf[1], fL = itf[2], fR = itf[3], o = itf[4];
    double* DL = diag + (size_t)eL * n * n;
    double* DR = diag + (size_t)eR * n * n;
    double* CLR = cpl ? cpl + ((size_t)nI * 2 + 0) * nb * nb : nullptr;
    double* CRL = cpl ? cpl + ((size_t)nI * 2 + 1) * nb * nb : nullptr;
    for (int i = 0; i < Nf; ++i) {
      const int iR = v.nbrperm(o, i);
      Dual<2 * NV> qL[NV], qR[NV], fl[NV];
      for (int c = 0; c < NV; ++c) {
        qL[c] = Dual<2 * NV>(0.0);
        qR[c] = Dual<2 * NV>(0.0);
      }
      for (int s = 0; s < S; ++s)
        for (int c = 0; c < NV; ++c) {
          qL[c].v += v.interp(fL, i, s) * q[((size_t)eL * Np + v.perm(fL, s)) * NV + c];
          qR[c].v += v.interp(fR, iR, s) * q[((size_t)eR * Np + v.perm(fR, s)) * NV + c];
        }
      for (int c = 0; c < NV; ++c) {
        qL[c].d[c] = 1.0;
        qR[c].d[NV + c] = 1.0;
      }
      const double* nrm = d->nrm_face + ((size_t)nI * Nf + i) * DIM;
      if (ep->face_flux == EG_FLUX_ROE)
        roe_solver<DIM>(p, qL, qR, nrm, fl);
      else
        ir_flux<DIM>(p, qL, qR, nrm, 1, fl);
      const double w = d->wface[i];
      for (int s = 0; s < S; ++s)
        for (int sp = 0; sp < S; ++sp) {
          const double lL = v.interp(fL, i, s) * w, lR = v.interp(fR, iR, s) * w;
          const double rL = v.interp(fL, i, sp), rR = v.interp(fR, iR, sp);
          for (int a = 0; a < NV; ++a)
            for (int b = 0; b < NV; ++b) {
              const double dl = fl[a].d[b], dr = fl[a].d[NV + b];
              DL[(size_t)(v.perm(fL, sp) * NV + b) * n + v.perm(fL, s) * NV + a] -= lL * rL * dl;
              DR[(size_t)(v.perm(fR, sp) * NV + b) * n + v.perm(fR, s) * NV + a] += lR * rR * dr;
              if (CLR) CLR[(size_t)(sp * NV + b) * nb + s * NV + a] -= lL * rR * dr;
              if (CRL) CRL[(size_t)(sp * NV + b) * nb + s * NV + a] += lR * rL * dl;
            }
        }
    }
  }
  return EG_OK;
}

// y = J x for the element-block storage
void jac_apply(const eg_mesh_desc* d, int n, int nb, const double* diag, const double* cpl,
               const double* x, double* y) {
  const int NV = d->dim + 2, S = d->stencil_size, Np = d->nodes_per_el;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < d->num_el; ++e) {
    const double* D = diag + (size_t)e * n * n;
    for (int r = 0; r < n; ++r) {
      double acc = 0;
      for (int c = 0; c < n; ++c) acc += D[(size_t)c * n + r] * x[(size_t)e * n + c];
      y[(size_t)e * n + r] = acc;
    }
  }
  (void)Np;
  // the coupling terms of every interface, computed in parallel, then added
  // to y in interface order (the sums of a serial loop, bit for bit)
  const int I = d->num_interfaces;
  std::vector<double> t((size_t)I * 2 * nb);
#pragma omp parallel for schedule(static)
  for (int nI = 0; nI < I; ++nI) {
    const int32_t* itf = d->interfaces + 5 * nI;
    const int eL = itf[0], eR = itf[1], fL = itf[2], fR = itf[3];
    const double* CLR = cpl + ((size_t)nI * 2 + 0) * nb * nb;
    const double* CRL = cpl + ((size_t)nI * 2 + 1) * nb * nb;
    double* tL = &t[((size_t)nI * 2 + 0) * nb];
    double* tR = &t[((size_t)nI * 2 + 1) * nb];
    for (int s = 0; s < S; ++s)
      for (int a = 0; a < NV; ++a) {
        double aL = 0, aR = 0;
        for (int sp = 0; sp < S; ++sp)
          for (int b = 0; b < NV; ++b) {
            aL += CLR[(size_t)(sp * NV + b) * nb + s * NV + a] *
                  x[(size_t)eR * n + d->perm[fR * S + sp] * NV + b];
            aR += CRL[(size_t)(sp * NV + b) * nb + s * NV + a] *
                  x[(size_t)eL * n + d->perm[fL * S + sp] * NV + b];
          }
        tL[s * NV + a] = aL;
        tR[s * NV + a] = aR;
      }
  }
  for (int nI = 0; nI < I; ++nI) {
    const int32_t* itf = d->interfaces + 5 * nI;
    const int eL = itf[0], eR = itf[1], fL = itf[2], fR = itf[3];
    const double* tL = &t[((size_t)nI * 2 + 0) * nb];
    const double* tR = &t[((size_t)nI * 2 + 1) * nb];
    for (int s = 0; s < S; ++s)
      for (int a = 0; a < NV; ++a) {
        y[(size_t)eL * n + d->perm[fL * S + s] * NV + a] += tL[s * NV + a];
        y[(size_t)eR * n + d->perm[fR * S + s] * NV + a] += tR[s * NV + a];
      }
  }
}

// LU with partial pivoting of every element block (reference
// preconditioning.jl:62-74, getrf!) and the matching solve (getrs)
struct BlockLU {
  int n = 0;
  std::vector<double> lu;
  std::vector<int> piv;
  bool factor(const eg_mesh_desc* d, const double* diag, int nn) {
    n = nn;
    const int E = d->num_el;
    lu.assign(diag, diag + (size_t)E * n * n);
    piv.assign((size_t)E * n, 0);
    bool ok = true;
#pragma omp parallel for schedule(static) reduction(&& : ok)
    for (int e = 0; e < E; ++e) {
      double* A = &lu[(size_t)e * n * n];  // column-major A[c*n + r]
      int* P = &piv[(size_t)e * n];
      for (int k = 0; k < n; ++k) {
        int p = k;
        double best = std::fabs(A[(size_t)k * n + k]);
        for (int i = k + 1; i < n; ++i)
          if (std::fabs(A[(size_t)k * n + i]) > best) { best = std::fabs(A[(size_t)k * n + i]); p = i; }
        P[k] = p;
        if (best == 0.0) { ok = false; continue; }
        if (p != k)
          for (int c = 0; c < n; ++c) std::swap(A[(size_t)c * n + k], A[(size_t)c * n + p]);
        const double dinv = 1.0 / A[(size_t)k * n + k];
        for (int i = k + 1; i < n; ++i) A[(size_t)k * n + i] *= dinv;
        for (int c = k + 1; c < n; ++c) {
          const double akc = A[(size_t)c * n + k];
          for (int i = k + 1; i < n; ++i) A[(size_t)c * n + i] -= A[(size_t)k * n + i] * akc;
        }
      }
    }
    return ok;
  }
  void solve(const eg_mesh_desc* d, const double* x, double* y) const {
#pragma omp parallel for schedule(static)
    for (int e = 0; e < d->num_el; ++e) {
      const double* A = &lu[(size_t)e * n * n];
      const int* P = &piv[(size_t)e * n];
      double* ye = y + (size_t)e * n;
      for (int i = 0; i < n; ++i) ye[i] = x[(size_t)e * n + i];
      for (int k = 0; k < n; ++k)
        if (P[k] != k) std::swap(ye[k], ye[P[k]]);
      for (int c = 0; c < n; ++c)
        for (int i = c + 1; i < n; ++i) ye[i] -= A[(size_t)c * n + i] * ye[c];
      for (int c = n - 1; c >= 0; --c) {
        ye[c] /= A[(size_t)c * n + c];
        for (int i = 0; i < c; ++i) ye[i] -= A[(size_t)c * n + i] * ye[c];
      }
    }
  }
};

// sum of a[i] b[i]: partial sums over fixed chunks of 8192 (in parallel),
// then over the chunks in order, so the result does not depend on the
// number of threads
double dot(const std::vector<double>& a, const std::vector<double>& b) {
  constexpr size_t kChunk = 8192;
  const size_t N = a.size();
  const long nc = (long)((N + kChunk - 1) / kChunk);
  std::vector<double> part(nc);
#pragma omp parallel for schedule(static)
  for (long c = 0; c < nc; ++c) {
    double s = 0;
    const size_t hi = std::min(N, (size_t)(c + 1) * kChunk);
    for (size_t i = (size_t)c * kChunk; i < hi; ++i) s += a[i] * b[i];
    part[c] = s;
  }
  double s = 0;
  for (long c = 0; c < nc; ++c) s += part[c];
  return s;
}

// right-preconditioned GMRES(m) with modified Gram-Schmidt (Saad, Iterative
// Methods for Sparse Linear Systems, alg. 9.5); the reference's PETSc KSP
// options (read_input.jl:559-569): GMRES(30), right PC, MGS.
int gmres(const eg_mesh_desc* d, int n, int nb, const double* diag, const double* cpl,
          const BlockLU& pc, const std::vector<double>& b, std::vector<double>& x, int m,
          double reltol, double abstol, int itermax, int* iters_out, bool* conv_out = nullptr) {
  const size_t N = b.size();
  std::vector<std::vector<double>> V(m + 1, std::vector<double>(N));
  std::vector<double> w(N), z(N);
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
  const double bnorm = std::sqrt(dot(b, b));
  const double tol = std::max(reltol * bnorm, abstol);
  int its = 0;
  while (true) {
    jac_apply(d, n, nb, diag, cpl, x.data(), w.data());
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)N; ++i) w[i] = b[i] - w[i];
    const double beta = std::sqrt(dot(w, w));
    if (conv_out) *conv_out = !(beta > tol);
    if (!(beta > tol) || its >= itermax) break;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)N; ++i) V[0][i] = w[i] / beta;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    double resid = beta;
    for (; j < m && its < itermax; ++j) {
      ++its;
      pc.solve(d, V[j].data(), z.data());
      jac_apply(d, n, nb, diag, cpl, z.data(), w.data());
      double* Hc = &H[(size_t)j * (m + 1)];
      for (int k = 0; k <= j; ++k) {
        Hc[k] = dot(V[k], w);
        const double hk = Hc[k];
        const double* vk = V[k].data();
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)N; ++i) w[i] -= hk * vk[i];
      }
      Hc[j + 1] = std::sqrt(dot(w, w));
      if (Hc[j + 1] > 0) {
        const double hn = Hc[j + 1];
        double* vn = V[j + 1].data();
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)N; ++i) vn[i] = w[i] / hn;
      }
      for (int k = 0; k < j; ++k) {
        const double t0 = cs[k] * Hc[k] + sn[k] * Hc[k + 1];
        Hc[k + 1] = -sn[k] * Hc[k] + cs[k] * Hc[k + 1];
        Hc[k] = t0;
      }
      const double den = std::hypot(Hc[j], Hc[j + 1]);
      cs[j] = Hc[j] / den;
      sn[j] = Hc[j + 1] / den;
      Hc[j] = den;
      Hc[j + 1] = 0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      resid = std::fabs(g[j + 1]);
      if (resid <= tol) { ++j; break; }
    }
    for (int k = j - 1; k >= 0; --k) {
      double s = g[k];
      for (int c = k + 1; c < j; ++c) s -= H[(size_t)c * (m + 1) + k] * y[c];
      y[k] = s / H[(size_t)k * (m + 1) + k];
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)N; ++i) {
      double acc = 0.0;
      for (int k = 0; k < j; ++k) acc += y[k] * V[k][i];
      w[i] = acc;
    }
    pc.solve(d, w.data(), z.data());
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)N; ++i) x[i] += z[i];
  }
  if (iters_out) *iters_out = its;
  return EG_OK;
}

// largest factor by which the pseudo-time step may grow in one iteration
constexpr double PTC_MAX_GROWTH = 1.5;
// a pseudo-time step that raises |R| by more than this factor is rejected
constexpr double PTC_MAX_INCREASE = 10.0;
// a step whose Krylov solve did not converge and that leaves |R| above this
// fraction of its previous value shrinks the pseudo-time step 4x
constexpr double PTC_STALL = 0.5;

double strong_norm(const eg_mesh_desc* d, const double* r) {
  const int nv = d->dim + 2, Np = d->nodes_per_el;
  double val = 0;
  for (int e = 0; e < d->num_el; ++e)
    for (int j = 0; j < Np; ++j) {
      const double minv = d->jac[(size_t)e * Np + j] / d->w[j];
      for (int c = 0; c < nv; ++c) {
        const double x = r[((size_t)e * Np + j) * nv + c];
        val += x * minv * x;
      }
    }
  return std::sqrt(val);
}

}  // namespace

extern "C" {

int oracle_eval_jacobian(const eg_mesh_desc* d, const eg_params* p, const double* q, double* diag,
                         double* cpl) {
  return d->dim == 2 ? eval_jacobian<2>(d, p, q, diag, cpl) : eval_jacobian<3>(d, p, q, diag, cpl);
}

// newton / newtonInner (newton.jl:137-304): FP64 Jacobian, element
// block-Jacobi LU, GMRES(restart) to krylov_reltol, q += dq, checkConvergence.
int oracle_newton(const eg_mesh_desc* d, const eg_params* p, double* q, const eg_newton_opts* o,
                  eg_newton_stats* stats) {
  const int NV = d->dim + 2, n = d->nodes_per_el * NV, nb = d->stencil_size * NV;
  const size_t N = (size_t)d->num_el * n;
  std::vector<double> res(N), diag((size_t)d->num_el * n * n),
      cpl((size_t)d->num_interfaces * 2 * nb * nb), b(N), dq(N);
  eg_newton_stats s;
  std::memset(&s, 0, sizeof(s));
  int st = oracle_eval_residual(d, p, q, res.data());
  if (st != EG_OK) return st;
  double norm = strong_norm(d, res.data());
  s.res_norm0 = s.res_norm = norm;
  const double rel = norm;
  bool conv = norm < o->res_abstol;
  BlockLU lu;
  // pseudo-transient continuation (globalization.jl:165-320): tau_l scaled by
  // |R|_{i-1}/|R|_i before every Jacobian after the first (growth capped at
  // euler_tau_growth per iteration); J -= M / tau_vec.  A step that leaves a
  // non-physical state (rho <= 0, p <= 0, non-finite R) is rejected: q is
  // restored and tau_l is divided by 4 (recovery not in the reference).
  double tau_l = o->euler_tau, norm_prev = 0.0;
  std::vector<double> qsave(q, q + N);
  for (int it = 1; !conv && it <= o->itermax; ++it) {
    oracle_eval_jacobian(d, p, q, diag.data(), cpl.data());
    if (o->globalize_euler) {
      if (norm_prev != 0.0) tau_l *= std::min(norm_prev / norm, PTC_MAX_GROWTH);
      norm_prev = norm;
      const int Np = d->nodes_per_el;
      for (int e = 0; e < d->num_el; ++e)
        for (int j = 0; j < Np; ++j) {
          const double jac = d->jac[(size_t)e * Np + j];
          const double M = d->w[j] / jac;
          const double tau_vec = tau_l / (1 + std::sqrt(jac));
          for (int a = 0; a < NV; ++a) {
            const int r = j * NV + a;
            diag[(size_t)e * n * n + (size_t)r * n + r] -= M / tau_vec;
          }
        }
    }
    if (!lu.factor(d, diag.data(), n)) return EG_ERR_LU_PIVOT;
    for (size_t i = 0; i < N; ++i) { b[i] = -res[i]; dq[i] = 0; }
    int its = 0;
    bool kconv = false;
    gmres(d, n, nb, diag.data(), cpl.data(), lu, b, dq, o->gmres_restart > 0 ? o->gmres_restart : 30,
          o->krylov_reltol, 1e-30, o->krylov_itermax > 0 ? o->krylov_itermax : 1000, &its, &kconv);
    s.krylov_iters += its;
    double sn2 = 0;
    for (size_t i = 0; i < N; ++i) { qsave[i] = q[i]; q[i] += dq[i]; sn2 += dq[i] * dq[i]; }
    s.step_norm = std::sqrt(sn2);
    st = oracle_eval_residual(d, p, q, res.data());
    s.iters = it;
    double nn = st == EG_OK ? strong_norm(d, res.data()) : NAN;
    if (std::getenv("ORACLE_VERBOSE"))
      std::fprintf(stderr, "newton %3d |R| %.3e -> %.3e tau %.3e krylov %d st %d\n", it, norm, nn, tau_l, its, st);
    if (st != EG_OK || !std::isfinite(nn) || (o->globalize_euler && nn > PTC_MAX_INCREASE * norm)) {
      if (!o->globalize_euler) {
        if (stats) *stats = s;
        return st != EG_OK ? st : EG_ERR_NONFINITE;
      }
      for (size_t i = 0; i < N; ++i) q[i] = qsave[i];
      oracle_eval_residual(d, p, q, res.data());
      tau_l *= 0.25;
      norm_prev = 0.0;   // no SER update right after a rejection
      continue;
    }
    // the Krylov solve hit its iteration limit and the step gained little:
    // keep the step, shrink the pseudo-time step (PTC_STALL)
    const bool stalled = o->globalize_euler && !kconv && nn > PTC_STALL * norm;
    norm = nn;
    s.res_norm = norm;
    conv = norm < o->res_abstol || norm / rel < o->res_reltol || s.step_norm <= o->step_tol;
    if (stalled && !conv) {
      tau_l *= 0.25;
      norm_prev = 0.0;
    }
  }
  s.converged = conv;
  if (stats) *stats = s;
  return conv ? EG_OK : EG_ERR_NOT_CONVERGED;
}

// rk4 (rk4.jl:144-336, 425-456) with res_vec = M^-1 R
int oracle_rk4(const eg_mesh_desc* d, const eg_params* p, double* q, double h, double t_max,
               int itermax, double res_tol, eg_rk4_stats* stats) {
  const int NV = d->dim + 2, Np = d->nodes_per_el;
  const size_t N = (size_t)d->num_el * Np * NV;
  std::vector<double> xold(q, q + N), k1(N), k2(N), k3(N), k4(N), res(N), minv(N);
  for (int e = 0; e < d->num_el; ++e)
    for (int j = 0; j < Np; ++j)
      for (int c = 0; c < NV; ++c)
        minv[((size_t)e * Np + j) * NV + c] = 1.0 / (d->w[j] / d->jac[(size_t)e * Np + j]);
  const long t_steps = std::lround(t_max / h);
  double t = 0, sol_norm = 0;
  int steps = 0;
  auto f = [&](std::vector<double>& k) -> int {
    int st = oracle_eval_residual(d, p, q, res.data());
    for (size_t i = 0; i < N; ++i) k[i] = minv[i] * res[i];
    return st;
  };
  for (long i = 2; i <= t_steps + 1; ++i) {
    t = (i - 2) * h;
    int st = f(k1);
    if (st != EG_OK) return st;
    // calcNorm(eqn, res_vec) with M weights
    double val = 0;
    for (size_t j = 0; j < N; ++j) val += k1[j] * (1.0 / minv[j]) * k1[j];
    sol_norm = std::sqrt(val);
    for (size_t j = 0; j < N; ++j) q[j] = xold[j] + (h / 2) * k1[j];
    if (res_tol > 0 && sol_norm < res_tol) break;
    if (itermax > 0 && i > itermax) break;
    if ((st = f(k2)) != EG_OK) return st;
    for (size_t j = 0; j < N; ++j) q[j] = xold[j] + (h / 2) * k2[j];
    if ((st = f(k3)) != EG_OK) return st;
    for (size_t j = 0; j < N; ++j) q[j] = xold[j] + h * k3[j];
    if ((st = f(k4)) != EG_OK) return st;
    for (size_t j = 0; j < N; ++j) {
      xold[j] = xold[j] + (h / 6) * (k1[j] + 2 * k2[j] + 2 * k3[j] + k4[j]);
      q[j] = xold[j];
    }
    ++steps;
  }
  t += h;
  if (stats) {
    stats->steps = steps;
    stats->t = t;
    stats->res_norm = sol_norm;
  }
  return EG_OK;
}

// integral of the pressure over the boundary faces of BC group `group`:
// sum_b sum_i wface_i p(q_face_i) |nrm_bndry_i|, with q_face interpolated by
// the SBP face operator (reference integratefunctional!, boundary_functional.jl:82-126)
double oracle_functional_pressure(const eg_mesh_desc* d, const eg_params* ep, const double* q, int group) {
  Params p = make_params(ep);
  View v(d);
  const int NV = d->dim + 2, Nf = v.Nf, S = v.S, Np = v.Np, dim = d->dim;
  double val = 0;
  for (int b = d->bndry_offsets[group]; b < d->bndry_offsets[group + 1]; ++b) {
    const int e = d->bndryfaces[2 * b], f = d->bndryfaces[2 * b + 1];
    for (int i = 0; i < Nf; ++i) {
      double qf[5] = {0, 0, 0, 0, 0};
      for (int s = 0; s < S; ++s)
        for (int c = 0; c < NV; ++c) qf[c] += v.interp(f, i, s) * q[((size_t)e * Np + v.perm(f, s)) * NV + c];
      const double* nr = d->nrm_bndry + ((size_t)b * Nf + i) * dim;
      double a2 = 0;
      for (int k = 0; k < dim; ++k) a2 += nr[k] * nr[k];
      const double pr = dim == 2 ? pressure<2>(p, qf) : pressure<3>(p, qf);
      val += d->wface[i] * pr * std::sqrt(a2);
    }
  }
  return val;
}

}  // extern "C"

extern "C" {
// Per-phase host times of one Newton iteration of the oracle (test
// infrastructure, used for a bounded CPU baseline sample): out[0] residual,
// out[1] Jacobian, out[2] block LU factorisation, out[3] one GMRES iteration
// (averaged over n_gmres iterations of GMRES(30)), all in seconds.
int oracle_newton_phase_times(const eg_mesh_desc* d, const eg_params* p, const double* q,
                              int n_gmres, double* out) {
  using clk = std::chrono::steady_clock;
  const int NV = d->dim + 2, n = d->nodes_per_el * NV, nb = d->stencil_size * NV;
  const size_t N = (size_t)d->num_el * n;
  std::vector<double> res(N), diag((size_t)d->num_el * n * n),
      cpl((size_t)d->num_interfaces * 2 * nb * nb), b(N), x(N, 0.0);
  auto t0 = clk::now();
  int st = oracle_eval_residual(d, p, q, res.data());
  if (st != EG_OK) return st;
  auto t1 = clk::now();
  oracle_eval_jacobian(d, p, q, diag.data(), cpl.data());
  auto t2 = clk::now();
  BlockLU lu;
  if (!lu.factor(d, diag.data(), n)) return EG_ERR_LU_PIVOT;
  auto t3 = clk::now();
  for (size_t i = 0; i < N; ++i) b[i] = -res[i];
  int its = 0;
  // GMRES(30) cycles, as in the timed solve: the per-iteration cost of the
  // Gram-Schmidt pass grows with the restart length
  gmres(d, n, nb, diag.data(), cpl.data(), lu, b, x, std::min(30, std::max(n_gmres, 1)), 1e-30, 0.0,
        n_gmres, &its);
  auto t4 = clk::now();
  out[0] = std::chrono::duration<double>(t1 - t0).count();
  out[1] = std::chrono::duration<double>(t2 - t1).count();
  out[2] = std::chrono::duration<double>(t3 - t2).count();
  out[3] = std::chrono::duration<double>(t4 - t3).count() / std::max(its, 1);
  return EG_OK;
}
}  // extern "C"
