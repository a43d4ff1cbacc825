// euler_oracle.cpp -- CPU oracle for the Euler SBP hot path (FP64).
//
// TEST INFRASTRUCTURE: a plain restatement of PDESolver.jl's algorithm used to
// check libeulergpu.so.  Only tests/, __graft_entry__.smoke() and the CPU
// baseline leg of bench.py load it.
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
#include <cmath>
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

template <int DIM>
int eval_residual(const eg_mesh_desc* d, const eg_params* ep, const double* q, double* res) {
  View v(d);
  Params p = make_params(ep);
  const int nv = DIM + 2, Np = v.Np, Nf = v.Nf, S = v.S;
  const size_t ndof = (size_t)v.E * Np * nv;
  // dataPrep: fill!(res, 0) (euler.jl:455)
  std::memset(res, 0, ndof * sizeof(double));
  // checkDensity / checkPressure (euler.jl:543-611)
  for (int e = 0; e < v.E; ++e)
    for (int j = 0; j < Np; ++j) {
      const double* qj = q + ((size_t)e * Np + j) * nv;
      if (!(qj[0] > 0)) return EG_ERR_NEG_DENSITY;
      if (!(pressure<DIM>(p, qj) > 0)) return EG_ERR_NEG_PRESSURE;
    }
  // ---------------------------------------------------------------- volume
  if (ep->volume_integral_type == 1) {
    // getEulerFlux + weakdifferentiate!(trans=true): res_e += sum_k Q_k^T F_k
#pragma omp parallel for schedule(static)
    for (int e = 0; e < v.E; ++e) {
      std::vector<double> flux((size_t)DIM * Np * nv);
      for (int j = 0; j < Np; ++j) {
        const double* qj = q + ((size_t)e * Np + j) * nv;
        for (int k = 0; k < DIM; ++k) {
          double nrm[3];
          for (int pp = 0; pp < DIM; ++pp) nrm[pp] = v.dxidx(e, j, pp, k);
          euler_flux<DIM>(p, qj, nrm, &flux[((size_t)k * Np + j) * nv]);
        }
      }
      double* re = res + (size_t)e * Np * nv;
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
      double* re = res + (size_t)e * Np * nv;
      for (int j = 0; j < Np; ++j) {
        const double* qj = q + ((size_t)e * Np + j) * nv;
        for (int k = 0; k < j; ++k) {
          const double* qk = q + ((size_t)e * Np + k) * nv;
          double Fd[3 * 5];
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
      double fl[16][5];
      for (int i = 0; i < Nf; ++i) {
        double qf[5] = {0}, qg[5];
        for (int s = 0; s < S; ++s) {
          const double* qs = q + ((size_t)e * Np + v.perm(f, s)) * nv;
          for (int c = 0; c < nv; ++c) qf[c] += v.interp(f, i, s) * qs[c];
        }
        const double* x = d->coords_bndry + ((size_t)b * Nf + i) * DIM;
        const double* nrm = d->nrm_bndry + ((size_t)b * Nf + i) * DIM;
        boundary_state<DIM>(p, bc, x, qg);
        roe_solver<DIM>(p, qf, qg, nrm, fl[i]);
      }
      double* re = res + (size_t)e * Np * nv;
      for (int i = 0; i < Nf; ++i)
        for (int s = 0; s < S; ++s) {
          double c0 = v.interp(f, i, s) * d->wface[i];
          for (int c = 0; c < nv; ++c) re[v.perm(f, s) * nv + c] -= c0 * fl[i][c];
        }
    }
  }
  // ---------------------------------------------------------------- faces
  // interiorfaceinterpolate! + calcFaceFlux + interiorfaceintegrate!(Subtract)
  std::vector<double> fbuf((size_t)d->num_interfaces * Nf * nv);
#pragma omp parallel for schedule(static)
  for (int n = 0; n < d->num_interfaces; ++n) {
    const int32_t* itf = d->interfaces + 5 * n;
    int eL = itf[0], eR = itf[1], fL = itf[2], fR = itf[3], o = itf[4];
    double* fl = &fbuf[(size_t)n * Nf * nv];
    for (int i = 0; i < Nf; ++i) {
      int iR = v.nbrperm(o, i);
      double qL[5] = {0}, qR[5] = {0};
      for (int s = 0; s < S; ++s) {
        const double* a = q + ((size_t)eL * Np + v.perm(fL, s)) * nv;
        const double* b = q + ((size_t)eR * Np + v.perm(fR, s)) * nv;
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
    const double* fl = &fbuf[(size_t)n * Nf * nv];
    double* rL = res + (size_t)eL * Np * nv;
    double* rR = res + (size_t)eR * Np * nv;
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
  return d->dim == 2 ? eval_residual<2>(d, p, q, res) : eval_residual<3>(d, p, q, res);
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
