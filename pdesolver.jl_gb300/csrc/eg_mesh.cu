// eg_mesh.cu -- mesh/equation object creation (reference createObjects,
// src/solver/euler/startup_func.jl:45): validates the caller's mesh and SBP
// arrays, uploads them, and builds the device-side tables the kernels use.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "eg_internal.h"

static thread_local char g_err[512] = "";

void eg_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int eg_cuda_fail(cudaError_t e, const char* what) {
  eg_set_error("%s: %s", what, cudaGetErrorString(e));
  // the error is reported through the status code: clear it from the
  // thread's last-error slot (a launch-configuration error is not sticky and
  // would otherwise surface in the caller's next, unrelated CUDA call)
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? EG_ERR_OOM : EG_ERR_CUDA;
}

extern "C" int eg_version(void) { return 1; }
extern "C" const char* eg_last_error(void) { return g_err; }

template <typename T>
static int upload(T** dst, const T* src, size_t n, const char* name) {
  *dst = nullptr;
  if (n == 0) return EG_OK;
  if (!src) {
    eg_set_error("eg_mesh_create: %s is NULL", name);
    return EG_ERR_INVALID;
  }
  EG_CUDA(cudaMalloc((void**)dst, n * sizeof(T)));
  EG_CUDA(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return EG_OK;
}

template <typename T>
static int alloc(T** dst, size_t n) {
  *dst = nullptr;
  if (n == 0) return EG_OK;
  EG_CUDA(cudaMalloc((void**)dst, n * sizeof(T)));
  return EG_OK;
}

// Dirichlet states of the weak boundary conditions (host, FP64).  Both are
// time-independent, so they are evaluated once per mesh.
// isentropic vortex: reference src/solver/euler/common_funcs.jl:25-79
static void vortex_state(const DevParams& p, const double* x, double* sol) {
  double gamma = p.gamma;
  double r = std::sqrt(x[0] * x[0] + x[1] * x[1]);
  double theta = std::atan2(x[1], x[0]);
  double tmp1 = ((gamma - 1) / 2) * p.M_in * p.M_in;
  double rho_r = p.rho_in * std::pow(1 + tmp1 * (1 - (p.r_in * p.r_in) / (r * r)), 1 / (gamma - 1));
  double p_r = (1.0 / gamma) * std::pow(rho_r / p.rho_in, gamma);
  double a_r = std::sqrt(gamma * p_r / rho_r);
  double M_r = std::sqrt((2 / (gamma - 1)) * std::pow(p.rho_in / rho_r, gamma - 1) * (1 + tmp1) - 2 / (gamma - 1));
  double U_r = M_r * a_r;
  double e_r = p.cv * p_r / (rho_r * p.R);
  sol[0] = rho_r;
  sol[1] = rho_r * (U_r * std::sin(theta));
  sol[2] = rho_r * (-U_r * std::cos(theta));
  sol[3] = rho_r * e_r + 0.5 * rho_r * U_r * U_r;
}

// free stream: reference common_funcs.jl:312-345
static void freestream_state(const DevParams& p, int dim, double* sol) {
  sol[0] = p.rho_free;
  sol[dim + 1] = p.E_free;
  sol[1] = p.rho_free * p.Ma * std::cos(p.aoa);
  if (dim == 2) {
    sol[2] = p.rho_free * p.Ma * std::sin(p.aoa);
  } else {
    sol[2] = 0.0;
    sol[3] = -p.rho_free * p.Ma * std::sin(p.aoa);
  }
}

// the kernels' copy of the physics parameters (reference ParamType fields,
// types.jl:236-260; E_free from calcFreeStream, common_funcs.jl:312-345)
static DevParams dev_params(const eg_params& pa) {
  DevParams p;
  p.gamma = pa.gamma;
  p.gamma_1 = pa.gamma - 1;
  p.Ma = pa.Ma;
  p.aoa = pa.aoa;
  p.rho_free = pa.rho_free;
  p.p_free = pa.p_free;
  p.E_free = pa.p_free / p.gamma_1 + 0.5 * pa.rho_free * pa.Ma * pa.Ma;
  p.r_in = pa.vortex_r_in;
  p.rho_in = pa.vortex_rho_in;
  p.M_in = pa.vortex_M_in;
  p.R = 287.058;
  p.cv = p.R / p.gamma_1;
  return p;
}

// Dirichlet state of every boundary face node from the boundary coordinates
// and each face's boundary condition
static void boundary_states(const DevParams& p, int dim, int B, int Nf, const int32_t* bc_of_b,
                            const double* coords_bndry, double* qg) {
  const int nv = dim + 2;
  for (int b = 0; b < B; ++b)
    for (int i = 0; i < Nf; ++i) {
      double* s = &qg[((size_t)b * Nf + i) * nv];
      if (bc_of_b[b] == EG_BC_VORTEX)
        vortex_state(p, coords_bndry + ((size_t)b * Nf + i) * dim, s);
      else if (bc_of_b[b] == EG_BC_NOPENETRATION_ES)
        for (int c = 0; c < nv; ++c) s[c] = 0.0;  // the wall's state follows q (no data)
      else
        freestream_state(p, dim, s);
    }
}

static void free_mesh(eg_mesh* m) {
  if (!m) return;
  eg_newton_ws_free(m);
  eg_rk4_ws_free(m);
  if (m->prolong_T) cudaFree(m->prolong_T);
  void* bufs[] = {m->Q, m->w, m->interp, m->perm, m->nbrperm, m->wface, m->lift, m->liftS,
                  m->nbrinv, m->dxidx,
                  m->jac, m->Minv, m->ifaces, m->nrm_face, m->bfaces, m->bc_of_b,
                  m->coords_bndry, m->nrm_bndry, m->qg_bndry, m->eface, m->fflux,
                  m->q_dev, m->res_dev, m->status, m->red};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (m->h_status) cudaFreeHost(m->h_status);
  if (m->h_red) cudaFreeHost(m->h_red);
  eg_timer_free(m);
  if (m->own_stream) cudaStreamDestroy(m->own_stream);
  delete m;
}

extern "C" int eg_mesh_create(const eg_mesh_desc* d, const eg_params* params, eg_mesh** out) {
  if (!d || !params || !out) {
    eg_set_error("eg_mesh_create: NULL argument");
    return EG_ERR_INVALID;
  }
  *out = nullptr;
  if (d->dim != 2 && d->dim != 3) {
    eg_set_error("eg_mesh_create: dim must be 2 or 3 (got %d)", d->dim);
    return EG_ERR_INVALID;
  }
  if (d->num_bc > 63) {
    eg_set_error("eg_mesh_create: at most 63 boundary-condition groups");
    return EG_ERR_INVALID;
  }
  if (d->num_el <= 0 || d->nodes_per_el <= 0 || d->nodes_per_el > EG_MAX_NP ||
      d->nodes_per_face <= 0 || d->nodes_per_face > EG_MAX_NF || d->stencil_size <= 0 ||
      d->stencil_size > EG_MAX_S || d->num_interfaces < 0 || d->num_bndry < 0 ||
      d->num_bc < 0 || d->num_orient <= 0) {
    eg_set_error("eg_mesh_create: sizes out of range (E=%d Np=%d Nf=%d S=%d)", d->num_el,
                 d->nodes_per_el, d->nodes_per_face, d->stencil_size);
    return EG_ERR_INVALID;
  }
  if (params->volume_integral_type != 1 && params->volume_integral_type != 2) {
    eg_set_error("eg_mesh_create: volume_integral_type must be 1 or 2");
    return EG_ERR_INVALID;
  }
  int dev = -1;
  EG_CUDA(cudaGetDevice(&dev));
  eg_mesh* m = new eg_mesh();
  std::memset(m, 0, sizeof(*m));
  m->device = dev;
  m->dim = d->dim;
  m->E = d->num_el;
  m->Np = d->nodes_per_el;
  m->Nf = d->nodes_per_face;
  m->S = d->stencil_size;
  m->F = d->dim + 1;
  m->I = d->num_interfaces;
  m->B = d->num_bndry;
  m->nbc = d->num_bc;
  m->norient = d->num_orient;
  m->nv = d->dim + 2;
  m->ndof = (int64_t)m->E * m->Np * m->nv;
  m->params = *params;
  m->dp = dev_params(*params);
  const DevParams& p = m->dp;

  const int dim = m->dim, E = m->E, Np = m->Np, Nf = m->Nf, S = m->S, F = m->F, I = m->I,
            B = m->B, nv = m->nv;
  // ---- host-side validation of indices
  for (int f = 0; f < F; ++f)
    for (int s = 0; s < S; ++s) {
      int v = d->perm[f * S + s];
      if (v < 0 || v >= Np) {
        eg_set_error("eg_mesh_create: perm[%d][%d] = %d out of range", f, s, v);
        free_mesh(m);
        return EG_ERR_INVALID;
      }
    }
  for (int o = 0; o < m->norient; ++o)
    for (int i = 0; i < Nf; ++i) {
      int v = d->nbrperm[o * Nf + i];
      if (v < 0 || v >= Nf) {
        eg_set_error("eg_mesh_create: nbrperm out of range");
        free_mesh(m);
        return EG_ERR_INVALID;
      }
    }
  std::vector<EFace> eface((size_t)E * F, EFace{-1, 0, 0, 0});
  for (int n = 0; n < I; ++n) {
    const int32_t* t = d->interfaces + 5 * n;
    if (t[0] < 0 || t[0] >= E || t[1] < 0 || t[1] >= E || t[2] < 0 || t[2] >= F || t[3] < 0 ||
        t[3] >= F || t[4] < 0 || t[4] >= m->norient) {
      eg_set_error("eg_mesh_create: interface %d out of range", n);
      free_mesh(m);
      return EG_ERR_INVALID;
    }
    EFace& a = eface[(size_t)t[0] * F + t[2]];
    EFace& b = eface[(size_t)t[1] * F + t[3]];
    if (a.slot >= 0 || b.slot >= 0) {
      eg_set_error("eg_mesh_create: element face used twice (interface %d)", n);
      free_mesh(m);
      return EG_ERR_INVALID;
    }
    a = EFace{n, 0, 0, 0};
    b = EFace{n, 1, t[4], 0};
  }
  std::vector<int32_t> bc_of_b(B, -1);
  if (m->nbc > 0 && (d->bndry_offsets[0] != 0 || d->bndry_offsets[m->nbc] != B)) {
    eg_set_error("eg_mesh_create: bndry_offsets must run from 0 to num_bndry");
    free_mesh(m);
    return EG_ERR_INVALID;
  }
  for (int g = 0; g < m->nbc; ++g)
    if (d->bndry_offsets[g] > d->bndry_offsets[g + 1] || d->bndry_offsets[g] < 0 ||
        d->bndry_offsets[g + 1] > B) {
      eg_set_error("eg_mesh_create: bndry_offsets not monotone in [0, num_bndry]");
      free_mesh(m);
      return EG_ERR_INVALID;
    }
  for (int g = 0; g <= m->nbc; ++g) m->h_bndry_offsets[g] = d->bndry_offsets[g];
  for (int g = 0; g < m->nbc; ++g) {
    int bct = d->bc_types[g];
    if (bct != EG_BC_VORTEX && bct != EG_BC_FREESTREAM && bct != EG_BC_NOPENETRATION_ES) {
      eg_set_error("eg_mesh_create: unsupported boundary condition %d", bct);
      free_mesh(m);
      return EG_ERR_UNSUPPORTED;
    }
    if (bct == EG_BC_VORTEX && dim != 2) {
      eg_set_error("eg_mesh_create: the isentropic vortex is 2D only");
      free_mesh(m);
      return EG_ERR_UNSUPPORTED;
    }
    for (int b = d->bndry_offsets[g]; b < d->bndry_offsets[g + 1]; ++b) bc_of_b[b] = bct;
  }
  for (int b = 0; b < B; ++b) {
    int e = d->bndryfaces[2 * b], f = d->bndryfaces[2 * b + 1];
    if (e < 0 || e >= E || f < 0 || f >= F || bc_of_b[b] < 0) {
      eg_set_error("eg_mesh_create: boundary face %d invalid", b);
      free_mesh(m);
      return EG_ERR_INVALID;
    }
    EFace& a = eface[(size_t)e * F + f];
    if (a.slot >= 0) {
      eg_set_error("eg_mesh_create: element face used twice (boundary %d)", b);
      free_mesh(m);
      return EG_ERR_INVALID;
    }
    a = EFace{I + b, 0, 0, 0};
  }
  for (size_t k = 0; k < eface.size(); ++k)
    if (eface[k].slot < 0) {
      eg_set_error("eg_mesh_create: element %zu face %zu is neither interface nor boundary",
                   k / F, k % F);
      free_mesh(m);
      return EG_ERR_INVALID;
    }
  // lift[f][j][i] = sum_s [perm[f][s] == j] interp[f][i][s] * wface[i]
  std::vector<double> lift((size_t)F * Np * Nf, 0.0);
  for (int f = 0; f < F; ++f)
    for (int i = 0; i < Nf; ++i)
      for (int s = 0; s < S; ++s)
        lift[((size_t)f * Np + d->perm[f * S + s]) * Nf + i] +=
            d->interp[((size_t)f * Nf + i) * S + s] * d->wface[i];
  std::vector<double> liftS((size_t)F * Nf * S);
  for (int f = 0; f < F; ++f)
    for (int i = 0; i < Nf; ++i)
      for (int s = 0; s < S; ++s)
        liftS[((size_t)f * Nf + i) * S + s] = d->interp[((size_t)f * Nf + i) * S + s] * d->wface[i];
  std::vector<int32_t> nbrinv((size_t)m->norient * Nf);
  for (int o = 0; o < m->norient; ++o)
    for (int i = 0; i < Nf; ++i) nbrinv[(size_t)o * Nf + d->nbrperm[o * Nf + i]] = i;
  m->sparse_face = (S == Nf);
  for (int f = 0; f < F && m->sparse_face; ++f)
    for (int i = 0; i < Nf; ++i)
      for (int s = 0; s < S; ++s)
        if (d->interp[((size_t)f * Nf + i) * S + s] != (i == s ? 1.0 : 0.0)) m->sparse_face = 0;
  // Dirichlet states at the boundary face nodes
  std::vector<double> qg((size_t)B * Nf * nv, 0.0);
  boundary_states(p, dim, B, Nf, bc_of_b.data(), d->coords_bndry, qg.data());
  std::vector<double> minv((size_t)E * Np);
  for (int e = 0; e < E; ++e)
    for (int j = 0; j < Np; ++j) minv[(size_t)e * Np + j] = d->jac[(size_t)e * Np + j] / d->w[j];

  int st = EG_OK;
#define UP(dst, src, n, name) \
  if (st == EG_OK) st = upload(&m->dst, src, n, name)
  UP(Q, d->Q, (size_t)dim * Np * Np, "Q");
  UP(w, d->w, (size_t)Np, "w");
  UP(interp, d->interp, (size_t)F * Nf * S, "interp");
  UP(perm, d->perm, (size_t)F * S, "perm");
  UP(nbrperm, d->nbrperm, (size_t)m->norient * Nf, "nbrperm");
  UP(wface, d->wface, (size_t)Nf, "wface");
  UP(lift, lift.data(), lift.size(), "lift");
  UP(liftS, liftS.data(), liftS.size(), "liftS");
  UP(nbrinv, nbrinv.data(), nbrinv.size(), "nbrinv");
  UP(dxidx, d->dxidx, (size_t)E * Np * dim * dim, "dxidx");
  UP(jac, d->jac, (size_t)E * Np, "jac");
  UP(Minv, minv.data(), minv.size(), "Minv");
  UP(ifaces, d->interfaces, (size_t)I * 5, "interfaces");
  UP(nrm_face, d->nrm_face, (size_t)I * Nf * dim, "nrm_face");
  UP(bfaces, d->bndryfaces, (size_t)B * 2, "bndryfaces");
  UP(bc_of_b, bc_of_b.data(), (size_t)B, "bc");
  UP(coords_bndry, d->coords_bndry, (size_t)B * Nf * dim, "coords_bndry");
  UP(nrm_bndry, d->nrm_bndry, (size_t)B * Nf * dim, "nrm_bndry");
  UP(qg_bndry, qg.data(), qg.size(), "qg");
  UP(eface, eface.data(), eface.size(), "eface");
#undef UP
  if (st == EG_OK) st = alloc(&m->fflux, (size_t)(I + B) * Nf * nv);
  if (st == EG_OK) st = alloc(&m->q_dev, (size_t)m->ndof);
  if (st == EG_OK) st = alloc(&m->res_dev, (size_t)m->ndof);
  if (st == EG_OK) st = alloc(&m->status, 1);
  if (st == EG_OK) st = alloc(&m->red, 4096);
  if (st == EG_OK) {
    cudaError_t e1 = cudaStreamCreateWithFlags(&m->own_stream, cudaStreamNonBlocking);
    if (e1 != cudaSuccess) st = eg_cuda_fail(e1, "cudaStreamCreate");
    m->stream = m->own_stream;
  }
  if (st == EG_OK) {
    cudaError_t e1 = cudaMallocHost((void**)&m->h_status, sizeof(unsigned int));
    if (e1 == cudaSuccess) e1 = cudaMallocHost((void**)&m->h_red, 64 * sizeof(double));
    if (e1 != cudaSuccess) st = eg_cuda_fail(e1, "cudaMallocHost");
  }
  if (st == EG_OK) {
    cudaError_t e1 = cudaMemset(m->status, 0, sizeof(unsigned int));
    if (e1 != cudaSuccess) st = eg_cuda_fail(e1, "cudaMemset");
  }
  if (st != EG_OK) {
    free_mesh(m);
    return st;
  }
  *out = m;
  return EG_OK;
}

extern "C" int eg_mesh_destroy(eg_mesh* m) {
  if (!m) return EG_OK;
  cudaStreamSynchronize(m->stream);
  free_mesh(m);
  return EG_OK;
}

extern "C" int64_t eg_mesh_num_dof(const eg_mesh* m) { return m ? m->ndof : -1; }

// New physics parameters on an existing mesh (the reference mutates
// eqn.params / opts between solves).  The boundary Dirichlet states are
// re-evaluated from the device copy of the boundary coordinates; the mesh
// stream is synchronised before and after, so no launch sees a half update.
extern "C" int eg_mesh_set_params(eg_mesh* m, const eg_params* params) {
  if (!m || !params) {
    eg_set_error("eg_mesh_set_params: NULL argument");
    return EG_ERR_INVALID;
  }
  if (params->volume_integral_type != 1 && params->volume_integral_type != 2) {
    eg_set_error("eg_mesh_set_params: volume_integral_type must be 1 or 2");
    return EG_ERR_INVALID;
  }
  if (m->capturing) {
    eg_set_error("eg_mesh_set_params: the mesh stream is being captured");
    return EG_ERR_INVALID;
  }
  const int B = m->B, Nf = m->Nf, dim = m->dim;
  std::vector<int32_t> bc(B);
  std::vector<double> xb((size_t)B * Nf * dim), qg((size_t)B * Nf * m->nv, 0.0);
  EG_CUDA(cudaStreamSynchronize(m->stream));
  if (B > 0) {
    EG_CUDA(cudaMemcpyAsync(bc.data(), m->bc_of_b, sizeof(int32_t) * B, cudaMemcpyDeviceToHost,
                            m->stream));
    EG_CUDA(cudaMemcpyAsync(xb.data(), m->coords_bndry, sizeof(double) * xb.size(),
                            cudaMemcpyDeviceToHost, m->stream));
    EG_CUDA(cudaStreamSynchronize(m->stream));
  }
  const DevParams p = dev_params(*params);
  boundary_states(p, dim, B, Nf, bc.data(), xb.data(), qg.data());
  if (B > 0) {
    EG_CUDA(cudaMemcpyAsync(m->qg_bndry, qg.data(), sizeof(double) * qg.size(),
                            cudaMemcpyHostToDevice, m->stream));
    EG_CUDA(cudaStreamSynchronize(m->stream));
  }
  m->params = *params;
  m->dp = p;
  return EG_OK;
}
