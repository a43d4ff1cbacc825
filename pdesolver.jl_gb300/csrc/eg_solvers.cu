// eg_solvers.cu -- Newton steady solve and RK4 time stepping on the device.
//
// newton / newtonInner: reference src/NonlinearSolvers/newton.jl:54-304 with
//   physicsRhs (src/jacobian/residual_evaluation.jl:64-84: residual + calcNorm
//   with M^-1), doRecalculation every iteration (jac_recalc.jl:60-97),
//   linearSolve to krylov_reltol (ls_standard.jl:321-371), q += dq,
//   checkConvergence (newton.jl:402-455).
// rk4: reference src/NonlinearSolvers/rk4.jl:144-336 with pde_pre_func /
//   pde_post_func (rk4.jl:425-456): k_s = M^-1 R(q_s), classical stages.
// The state, residual, norms and update stay FP64; with EG_F32 the Jacobian,
// preconditioner and Krylov vectors are FP32 (inexact Newton against the FP64
// residual).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "eg_internal.h"
#include "eg_kernels.cuh"
#include "eg_linalg.h"

namespace {

// y = a*x + b*y (FP64)
__global__ void k_axpby64(double a, const double* __restrict__ x, double b, double* __restrict__ y,
                          int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}

// RK4 stage: k_s = M^-1 res (in place into ks), q = x_old + c * k_s
__global__ void k_rk4_stage(const double* __restrict__ res, const double* __restrict__ Minv,
                            const double* __restrict__ xold, double c, double* __restrict__ ks,
                            double* __restrict__ q, int64_t nnode, int nv) {
  const int64_t N = nnode * nv;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const double k = Minv[i / nv] * res[i];
    ks[i] = k;
    q[i] = xold[i] + c * k;
  }
}

// final RK4 update: x_old += h/6 (k1 + 2 k2 + 2 k3 + k4), q = x_old (k4 = M^-1 res)
__global__ void k_rk4_final(const double* __restrict__ k1, const double* __restrict__ k2,
                            const double* __restrict__ k3, const double* __restrict__ res,
                            const double* __restrict__ Minv, double h, double* __restrict__ xold,
                            double* __restrict__ q, int64_t nnode, int nv) {
  const int64_t N = nnode * nv;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const double k4 = Minv[i / nv] * res[i];
    const double x = xold[i] + (h / 6) * (k1[i] + 2 * k2[i] + 2 * k3[i] + k4);
    xold[i] = x;
    q[i] = x;
  }
}

// pseudo-transient continuation: J(e,(j,a),(j,a)) -= M_j / tau_vec_j with
// tau_vec = tau_l / (1 + sqrt(jac))  (reference globalization.jl:165-320)
template <typename T>
__global__ void k_ptc_shift(T* __restrict__ diag, const double* __restrict__ jac,
                            const double* __restrict__ w, double tau_l, int E, int Np, int nv) {
  const int n = Np * nv;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)E * n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(t / n), r = (int)(t - (int64_t)e * n);
    const int j = r / nv;
    const double jj = jac[(size_t)e * Np + j];
    const double M = w[j] / jj;
    const double tv = tau_l / (1.0 + sqrt(jj));
    diag[(size_t)e * n * n + (size_t)r * n + r] -= T(M / tv);
  }
}

int grid64(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b > 152 * 16 ? 152 * 16 : (b < 1 ? 1 : b));
}

// residual + strong norm; synchronises and reports device status
int residual_and_norm(eg_mesh* m, const double* q, double* res, double* norm) {
  EG_CUDA(cudaMemsetAsync(m->status, 0, sizeof(unsigned int), m->stream));
  int st = eg_launch_residual(m, q, res);
  if (st != EG_OK) return st;
  eg_launch_norm(m, res, 1, m->red + 2048);
  EG_CUDA(cudaGetLastError());
  EG_CUDA(cudaMemcpyAsync(m->h_red, m->red + 2048, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  EG_CUDA(cudaMemcpyAsync(m->h_status, m->status, sizeof(unsigned int), cudaMemcpyDeviceToHost, m->stream));
  EG_CUDA(cudaStreamSynchronize(m->stream));
  st = eg_check_status(m);
  if (st != EG_OK) return st;
  *norm = m->h_red[0];
  if (!std::isfinite(*norm)) {
    eg_set_error("non-finite residual norm");
    return EG_ERR_NONFINITE;
  }
  return EG_OK;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

// largest factor by which the pseudo-time step may grow in one iteration, and
// the residual growth that makes a pseudo-time step be rejected (recovery
// added here; the reference has neither)
constexpr double PTC_MAX_GROWTH = 1.5;
constexpr double PTC_MAX_INCREASE = 10.0;
// a step whose Krylov solve did not reach its tolerance and that leaves |R|
// above this fraction of its previous value shrinks the pseudo-time step 4x
// (recovery added here: restarted GMRES with the element block-Jacobi
// preconditioner stagnates on the nearly steady Jacobian of fine meshes, and
// the reference's SER update would keep the pseudo-time step there)
constexpr double PTC_STALL = 0.5;

// Newton work objects of a mesh, kept between solves so that repeated solves
// (continuation levels, batches, serving) allocate nothing after the first:
// cudaFree synchronises the device and would serialise concurrent streams.
// With the graph path, one Newton iteration runs as three CUDA graphs around
// the persistent GMRES launch (see newton_graph_iteration); the graphs are
// bound to the work objects' pointers and captured once per option set.
struct GraphKey {
  eg_params params;
  int elem_epb, vol_mma, globalize, itermax;
  double reltol;
};

struct eg_newton_ws {
  int prec = -1, restart = 0;
  eg_lo* lo = nullptr;
  eg_pc* pc = nullptr;
  eg_ls* ls = nullptr;
  double* res = nullptr;    // [N] residual
  double* dq = nullptr;     // [N] Newton step
  double* qsave = nullptr;  // [N] state before the step (rejection, pivot failure)
  double* qd = nullptr;     // [N] the state the graphs update (caller's q staged here)
  // graph path
  bool graph_tried = false, graph_ok = false;
  GraphKey key;
  cudaGraphExec_t gJ = nullptr, gP = nullptr, gU = nullptr;  // Jacobian, PC + rhs, update + residual
  int64_t nJ = 0, nP = 0, nU = 0;                             // kernel nodes of each
  double* h_tau = nullptr;  // pinned: pseudo-time step of the next iteration
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
};

void eg_newton_ws_free(eg_mesh* m) {
  eg_newton_ws* w = m ? m->nws : nullptr;
  if (!w) return;
  cudaGraphExec_t gs[] = {w->gJ, w->gP, w->gU};
  for (cudaGraphExec_t g : gs)
    if (g) cudaGraphExecDestroy(g);
  for (cudaEvent_t e : w->ev)
    if (e) cudaEventDestroy(e);
  if (w->h_tau) cudaFreeHost(w->h_tau);
  if (w->ls) eg_ls_destroy(w->ls);
  if (w->pc) eg_pc_destroy(w->pc);
  if (w->lo) eg_lo_destroy(w->lo);
  double* bufs[] = {w->res, w->dq, w->qsave, w->qd};
  for (double* b : bufs)
    if (b) cudaFree(b);
  delete w;
  m->nws = nullptr;
}

extern "C" int eg_newton_release(eg_mesh* m) {
  if (!m) return EG_ERR_INVALID;
  EG_CUDA(cudaStreamSynchronize(m->stream));
  eg_newton_ws_free(m);
  return EG_OK;
}

namespace {
// the mesh's Newton work objects for (precision, restart), created on first use
int newton_ws(eg_mesh* m, int prec, int restart, eg_newton_ws** out) {
  eg_newton_ws* w = m->nws;
  if (w && (w->prec != prec || w->restart != restart)) {
    EG_CUDA(cudaStreamSynchronize(m->stream));
    eg_newton_ws_free(m);
    w = nullptr;
  }
  const int64_t N = m->ndof;
  if (!w) {
    w = new eg_newton_ws();
    m->nws = w;
    w->prec = prec;
    w->restart = restart;
    cudaError_t ce = cudaMalloc((void**)&w->res, 8 * N);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&w->dq, 8 * N);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&w->qsave, 8 * N);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&w->qd, 8 * N);
    if (ce == cudaSuccess) ce = cudaMallocHost((void**)&w->h_tau, sizeof(double));
    for (int k = 0; k < 5 && ce == cudaSuccess; ++k) ce = cudaEventCreate(&w->ev[k]);
    if (ce != cudaSuccess) {
      eg_newton_ws_free(m);
      return eg_cuda_fail(ce, "eg_newton_solve");
    }
    int st = eg_lo_create(m, prec, &w->lo);
    if (st == EG_OK) st = eg_pc_create(w->lo, &w->pc);
    if (st == EG_OK) st = eg_ls_create(w->lo, w->pc, restart, &w->ls);
    if (st != EG_OK) {
      eg_newton_ws_free(m);
      return st;
    }
  }
  *out = w;
  return EG_OK;
}

// pseudo-time shift with tau_l read from device memory (graph path: the
// host writes the step of each iteration into pinned memory, a captured copy
// brings it to the device)
template <typename T>
__global__ void k_ptc_shift_dev(T* __restrict__ diag, const double* __restrict__ jac,
                                const double* __restrict__ w, const double* __restrict__ tau, int E,
                                int Np, int nv) {
  const int n = Np * nv;
  const double tau_l = *tau;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)E * n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(t / n), r = (int)(t - (int64_t)e * n);
    const int j = r / nv;
    const double jj = jac[(size_t)e * Np + j];
    const double M = w[j] / jj;
    const double tv = tau_l / (1.0 + sqrt(jj));
    diag[(size_t)e * n * n + (size_t)r * n + r] -= T(M / tv);
  }
}

// fresh GMRES state for one linear solve (the values linearSolve starts from)
__global__ void k_gmres_reset(double* __restrict__ scal, int* __restrict__ flags, double reltol,
                              double abstol, int itermax) {
  if (threadIdx.x != 0) return;
  for (int k = 0; k < 8; ++k) {
    scal[k] = 0.0;
    flags[k] = 0;
  }
  scal[S_RELTOL] = reltol;
  scal[S_ABSTOL] = abstol;
  flags[F_ITERMAX] = itermax;
}

// capture fn on the mesh stream into an executable graph; false (and no
// graph) when the stream cannot be captured or the capture fails
template <typename F>
bool capture_graph(eg_mesh* m, F fn, cudaGraphExec_t* exec, int64_t* nodes) {
  *exec = nullptr;
  if (m->stream == 0 || m->stream == cudaStreamLegacy || m->stream == cudaStreamPerThread) return false;
  cudaGraph_t graph = nullptr;
  const int64_t l0 = m->launches;
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
  m->launches = l0;
  if (e != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return false;
  }
  // kernel nodes (the launch count of one replay)
  size_t n = 0;
  cudaGraphGetNodes(graph, nullptr, &n);
  std::vector<cudaGraphNode_t> nl(n);
  int64_t kernels = 0;
  if (n && cudaGraphGetNodes(graph, nl.data(), &n) == cudaSuccess)
    for (size_t k = 0; k < n; ++k) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nl[k], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
    }
  e = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    *exec = nullptr;
    cudaGetLastError();
    return false;
  }
  *nodes = kernels;
  return true;
}

// the three graphs of one Newton iteration:
//   gJ  status word cleared, pseudo-time step to the device, Jacobian blocks,
//       pseudo-time diagonal shift
//   gP  block-Jacobi inverses, dq = 0, b = -R and x = 0 in the operator
//       precision, fresh GMRES state
//   gU  dq from the Krylov solution, ||dq||, q saved, q += dq, R(q), ||R||_{M^-1},
//       read-back of the norms, the status word and the GMRES state
bool capture_newton_graphs(eg_mesh* m, eg_newton_ws* w, const GraphKey& key) {
  eg_lo* lo = w->lo;
  eg_pc* pc = w->pc;
  eg_ls* ls = w->ls;
  const int64_t N = m->ndof;
  cudaStream_t s = m->stream;
  double* d_tau = m->red + 2050;
  bool ok = capture_graph(m, [&]() {
    cudaMemsetAsync(m->status, 0, sizeof(unsigned int), s);
    if (key.globalize) cudaMemcpyAsync(d_tau, w->h_tau, sizeof(double), cudaMemcpyHostToDevice, s);
    eg_jacobian_launch(lo, w->qd);
    if (key.globalize) {
      const int blocks = grid64((int64_t)m->E * lo->n);
      if (lo->prec == EG_F64)
        k_ptc_shift_dev<double><<<blocks, 256, 0, s>>>((double*)lo->diag, m->jac, m->w, d_tau, m->E, m->Np, m->nv);
      else
        k_ptc_shift_dev<float><<<blocks, 256, 0, s>>>((float*)lo->diag, m->jac, m->w, d_tau, m->E, m->Np, m->nv);
    }
  }, &w->gJ, &w->nJ);
  lo->valid = true;
  ok = ok && capture_graph(m, [&]() {
    eg_pc_calc(pc);
    cudaMemsetAsync(w->dq, 0, 8 * N, s);
    eg_convert(m, w->res, ls->bT, lo->prec, N, -1.0);
    eg_convert(m, w->dq, ls->xT, lo->prec, N, 1.0);
    k_gmres_reset<<<1, 32, 0, s>>>(ls->dscal, ls->dflags, key.reltol, 1e-30, key.itermax);
  }, &w->gP, &w->nP);
  ok = ok && capture_graph(m, [&]() {
    eg_convert_back(m, ls->xT, w->dq, lo->prec, N);
    eg_launch_norm(m, w->dq, 2, m->red + 2049);
    cudaMemcpyAsync(w->qsave, w->qd, 8 * N, cudaMemcpyDeviceToDevice, s);
    k_axpby64<<<grid64(N), 256, 0, s>>>(1.0, w->dq, 1.0, w->qd, N);
    eg_launch_residual(m, w->qd, w->res);
    eg_launch_norm(m, w->res, 1, m->red + 2048);
    cudaMemcpyAsync(m->h_red, m->red + 2048, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(m->h_status, m->status, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ls->hh, ls->dscal, 8 * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ls->hh + 8, ls->dflags, 8 * sizeof(int), cudaMemcpyDeviceToHost, s);
  }, &w->gU, &w->nU);
  if (!ok) {
    cudaGraphExec_t gs[] = {w->gJ, w->gP, w->gU};
    for (cudaGraphExec_t g : gs)
      if (g) cudaGraphExecDestroy(g);
    w->gJ = w->gP = w->gU = nullptr;
  }
  return ok;
}

// Result of one Newton iteration (either path).
struct IterOut {
  int st = EG_OK;
  bool updated = false;    // q holds q + dq (else q is the iteration's start)
  double norm = 0.0;       // ||R(q + dq)||_{M^-1}
  double step = 0.0;       // ||dq||_2
  int kits = 0, kconv = 0;
  double tj = 0, tp = 0, tk = 0, tr = 0;  // ms: Jacobian, PC, Krylov, update + residual
};

// One iteration on the graph path: gJ, gP, the persistent GMRES launch, gU,
// then one synchronisation.  A zero pivot restores q from its saved copy.
IterOut newton_graph_iteration(eg_mesh* m, eg_newton_ws* w, double tau_l) {
  IterOut r;
  cudaStream_t s = m->stream;
  eg_ls* ls = w->ls;
  *w->h_tau = tau_l;
  cudaError_t ce = cudaEventRecord(w->ev[0], s);
  if (ce == cudaSuccess) ce = cudaGraphLaunch(w->gJ, s);
  if (ce == cudaSuccess) ce = cudaEventRecord(w->ev[1], s);
  if (ce == cudaSuccess) ce = cudaGraphLaunch(w->gP, s);
  if (ce == cudaSuccess) ce = cudaEventRecord(w->ev[2], s);
  if (ce != cudaSuccess) {
    r.st = eg_cuda_fail(ce, "eg_newton_solve graph");
    return r;
  }
  m->launches += w->nJ + w->nP;
  r.st = eg_gmres_coop(ls);
  if (r.st != EG_OK) return r;
  ce = cudaEventRecord(w->ev[3], s);
  if (ce == cudaSuccess) ce = cudaGraphLaunch(w->gU, s);
  if (ce == cudaSuccess) ce = cudaEventRecord(w->ev[4], s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) {
    r.st = eg_cuda_fail(ce, "eg_newton_solve graph");
    return r;
  }
  m->launches += w->nU;
  r.updated = true;
  float t[4] = {0, 0, 0, 0};
  for (int k = 0; k < 4; ++k) cudaEventElapsedTime(&t[k], w->ev[k], w->ev[k + 1]);
  r.tj = t[0];
  r.tp = t[1];
  r.tk = t[2];
  r.tr = t[3];
  double scal[8];
  int flags[8];
  std::memcpy(scal, ls->hh, sizeof(scal));
  std::memcpy(flags, ls->hh + 8, sizeof(flags));
  r.kits = flags[F_ITS];
  r.kconv = flags[F_CONV];
  r.step = m->h_red[1];
  r.norm = m->h_red[0];
  const unsigned int status = *m->h_status;
  if (status & EG_DEV_LU_PIVOT) {
    // the eager path stops before the update: put q back
    cudaMemcpyAsync(w->qd, w->qsave, 8 * m->ndof, cudaMemcpyDeviceToDevice, s);
    cudaStreamSynchronize(s);
    eg_set_error("zero pivot in block LU");
    r.st = EG_ERR_LU_PIVOT;
    r.updated = false;
    return r;
  }
  if (!std::isfinite(scal[S_BETA])) {
    cudaMemcpyAsync(w->qd, w->qsave, 8 * m->ndof, cudaMemcpyDeviceToDevice, s);
    cudaStreamSynchronize(s);
    eg_set_error("GMRES: non-finite residual");
    r.st = EG_ERR_NONFINITE;
    r.updated = false;
    return r;
  }
  r.st = eg_check_status(m);
  if (r.st == EG_OK && !std::isfinite(r.norm)) {
    eg_set_error("non-finite residual norm");
    r.st = EG_ERR_NONFINITE;
  }
  return r;
}

// One iteration launched eagerly (timers on, a stream that cannot be
// captured, or a system the persistent GMRES kernel does not take).
IterOut newton_eager_iteration(eg_mesh* m, eg_newton_ws* w, double* qd, bool globalize, double tau_l) {
  IterOut r;
  eg_lo* lo = w->lo;
  eg_pc* pc = w->pc;
  eg_ls* ls = w->ls;
  const int64_t N = m->ndof;
  auto t0 = std::chrono::steady_clock::now();
  int st = eg_lo_calc(lo, qd, EG_MEM_DEVICE);
  if (st == EG_OK && globalize) {
    const int blocks = grid64((int64_t)m->E * lo->n);
    if (lo->prec == EG_F64)
      k_ptc_shift<double><<<blocks, 256, 0, m->stream>>>((double*)lo->diag, m->jac, m->w, tau_l, m->E, m->Np, m->nv);
    else
      k_ptc_shift<float><<<blocks, 256, 0, m->stream>>>((float*)lo->diag, m->jac, m->w, tau_l, m->E, m->Np, m->nv);
    m->launches += 1;
  }
  if (st == EG_OK) {
    cudaError_t ce = cudaStreamSynchronize(m->stream);
    if (ce != cudaSuccess) st = eg_cuda_fail(ce, "eg_newton_solve");
  }
  r.tj = ms_since(t0);
  if ((r.st = st) != EG_OK) return r;
  t0 = std::chrono::steady_clock::now();
  st = eg_pc_calc(pc);
  if (st == EG_OK) {
    cudaError_t ce = cudaMemcpyAsync(m->h_status, m->status, sizeof(unsigned int), cudaMemcpyDeviceToHost, m->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(m->stream);
    st = ce != cudaSuccess ? eg_cuda_fail(ce, "eg_newton_solve") : eg_check_status(m);
  }
  r.tp = ms_since(t0);
  if ((r.st = st) != EG_OK) return r;
  // J dq = -R, dq0 = 0
  t0 = std::chrono::steady_clock::now();
  cudaMemsetAsync(w->dq, 0, 8 * N, m->stream);
  eg_convert(m, w->res, ls->bT, lo->prec, N, -1.0);
  eg_convert(m, w->dq, ls->xT, lo->prec, N, 1.0);
  eg_ls_stats ks;
  st = eg_gmres_T(ls, ls->bT, ls->xT, &ks);
  if ((r.st = st) != EG_OK) return r;
  eg_convert_back(m, ls->xT, w->dq, lo->prec, N);
  r.kits = ks.iters;
  r.kconv = ks.converged;
  // step norm ||dq||_2 (reference newton.jl:238: norm(delta_q_vec))
  eg_launch_norm(m, w->dq, 2, m->red + 2049);
  cudaMemcpyAsync(w->qsave, qd, 8 * N, cudaMemcpyDeviceToDevice, m->stream);
  k_axpby64<<<grid64(N), 256, 0, m->stream>>>(1.0, w->dq, 1.0, qd, N);
  m->launches += 1;
  r.updated = true;
  cudaMemcpyAsync(m->h_red + 1, m->red + 2049, sizeof(double), cudaMemcpyDeviceToHost, m->stream);
  cudaError_t ce = cudaStreamSynchronize(m->stream);
  if (ce != cudaSuccess) {
    r.st = eg_cuda_fail(ce, "eg_newton_solve");
    return r;
  }
  r.step = m->h_red[1];
  r.tk = ms_since(t0);
  // residual at the new state
  t0 = std::chrono::steady_clock::now();
  r.st = residual_and_norm(m, qd, w->res, &r.norm);
  r.tr = ms_since(t0);
  return r;
}
}  // namespace

extern "C" int eg_newton_solve(eg_mesh* m, double* q, int32_t mem, const eg_newton_opts* o,
                               eg_newton_stats* stats) {
  if (!m || !q || !o) {
    eg_set_error("eg_newton_solve: NULL argument");
    return EG_ERR_INVALID;
  }
  const int64_t N = m->ndof;
  eg_newton_stats s;
  std::memset(&s, 0, sizeof(s));
  eg_newton_ws* w = nullptr;
  int st = newton_ws(m, o->precision, o->gmres_restart > 0 ? o->gmres_restart : 30, &w);
  if (st != EG_OK) return st;
  eg_ls* ls = w->ls;
  // with batched GMRES, the batcher waits for the multi-block solves of the
  // threads in here
  struct BatchGuard {
    int dev = -1;
    explicit BatchGuard(const eg_ls* ls) {
      if (eg_gmres_batching() && eg_coop_usable(ls) && eg_gmres_wanted_blocks(ls) > 1 &&
          cudaGetDevice(&dev) == cudaSuccess)
        eg_batch_enter(dev);
      else
        dev = -1;
    }
    ~BatchGuard() {
      if (dev >= 0) eg_batch_leave(dev);
    }
  } batch_guard(ls);
  const int kmax = o->krylov_itermax > 0 ? o->krylov_itermax : 1000;
  st = eg_ls_set_tolerances(ls, o->krylov_reltol, 1e-30, -1, kmax);
  if (st != EG_OK) return st;
  const bool globalize = o->globalize_euler != 0;
  // graph path: the state lives in the work objects' own vector
  GraphKey key;
  std::memset(&key, 0, sizeof(key));
  key.params = m->params;
  key.elem_epb = m->elem_epb;
  key.vol_mma = m->vol_mma;
  key.globalize = globalize;
  key.itermax = kmax;
  key.reltol = o->krylov_reltol;
  bool graph = !eg_timing_on(m) && !m->capturing && eg_coop_usable(ls);
  double* qd = (mem == EG_MEM_HOST || graph) ? w->qd : q;
  cudaError_t ce = cudaSuccess;
  if (qd != q) {
    ce = cudaMemcpyAsync(qd, q, 8 * N, mem == EG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                         m->stream);
    if (ce != cudaSuccess) return eg_cuda_fail(ce, "eg_newton_solve");
  }
  auto t0 = std::chrono::steady_clock::now();
  double norm = 0;
  st = residual_and_norm(m, qd, w->res, &norm);
  s.t_residual += ms_since(t0);
  if (st != EG_OK) return st;
  if (graph && (!w->graph_tried || std::memcmp(&key, &w->key, sizeof(key)) != 0)) {
    cudaGraphExec_t gs[] = {w->gJ, w->gP, w->gU};
    for (cudaGraphExec_t g : gs)
      if (g) cudaGraphExecDestroy(g);
    w->gJ = w->gP = w->gU = nullptr;
    w->key = key;
    w->graph_tried = true;
    w->graph_ok = capture_newton_graphs(m, w, key);
  }
  // no graphs: a device caller's state is iterated in place (it still holds q0)
  if (graph && !w->graph_ok && mem == EG_MEM_DEVICE) qd = q;
  graph = graph && w->graph_ok;
  s.res_norm0 = norm;
  s.res_norm = norm;
  const double norm_rel = norm;
  bool conv = norm < o->res_abstol;
  double tau_l = o->euler_tau, norm_prev = 0.0;
  // per-iteration trace on stderr (the reference's newton_verbosity output)
  const bool verbose = std::getenv("EG_NEWTON_VERBOSE") != nullptr;
  for (int it = 1; !conv && it <= o->itermax; ++it) {
    if (globalize) {
      if (norm_prev != 0.0) tau_l *= fmin(norm_prev / norm, PTC_MAX_GROWTH);
      norm_prev = norm;
    }
    const IterOut r = graph ? newton_graph_iteration(m, w, tau_l)
                            : newton_eager_iteration(m, w, qd, globalize, tau_l);
    s.t_jacobian += r.tj;
    s.t_pc += r.tp;
    s.t_krylov += r.tk;
    s.t_residual += r.tr;
    s.krylov_iters += r.kits;
    if (graph) s.graph_iters += 1;
    st = r.st;
    if (st != EG_OK && !r.updated) break;  // failed before the update: q unchanged
    s.step_norm = r.step;
    const double nn = r.norm;
    s.iters = it;
    if (verbose)
      std::fprintf(stderr, "eg_newton %3d |R| %.3e -> %.3e tau %.3e krylov %d st %d\n", it, norm, nn,
                   tau_l, r.kits, st);
    const bool bad = st == EG_ERR_NEG_DENSITY || st == EG_ERR_NEG_PRESSURE || st == EG_ERR_NONFINITE ||
                     (st == EG_OK && nn > PTC_MAX_INCREASE * norm);
    if (bad && globalize) {
      // reject the pseudo-time step: restore q, shrink tau
      EG_CUDA(cudaMemcpyAsync(qd, w->qsave, 8 * N, cudaMemcpyDeviceToDevice, m->stream));
      double nr = 0.0;
      st = residual_and_norm(m, qd, w->res, &nr);
      if (st != EG_OK) break;
      tau_l *= 0.25;
      norm_prev = 0.0;
      continue;
    }
    if (st != EG_OK) break;
    const bool stalled = globalize && !r.kconv && nn > PTC_STALL * norm;
    norm = nn;
    s.res_norm = norm;
    conv = norm < o->res_abstol || (norm / norm_rel < o->res_reltol) || (s.step_norm <= o->step_tol);
    if (stalled && !conv) {
      tau_l *= 0.25;
      norm_prev = 0.0;  // no SER growth right after
    }
  }
  s.converged = conv ? 1 : 0;
  if (st == EG_OK && qd != q) {
    ce = cudaMemcpyAsync(q, qd, 8 * N, mem == EG_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                         m->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(m->stream);
    if (ce != cudaSuccess) st = eg_cuda_fail(ce, "eg_newton_solve copy-out");
  }
  if (stats) *stats = s;
  if (st == EG_OK && !conv) {
    eg_set_error("Newton did not converge in %d iterations (|R| = %g)", o->itermax, s.res_norm);
    return EG_ERR_NOT_CONVERGED;
  }
  return st;
}

// RK4 work objects a mesh keeps between eg_rk4 calls: the six state-sized
// vectors of the step loop, and CUDA graphs of one step (whole step; stage 1
// with the norm read-back; stages 2-4), captured on first use and bound to
// the vectors, the step size and the launch configuration they were taken
// with.
struct eg_rk4_ws {
  double* buf = nullptr;  // [6][N]: x_old, k1, k2, k3, res, q
  bool tried = false;     // capture attempted for `key`
  bool have = false;      // graphs valid for `key`
  struct {
    eg_params params;
    double h;
    int elem_epb, vol_mma;
    cudaStream_t stream;
  } key;
  cudaGraphExec_t g_step = nullptr, g_stage1 = nullptr, g_rest = nullptr;
  int64_t n_step = 0, n_stage1 = 0, n_rest = 0;
};

namespace {

void rk4_graphs_free(eg_rk4_ws* w) {
  cudaGraphExec_t gs[] = {w->g_step, w->g_stage1, w->g_rest};
  for (cudaGraphExec_t g : gs)
    if (g) cudaGraphExecDestroy(g);
  w->g_step = w->g_stage1 = w->g_rest = nullptr;
  w->have = false;
}

// stage 1: k1 = M^-1 R(q), q = x_old + h/2 k1, and (with_norm) the norm of
// k1 weighted by M, sqrt(sum k1^2 M), read back into m->h_red[0]
int rk4_stage1(eg_mesh* m, double* buf, double h, bool with_norm) {
  const int64_t N = m->ndof;
  double *xold = buf, *k1 = buf + N, *res = buf + 4 * N, *qd = buf + 5 * N;
  int st = eg_launch_residual(m, qd, res);
  if (st != EG_OK) return st;
  eg_launch_rk4_stage(m, res, xold, h / 2, k1, qd);
  m->launches += 1;
  if (with_norm) {
    eg_launch_norm(m, k1, 0, m->red + 2048);
    EG_CUDA(cudaMemcpyAsync(m->h_red, m->red + 2048, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  }
  EG_CUDA(cudaGetLastError());
  return EG_OK;
}

// stages 2, 3, 4 and the update of x_old and q
int rk4_rest(eg_mesh* m, double* buf, double h) {
  const int64_t N = m->ndof;
  double *xold = buf, *k1 = buf + N, *k2 = buf + 2 * N, *k3 = buf + 3 * N, *res = buf + 4 * N,
         *qd = buf + 5 * N;
  int st = eg_launch_residual(m, qd, res);
  if (st == EG_OK) {
    eg_launch_rk4_stage(m, res, xold, h / 2, k2, qd);
    st = eg_launch_residual(m, qd, res);
  }
  if (st == EG_OK) {
    eg_launch_rk4_stage(m, res, xold, h, k3, qd);
    st = eg_launch_residual(m, qd, res);
  }
  if (st != EG_OK) return st;
  eg_launch_rk4_final(m, k1, k2, k3, res, h, xold, qd);
  m->launches += 3;
  EG_CUDA(cudaGetLastError());
  return EG_OK;
}

// graphs of the step for (h, the mesh's launch configuration and parameters,
// the stream); false when the stream cannot be captured (the caller falls
// back to eager launches of the same kernels)
bool rk4_graphs(eg_mesh* m, eg_rk4_ws* w, double h) {
  const bool same = w->tried && w->key.h == h && w->key.elem_epb == m->elem_epb &&
                    w->key.vol_mma == m->vol_mma && w->key.stream == m->stream &&
                    std::memcmp(&w->key.params, &m->params, sizeof(eg_params)) == 0;
  if (same) return w->have;
  rk4_graphs_free(w);
  w->tried = true;
  w->key.params = m->params;
  w->key.h = h;
  w->key.elem_epb = m->elem_epb;
  w->key.vol_mma = m->vol_mma;
  w->key.stream = m->stream;
  double* buf = w->buf;
  bool ok = capture_graph(m, [&]() {
    rk4_stage1(m, buf, h, false);
    rk4_rest(m, buf, h);
  }, &w->g_step, &w->n_step);
  ok = ok && capture_graph(m, [&]() { rk4_stage1(m, buf, h, true); }, &w->g_stage1, &w->n_stage1);
  ok = ok && capture_graph(m, [&]() { rk4_rest(m, buf, h); }, &w->g_rest, &w->n_rest);
  if (!ok) rk4_graphs_free(w);
  w->have = ok;
  return ok;
}

int rk4_ws(eg_mesh* m, eg_rk4_ws** out) {
  if (!m->rws) {
    eg_rk4_ws* w = new eg_rk4_ws();
    cudaError_t ce = cudaMalloc((void**)&w->buf, 6 * 8 * (size_t)m->ndof);
    if (ce != cudaSuccess) {
      delete w;
      return eg_cuda_fail(ce, "eg_rk4");
    }
    m->rws = w;
  }
  *out = m->rws;
  return EG_OK;
}

}  // namespace

void eg_rk4_ws_free(eg_mesh* m) {
  eg_rk4_ws* w = m ? m->rws : nullptr;
  if (!w) return;
  rk4_graphs_free(w);
  if (w->buf) cudaFree(w->buf);
  delete w;
  m->rws = nullptr;
}

int eg_rk4_loop(eg_mesh* m, double* buf, double h, double t_max, int itermax, double res_tol,
                bool use_graphs, eg_rk4_stats* out) {
  eg_rk4_ws* w = m->rws;
  const bool graphs = use_graphs && w && w->buf == buf && !eg_timing_on(m) && !m->capturing &&
                      rk4_graphs(m, w, h);
  const bool with_norm = res_tol > 0;
  const long t_steps = lround(t_max / h);
  double t = 0.0, last_norm = 0.0;
  int steps = 0, st = EG_OK;
  // loop i = 2 .. t_steps+1 of the reference (rk4.jl:201)
  for (long i = 2; i <= t_steps + 1; ++i) {
    t = (i - 2) * h;
    const bool stop_after_stage1 = itermax > 0 && i > itermax;
    if (graphs && !with_norm && !stop_after_stage1) {
      cudaError_t ce = cudaGraphLaunch(w->g_step, m->stream);
      if (ce != cudaSuccess) {
        st = eg_cuda_fail(ce, "eg_rk4 graph");
        break;
      }
      m->launches += w->n_step;
      ++steps;
      continue;
    }
    // stage 1 (with the norm, as pde_post_func with calc_norm=true)
    if (graphs && with_norm) {
      cudaError_t ce = cudaGraphLaunch(w->g_stage1, m->stream);
      if (ce != cudaSuccess) {
        st = eg_cuda_fail(ce, "eg_rk4 graph");
        break;
      }
      m->launches += w->n_stage1;
    } else {
      st = rk4_stage1(m, buf, h, with_norm);
      if (st != EG_OK) break;
    }
    if (with_norm) {
      cudaError_t ce = cudaStreamSynchronize(m->stream);
      if (ce != cudaSuccess) {
        st = eg_cuda_fail(ce, "eg_rk4");
        break;
      }
      last_norm = m->h_red[0];
      // the reference breaks after the stage-1 update of q (rk4.jl:258-280)
      if (last_norm < res_tol) break;
    }
    if (stop_after_stage1) break;
    // stages 2, 3, 4
    if (graphs) {
      cudaError_t ce = cudaGraphLaunch(w->g_rest, m->stream);
      if (ce != cudaSuccess) {
        st = eg_cuda_fail(ce, "eg_rk4 graph");
        break;
      }
      m->launches += w->n_rest;
    } else {
      st = rk4_rest(m, buf, h);
      if (st != EG_OK) break;
    }
    ++steps;
  }
  t += h;
  // a failed launch leaves earlier work queued: let it finish before the
  // caller reuses or frees the buffers
  if (st != EG_OK) cudaStreamSynchronize(m->stream);
  if (out) {
    out->steps = steps;
    out->t = t;
    out->res_norm = last_norm;
  }
  return st;
}

extern "C" int eg_rk4(eg_mesh* m, double* q, double h, double t_max, int32_t itermax, double res_tol,
                      int32_t mem, eg_rk4_stats* stats) {
  if (!m || !q || !(h > 0) || (mem != EG_MEM_HOST && mem != EG_MEM_DEVICE)) {
    eg_set_error("eg_rk4: invalid argument");
    return EG_ERR_INVALID;
  }
  int st = eg_check_device(m, "eg_rk4");
  if (st != EG_OK) return st;
  eg_rk4_ws* w = nullptr;
  if ((st = rk4_ws(m, &w)) != EG_OK) return st;
  const int64_t N = m->ndof;
  double* buf = w->buf;
  double* qd = buf + 5 * N;
  // the loop iterates in the mesh's own copy of the state (the graphs are
  // bound to it); x_old starts as the same state
  EG_CUDA(cudaMemcpyAsync(qd, q, 8 * N, mem == EG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                          m->stream));
  EG_CUDA(cudaMemcpyAsync(buf, qd, 8 * N, cudaMemcpyDeviceToDevice, m->stream));
  EG_CUDA(cudaMemsetAsync(m->status, 0, sizeof(unsigned int), m->stream));
  eg_rk4_stats s;
  st = eg_rk4_loop(m, buf, h, t_max, itermax, res_tol, true, &s);
  if (st == EG_OK) {
    cudaError_t ce = cudaMemcpyAsync(m->h_status, m->status, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                     m->stream);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(q, qd, 8 * N, mem == EG_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                           m->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(m->stream);
    if (ce != cudaSuccess) {
      cudaStreamSynchronize(m->stream);
      st = eg_cuda_fail(ce, "eg_rk4");
    } else {
      st = eg_check_status(m);
    }
  }
  if (stats) *stats = s;
  return st;
}

namespace {
// q_hi[e][r] = sum_c T[r][c] q_lo[e][c]
__global__ void k_prolong(const double* __restrict__ T, const double* __restrict__ qlo,
                          double* __restrict__ qhi, int E, int nlo, int nhi) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)E * nhi;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(t / nhi), r = (int)(t - (int64_t)e * nhi);
    const double* x = qlo + (size_t)e * nlo;
    const double* Tr = T + (size_t)r * nlo;
    double acc = 0.0;
    for (int c = 0; c < nlo; ++c) acc = fma(Tr[c], x[c], acc);
    qhi[t] = acc;
  }
}
}  // namespace

extern "C" int eg_prolong(eg_mesh* lo, const double* q_lo, eg_mesh* hi, double* q_hi, const double* T,
                          int32_t mem) {
  if (!lo || !hi || !q_lo || !q_hi || !T || lo->E != hi->E || lo->nv != hi->nv) {
    eg_set_error("eg_prolong: invalid argument (meshes must share their elements)");
    return EG_ERR_INVALID;
  }
  const int nlo = lo->Np * lo->nv, nhi = hi->Np * hi->nv;
  const size_t nT = (size_t)nlo * nhi;
  if (hi->prolong_T_n < nT) {  // device copy of T, kept by the fine mesh
    EG_CUDA(cudaStreamSynchronize(hi->stream));
    if (hi->prolong_T) cudaFree(hi->prolong_T);
    hi->prolong_T = nullptr;
    hi->prolong_T_n = 0;
    EG_CUDA(cudaMalloc((void**)&hi->prolong_T, sizeof(double) * nT));
    hi->prolong_T_n = nT;
  }
  double* dT = hi->prolong_T;
  EG_CUDA(cudaMemcpyAsync(dT, T, sizeof(double) * nT, cudaMemcpyHostToDevice, hi->stream));
  const double* src = q_lo;
  double* dst = q_hi;
  if (mem == EG_MEM_HOST) {
    EG_CUDA(cudaMemcpyAsync(lo->q_dev, q_lo, 8 * (size_t)lo->ndof, cudaMemcpyHostToDevice, hi->stream));
    src = lo->q_dev;
    dst = hi->q_dev;
  }
  k_prolong<<<grid64((int64_t)hi->E * nhi), 256, 0, hi->stream>>>(dT, src, dst, hi->E, nlo, nhi);
  hi->launches += 1;
  EG_CUDA(cudaGetLastError());
  if (mem == EG_MEM_HOST)
    EG_CUDA(cudaMemcpyAsync(q_hi, dst, 8 * (size_t)hi->ndof, cudaMemcpyDeviceToHost, hi->stream));
  EG_CUDA(cudaStreamSynchronize(hi->stream));
  return EG_OK;
}

// RK4 stage launches for other translation units: the kernels, grid and
// launch counting of eg_rk4
void eg_launch_rk4_stage(eg_mesh* m, const double* res, const double* xold, double c, double* ks,
                         double* q) {
  k_rk4_stage<<<grid64(m->ndof), 256, 0, m->stream>>>(res, m->Minv, xold, c, ks, q,
                                                      (int64_t)m->E * m->Np, m->nv);
}

void eg_launch_rk4_final(eg_mesh* m, const double* k1, const double* k2, const double* k3,
                         const double* res, double h, double* xold, double* q) {
  k_rk4_final<<<grid64(m->ndof), 256, 0, m->stream>>>(k1, k2, k3, res, m->Minv, h, xold, q,
                                                      (int64_t)m->E * m->Np, m->nv);
}
