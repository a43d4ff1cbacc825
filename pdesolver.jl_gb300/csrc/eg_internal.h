// eg_internal.h -- device-side mesh object and shared helpers of libeulergpu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "eulergpu.h"

#define EG_MAX_NV 5
#define EG_MAX_NF 16
#define EG_MAX_NP 64
#define EG_MAX_S 64

// device status word bits (set with atomicOr by kernels, read by the host)
#define EG_DEV_NEG_DENSITY 1u
#define EG_DEV_NEG_PRESSURE 2u
#define EG_DEV_NONFINITE 4u
#define EG_DEV_LU_PIVOT 8u

void eg_set_error(const char* fmt, ...);
int eg_cuda_fail(cudaError_t e, const char* what);

#define EG_CUDA(call)                                      \
  do {                                                     \
    cudaError_t _e = (call);                               \
    if (_e != cudaSuccess) return eg_cuda_fail(_e, #call); \
  } while (0)

// Physics constants in the form the kernels read them.
struct DevParams {
  double gamma, gamma_1;
  double Ma, aoa, rho_free, p_free, E_free;
  double r_in, rho_in, M_in;
  double R, cv;
};

// Per-element face table entry: which face-flux slot a local face reads and
// from which side.  slot < I: interface slot; slot >= I: boundary slot.
struct EFace {
  int32_t slot;
  int32_t side;    // 0: element is elementL (or boundary owner), 1: elementR
  int32_t orient;  // nbrperm column for side 1
  int32_t pad;
};

// phase ids of the device timers (eg_timings fields)
enum { EG_PHASE_FACE = 0, EG_PHASE_ELEMENT = 1, EG_PHASE_NORM = 2, EG_PHASE_OTHER = 3, EG_NPHASE = 4 };

struct TimerState;     // event pool (eg_timing.cu)
struct eg_newton_ws;   // cached Newton work objects (eg_solvers.cu)
struct eg_rk4_ws;      // cached RK4 work vectors and step graphs (eg_solvers.cu)

struct eg_mesh {
  // sizes
  int dim, E, Np, Nf, S, F, I, B, nbc, norient, nv;
  int64_t ndof;
  int device;       // CUDA device current when the mesh was created (owns its arrays)
  eg_params params;
  DevParams dp;
  cudaStream_t stream;
  // operator (device)
  double* Q;        // [dim][Np(j)][Np(i)]: Q[k][j][i] = Q_k(i, j)
  double* w;        // [Np]
  double* interp;   // [F][Nf][S]
  int32_t* perm;    // [F][S]
  int32_t* nbrperm; // [norient][Nf]
  double* wface;    // [Nf]
  double* lift;     // [F][Np][Nf]: sum_s [perm[f][s]==j] interp[f][i][s] * wface[i]
  double* liftS;    // [F][Nf][S]: interp[f][i][s] * wface[i]
  int32_t* nbrinv;  // [norient][Nf]: inverse permutations of nbrperm
  int sparse_face;  // interp is the identity on every face (diagonal-E operators)
  // mesh (device)
  double* dxidx;    // [E][Np][dim][dim]
  double* jac;      // [E][Np]
  double* Minv;     // [E][Np] = jac / w
  int32_t* ifaces;  // [I][5]
  double* nrm_face; // [I][Nf][dim]
  int32_t* bfaces;  // [B][2]
  int32_t* bc_of_b; // [B] boundary condition of each boundary face
  double* coords_bndry; // [B][Nf][dim]
  double* nrm_bndry;    // [B][Nf][dim]
  double* qg_bndry;     // [B][Nf][nv] Dirichlet states (time-independent, set at creation)
  EFace* eface;     // [E][F]
  // work buffers (device)
  double* fflux;    // [(I+B)][Nf][nv] face fluxes times wface
  double* q_dev;    // [ndof] staging for host inputs
  double* res_dev;  // [ndof] staging for host outputs
  unsigned int* status;   // device status word
  double* red;      // reduction scratch
  unsigned int* h_status; // pinned host mirror
  double* h_red;          // pinned host scalar
  cudaStream_t own_stream;  // the library's stream (stream may be a caller's)
  TimerState* timer;        // phase timers (null until enabled)
  int64_t launches;         // kernel launches since creation
  int32_t h_bndry_offsets[64];  // host copy of the BC-group offsets
  bool capturing;           // a CUDA graph is being captured on `stream`
  eg_newton_ws* nws;        // Newton operator / preconditioner / solver / vectors, kept
                            // between solves (released by eg_newton_release or destroy)
  eg_rk4_ws* rws;           // RK4 work vectors and step graphs, kept between eg_rk4 calls
  double* prolong_T;        // device copy of the last prolongation matrix (eg_prolong)
  size_t prolong_T_n;
  // launch configuration of the element kernels (eg_set_launch_config /
  // eg_autotune); 0 = the built-in choice
  int elem_epb;             // elements per CTA
  int vol_mma;              // weak-form Q^T F on the FP64 tensor cores (mma.sync m8n8k4)
};
void eg_newton_ws_free(eg_mesh* m);
void eg_rk4_ws_free(eg_mesh* m);
// EG_OK when the calling thread's current device is the mesh's and the mesh
// stream belongs to it; EG_ERR_INVALID (with a message naming `who`) otherwise
int eg_check_device(const eg_mesh* m, const char* who);
// The RK4 step loop of eg_rk4 (reference rk4.jl:201-330) on the device
// buffers buf[6][ndof] = x_old, k1, k2, k3, res, q, with q = x_old = the
// start state already in place and the status word cleared.  use_graphs:
// replay captured CUDA graphs of the step (the mesh keeps them) where the
// stream can be captured.  On return the stream has no work of the loop left
// when the status is not EG_OK.
int eg_rk4_loop(eg_mesh* m, double* buf, double h, double t_max, int itermax, double res_tol,
                bool use_graphs, eg_rk4_stats* out);

// phase timers: bracket a group of launches on m->stream
void eg_phase_begin(eg_mesh* m, int phase);
void eg_phase_end(eg_mesh* m, int phase, int nlaunch);
void eg_timer_free(eg_mesh* m);

// kernels entry points used across translation units
int eg_residual_device(eg_mesh* m, const double* q, double* res);
// the element kernel alone (volume + face lifting from m->fflux), with the
// mesh's launch configuration
int eg_launch_element(eg_mesh* m, const double* q, double* res);
// effective launch shape of the element kernel: elements per CTA, threads,
// dynamic shared memory; EG_ERR_INVALID if the configuration does not fit
int eg_element_shape(const eg_mesh* m, int epb, int mma, int* threads, size_t* smem);
int eg_check_status(eg_mesh* m);
// phase timers enabled (they take CUDA events from a growing pool)
bool eg_timing_on(const eg_mesh* m);
// the RK4 stage kernels of eg_rk4 on m->stream (eg_solvers.cu)
void eg_launch_rk4_stage(eg_mesh* m, const double* res, const double* xold, double c, double* ks,
                         double* q);
void eg_launch_rk4_final(eg_mesh* m, const double* k1, const double* k2, const double* k3,
                         const double* res, double h, double* xold, double* q);
