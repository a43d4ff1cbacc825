// eg_linalg.h -- Jacobian operator, block-Jacobi preconditioner and GMRES
// objects behind the eg_lo / eg_pc / eg_ls handles of the C ABI.
#pragma once
#include <mutex>

#include "eg_internal.h"

struct eg_lo {
  eg_mesh* mesh;
  int prec;        // EG_F64 / EG_F32
  int n;           // Np * nv: element block size
  int nb;          // S * nv: coupling block size
  void* diag;      // [E][n][n] column-major element blocks
  void* cpl;       // [I][2][nb][nb] row-major coupling blocks; face-diagonal
                   // (cpl_sparse): [I][2][S][nv][nv], see eg_lo_coupling_size
  int cpl_sparse;  // the face operator is the identity on the stencil (face
                   // nodes are volume nodes): row stencil node s couples only
                   // to the neighbour's node facing it
  void* dF;        // [(I+B)][Nf][2][nv][nv] point flux Jacobians
  int32_t* spos;   // [F][Np]: stencil position of node j on face f, or -1
  int32_t* fside;  // [E][F]: coupling block (slot * 2 + side) of face f of e, or -1
  void* xT;        // [ndof] operand in the operator precision
  void* yT;        // [ndof]
  double* xd;      // [ndof] FP64 staging
  double* yd;      // [ndof]
  bool valid;      // blocks computed
};

struct eg_pc {
  eg_lo* lo;
  void* inv;       // [E][n][n] column-major inverses of the element blocks
  bool valid;
};

struct eg_ls {
  eg_lo* lo;
  eg_pc* pc;
  int m;           // restart length
  double reltol, abstol, dtol;
  int itermax;
  void* V;         // [(m+1)][ndof]
  void* w;         // [ndof]
  void* z;         // [ndof]
  void* cfs;       // [I][2][nb] coupling products of each face side (persistent Arnoldi)
  void* xT;        // [ndof]
  void* bT;        // [ndof]
  void* part;      // [nblk][m+2] partial sums (operator precision)
  void* h;         // [m+2] device Hessenberg column (operator precision)
  double* hh;      // pinned host copy [m+2]
  void* y;         // [m+1] device least-squares solution
  double* xd;      // [ndof] FP64 staging
  double* bd;      // [ndof]
  int nblk;
  int coop_grid;   // blocks of the persistent GMRES grid (0: automatic)
  // device-side GMRES state (eg_gmres.cu)
  double* dH;      // H | cs | sn | g | y  (FP64)
  int* dflags;     // done, jdone, its, converged, itermax
  double* dscal;   // tol, resid, beta, bnorm, reltol, abstol
  void* g_init;    // cudaGraphExec_t: residual + cycle initialisation
  void* g_cycle;   // cudaGraphExec_t: one restart cycle + update + re-initialisation
  int64_t g_init_nodes, g_cycle_nodes;
  bool graphs_ok;  // capture succeeded (else the same launches run eagerly)
  // transposed solves (linearSolveTranspose): the same cycle on J^T M^-T,
  // with graphs of its own
  int trans;       // the enqueue functions build the transposed cycle
  void* g_init_t;
  void* g_cycle_t;
  int64_t g_init_t_nodes, g_cycle_t_nodes;
  bool graphs_t_ok, graphs_t_tried;
  // batched persistent GMRES: the solve's kernel arguments (device copy and
  // pinned staging) and the event marking them ready on the mesh stream
  void* dargs;
  void* hargs;
  cudaEvent_t ev_in;
};
void eg_gmres_release(eg_ls* ls);
// slots of the device GMRES state: dflags[] and dscal[]
enum { F_DONE = 0, F_JDONE = 1, F_ITS = 2, F_CONV = 3, F_ITERMAX = 4, F_REORTH = 5, F_CYCLES = 6, F_NREORTH = 7 };
enum { S_TOL = 0, S_RESID = 1, S_BETA = 2, S_BNORM = 3, S_RELTOL = 4, S_ABSTOL = 5, S_BETA0 = 6 };
// the whole GMRES solve as one persistent cooperative kernel (eg_arnoldi.cu)
#define EG_COOP_MAX_BLOCKS 1024
// blocks of the thread-block cluster that runs a small system's GMRES solve
// (16, a non-portable cluster size, measured faster than 8 on GB300; 8 is
// taken where a 16-block cluster cannot be placed)
#ifndef EG_GMRES_CLUSTER_BLOCKS
#define EG_GMRES_CLUSTER_BLOCKS 16
#endif
// blocks of the stream GMRES path's reduction kernels (4 per SM)
#define EG_GMRES_STREAM_BLOCKS 608
// partial-sum slots of a GMRES(m) solver: the stream path's [blocks][m+2][2]
// or the persistent kernel's [4][blocks][33], whichever is larger
inline size_t eg_gmres_partials(int m) {
  const size_t a = (size_t)EG_GMRES_STREAM_BLOCKS * (m + 2) * 2, b = (size_t)4 * EG_COOP_MAX_BLOCKS * 33;
  return a > b ? a : b;
}
int eg_gmres_coop(eg_ls* ls);
// the persistent solve of a small system by one cluster of C blocks
// (EG_ERR_UNSUPPORTED when no such cluster can be placed)
int eg_gmres_cluster(eg_ls* ls, int C);
// one cooperative GMRES grid at a time per device (held across launch and
// completion of multi-block grids, single or batched)
std::mutex& eg_coop_mutex(int dev);
// batched persistent GMRES (eg_arnoldi_batch.cu): on when enabled by
// eg_set_gmres_batching; eg_gmres_coop then hands the solve to the batcher
bool eg_gmres_batching();
int eg_gmres_coop_batched(eg_ls* ls);
// blocks the persistent GMRES kernel gives this solver's system (alone or in
// a batch)
int eg_gmres_wanted_blocks(const eg_ls* ls);
// threads inside eg_newton_solve on a device with a multi-block Krylov solve
// while batching is on (the batcher waits for their solves before launching)
void eg_batch_enter(int dev);
void eg_batch_leave(int dev);
bool eg_coop_supported();
// the persistent kernel handles this system (device support, coupling blocks
// of at most 64 rows, small face tables)
bool eg_coop_usable(const eg_ls* ls);

// kernels shared across translation units
int eg_jacobian_launch(eg_lo* lo, const double* q);
// y = J x in the operator precision (device pointers of that precision);
// with `done` non-null the launch does nothing while *done != 0
int eg_lo_apply_T(eg_lo* lo, const void* x, void* y, const int* done = nullptr);
// values of the coupling storage: I*2*nb*nb, or I*2*S*nv*nv when face-diagonal
size_t eg_lo_coupling_size(const eg_lo* lo);
// w = v + C z: the preconditioned operator J M^-1 v with z = M^-1 v, using the
// coupling blocks only (the element blocks times their inverses are I)
int eg_cpl_apply_T(eg_lo* lo, const void* v, const void* z, void* w, const int* done = nullptr);
// y = M^-1 x in the operator precision
int eg_pc_apply_T(eg_pc* pc, const void* x, void* y, const int* done = nullptr);
// the transposes, in the operator precision: y = J^T x; w = v + C^T z (the
// transposed right-preconditioned operator J^T M^-T v with z = M^-T v); y = M^-T x
int eg_lo_apply_t_T(eg_lo* lo, const void* x, void* y, const int* done = nullptr);
int eg_cpl_apply_t_T(eg_lo* lo, const void* v, const void* z, void* w, const int* done = nullptr);
int eg_pc_apply_t_T(eg_pc* pc, const void* x, void* y, const int* done = nullptr);
// precision conversion helpers (device)
int eg_convert(eg_mesh* m, const double* src, void* dst, int prec, int64_t n, double scale);
int eg_convert_back(eg_mesh* m, const void* src, double* dst, int prec, int64_t n);
// x_T <- GMRES solution of J x = b_T (or J^T x = b_T with `transpose`);
// returns status, fills stats
int eg_gmres_T(eg_ls* ls, const void* bT, void* xT, eg_ls_stats* st, int transpose = 0);
