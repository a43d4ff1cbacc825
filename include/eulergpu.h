/*
 * eulergpu.h -- C ABI of libeulergpu.so, the GB300 (sm_103a) implementation of
 * the Euler summation-by-parts hot path of PDESolver.jl:
 *   residual evaluation, explicit element Jacobian assembly (block-sparse),
 *   block-Jacobi preconditioned GMRES, Newton steady solves and RK4 stepping.
 *
 * Conventions
 *   - Every entry point returns an eg_status (0 = EG_OK).  No C++ exception
 *     crosses the ABI; eg_last_error() gives a message for the calling thread.
 *   - Index arrays are 0-based int32.  A Julia caller subtracts 1 from its
 *     1-based Interface/Boundary fields.
 *   - Floating-point arrays use the reference's column-major layouts read in
 *     reverse index order (q[nv, Np, E] in Julia == q[E][Np][nv] here), so a
 *     Julia caller passes its own arrays without copies.
 *   - Arrays passed to eg_mesh_create are copied to the device; the caller
 *     keeps ownership of its host arrays.  The library owns every device
 *     buffer it allocates and releases it in the matching *_destroy call.
 *   - State/residual pointers are host or device memory as the `mem` flag of
 *     each call says (EG_MEM_HOST / EG_MEM_DEVICE).
 *   - Each eg_mesh owns one CUDA stream.  Calls on one eg_mesh are not
 *     thread-safe; different meshes may be driven from different threads.
 */
#ifndef EULERGPU_H
#define EULERGPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  EG_OK = 0,
  EG_ERR_INVALID = 1,        /* bad argument / inconsistent sizes            */
  EG_ERR_CUDA = 2,           /* CUDA runtime error                           */
  EG_ERR_OOM = 3,            /* device allocation failed                     */
  EG_ERR_NEG_DENSITY = 4,    /* rho <= 0 at a node (reference euler.jl:543)  */
  EG_ERR_NEG_PRESSURE = 5,   /* p <= 0 at a node (reference euler.jl:586)    */
  EG_ERR_NONFINITE = 6,      /* NaN/Inf in a residual or update              */
  EG_ERR_LU_PIVOT = 7,       /* zero pivot in a block LU factorisation       */
  EG_ERR_KRYLOV = 8,         /* GMRES breakdown / not converged              */
  EG_ERR_NOT_CONVERGED = 9,  /* Newton did not reach its tolerances          */
  EG_ERR_TIMEOUT = 10,       /* bounded device wait gave up                  */
  EG_ERR_UNSUPPORTED = 11    /* option combination not built                 */
} eg_status;

typedef enum { EG_MEM_HOST = 0, EG_MEM_DEVICE = 1 } eg_mem;

/* numerical flux names (reference FluxDict, src/solver/euler/flux.jl) */
typedef enum { EG_FLUX_ROE = 0, EG_FLUX_IR = 1 } eg_flux;

/* boundary condition functors (reference BCDict, src/solver/euler/bc.jl):
   isentropicVortexBC (bc.jl:542-568), FreeStreamBC (bc.jl:1562-1647),
   noPenetrationESBC (bc.jl:767-795: mirror state and Lax-Friedrichs flux,
   entropy stable with diagonal-E operators) */
typedef enum { EG_BC_VORTEX = 0, EG_BC_FREESTREAM = 1, EG_BC_NOPENETRATION_ES = 2 } eg_bc;

/*
 * Physics parameters: the subset of ParamType / opts the hot path reads
 * (reference src/solver/euler/types.jl:236-260, src/input/read_input.jl).
 */
typedef struct {
  double gamma;              /* opts["gamma"], 1.4                              */
  double Ma;                 /* opts["Ma"], free-stream Mach number             */
  double aoa;                /* angle of attack in radians (types.jl:247)       */
  double rho_free;           /* 1.0 (types.jl:249)                              */
  double p_free;             /* opts["p_free"], default 1/gamma                 */
  double vortex_r_in;        /* isentropic vortex inner radius (1)              */
  double vortex_rho_in;      /* density at the inner radius (2)                 */
  double vortex_M_in;        /* Mach number at the inner radius.  The reference
                                hard-codes 0.95 (common_funcs.jl:43-45); it is
                                a parameter here.                               */
  int32_t face_flux;         /* eg_flux at interior faces, opts["Flux_name"]    */
  int32_t volume_integral_type; /* 1: Q^T F weak form; 2: Hadamard split form  */
  int32_t volume_flux;       /* eg_flux of the split form, "Volume_flux_name"   */
  int32_t reserved;
} eg_params;

/*
 * Mesh + SBP operator description (reference AbstractMesh fields,
 * docs/src/interfaces.md:210-470, and sbp / sbpface fields).
 *   E  = numEl, Np = numNodesPerElement, Nf = numNodesPerFace,
 *   F  = faces per element (dim+1), S = face stencil size,
 *   I  = numInterfaces, B = numBoundaryFaces, nv = dim+2.
 */
typedef struct {
  int32_t dim;               /* 2 or 3                                          */
  int32_t num_el;            /* E                                               */
  int32_t nodes_per_el;      /* Np                                              */
  int32_t nodes_per_face;    /* Nf                                              */
  int32_t stencil_size;      /* S                                               */
  int32_t num_interfaces;    /* I                                               */
  int32_t num_bndry;         /* B                                               */
  int32_t num_bc;            /* number of boundary-condition groups             */
  int32_t num_orient;        /* columns of nbrperm                              */
  int32_t reserved;
  /* SBP volume operator: Q[dim][Np][Np] with Q[k][j][i] = Q_k(i, j)
     (Julia sbp.Q[i, j, k]); w[Np] the diagonal norm (sbp.w)                   */
  const double* Q;
  const double* w;
  /* SBP face operator: interp[F][Nf][S] (sbpface.interp, per local face),
     perm[F][S] stencil volume nodes (sbpface.perm), nbrperm[num_orient][Nf]
     (sbpface.nbrperm), wface[Nf] (sbpface.wface)                              */
  const double* interp;
  const int32_t* perm;
  const int32_t* nbrperm;
  const double* wface;
  /* element metrics: dxidx[E][Np][dim(x)][dim(xi)] = |J| dxi_k/dx_p
     (Julia mesh.dxidx[k, p, j, e]); jac[E][Np] = det(dxi/dx); coords[E][Np][dim] */
  const double* dxidx;
  const double* jac;
  const double* coords;
  /* interfaces[I][5] = (elementL, elementR, faceL, faceR, orient);
     nrm_face[I][Nf][dim] scaled normal outward from elementL                  */
  const int32_t* interfaces;
  const double* nrm_face;
  /* bndryfaces[B][2] = (element, face); bndry_offsets[num_bc + 1];
     bc_types[num_bc] (eg_bc); coords_bndry / nrm_bndry [B][Nf][dim]           */
  const int32_t* bndryfaces;
  const int32_t* bndry_offsets;
  const int32_t* bc_types;
  const double* coords_bndry;
  const double* nrm_bndry;
} eg_mesh_desc;

typedef struct eg_mesh eg_mesh;

/* ---- library ------------------------------------------------------------ */
int eg_version(void);
/* message of the last failing call on this thread */
const char* eg_last_error(void);

/* ---- mesh / equation object (reference createObjects, startup_func.jl:45) */
int eg_mesh_create(const eg_mesh_desc* desc, const eg_params* params, eg_mesh** out);
int eg_mesh_destroy(eg_mesh* mesh);
/* number of degrees of freedom E*Np*nv */
int64_t eg_mesh_num_dof(const eg_mesh* mesh);

/*
 * evalResidual (reference src/solver/euler/euler.jl:111; interface.jl:33):
 * res is overwritten with R(q) (weak form, not multiplied by M^-1).
 * q, res: [E][Np][nv] in host or device memory per `mem`.
 * Returns EG_ERR_NEG_DENSITY / EG_ERR_NEG_PRESSURE if a node has rho <= 0 or
 * p <= 0 (reference checkDensity / checkPressure, euler.jl:543-611).
 */
int eg_eval_residual(eg_mesh* mesh, const double* q, double* res, double t, int32_t mem);

/*
 * calcNorm (reference src/Utils/Utils.jl:427-449):
 * strongres = 0: sqrt(sum r^2 M); strongres = 1: sqrt(sum r^2 M^-1).
 */
int eg_calc_norm(eg_mesh* mesh, const double* r, int32_t strongres, int32_t mem, double* out);

/*
 * Boundary functional: integral of the pressure over the faces of one
 * boundary-condition group, sum_b sum_i wface_i p(q_face) |nrm_bndry|
 * (the SBP face quadrature of the reference's integratefunctional!,
 * boundary_functional.jl:82-126).  For the quarter annulus, group 0 is r = 1.
 */
int eg_calc_functional(eg_mesh* mesh, const double* q, int32_t bc_group, int32_t mem, double* out);

/* calcMaxWaveSpeed (reference src/solver/euler/euler_funcs.jl:1810-1834):
   max over the nodes of a + |u|, the wave speed of the CFL time step
   delta_t = CFL * min_el_size / wave_speed (startup_func.jl:241-247). */
int eg_calc_max_wave_speed(eg_mesh* mesh, const double* q, int32_t mem, double* out);

/* ---- streams, asynchronous launch and phase timers ---------------------- */

/* Run this mesh's work on `stream` (a cudaStream_t; NULL is CUDA's default
   stream), or on the library's own stream when use_own != 0.  Lets a caller
   order library work with its own kernels and CUDA events.  A stream of
   another device than the mesh's is refused (EG_ERR_INVALID). */
int eg_mesh_set_stream(eg_mesh* mesh, void* stream, int32_t use_own);

/* evalResidual with device pointers, enqueued on the mesh stream without a
   host synchronisation; the density/pressure checks are reported by the next
   eg_sync. */
int eg_eval_residual_async(eg_mesh* mesh, const double* q_dev, double* res_dev);

/* Wait for the mesh stream and report (and clear) the device status word. */
int eg_sync(eg_mesh* mesh);

/*
 * Per-phase device timers (reference Timings struct, src/Utils/Utils.jl:567):
 * when enabled, CUDA events bracket every kernel the library launches; the
 * sums are in milliseconds.  `launches` counts every kernel launched since
 * the mesh was created (timers on or off).
 */
typedef struct {
  double t_face_flux;    /* interface + boundary numerical fluxes          */
  double t_element;      /* volume integrals + face lifting                */
  double t_norm;         /* calcNorm reductions                            */
  double t_other;        /* everything else                                */
  int64_t launches;      /* kernel launches since creation                 */
  int64_t timed;         /* launches covered by the sums                   */
} eg_timings;

int eg_set_timing(eg_mesh* mesh, int32_t enable);
/* synchronises the mesh stream, returns the sums since the last reset */
int eg_get_timings(eg_mesh* mesh, eg_timings* out);
int eg_reset_timings(eg_mesh* mesh);

/* ---- Jacobian, preconditioner, Krylov solver ----------------------------
 * Reference: src/linearsolvers/LinearSolvers.jl:68-660 (LinearSolver,
 * AbstractPC, AbstractLO), ls_standard.jl:28-511, src/jacobian/jacobian.jl,
 * src/NonlinearSolvers/preconditioning*.jl.
 *
 * The explicit Jacobian is stored element-block sparse: one dense
 * (Np nv) x (Np nv) block per element (volume terms + the element's own face
 * terms: the reference's element and LL/RR blocks) and two (S nv) x (S nv)
 * coupling blocks per interface (LR, RL).  Blocks are column-major:
 *   diag[e][col = m*nv + b][row = j*nv + a] = dR(e,j,a) / dq(e,m,b)
 *   coupling[n][0][col = s'*nv + b][row = s*nv + a]
 *       = dR(elementL, perm[faceL][s], a) / dq(elementR, perm[faceR][s'], b)
 *   coupling[n][1][...] the same with L and R exchanged.
 */
typedef enum { EG_F64 = 0, EG_F32 = 1 } eg_precision;

typedef struct eg_lo eg_lo;   /* explicit Jacobian operator (AbstractLO)   */
typedef struct eg_pc eg_pc;   /* element block-Jacobi (NewtonBDiagPC)      */
typedef struct eg_ls eg_ls;   /* right-preconditioned GMRES(m)             */

int eg_lo_create(eg_mesh* mesh, int32_t precision, eg_lo** out);
int eg_lo_destroy(eg_lo* lo);
/* calcLinearOperator -> evalJacobian (reference evalJacobian.jl:6-72,
   jacobian.jl:69-176): J = dR/dq at q, overwriting the blocks.  Weak-form
   volume (volume_integral_type 1) or the entropy-stable split form
   (volume_integral_type 2, reference calcVolumeIntegralsSplitForm_diff,
   euler_funcs_diff.jl:330-430); Roe or IR faces. */
int eg_lo_calc(eg_lo* lo, const double* q, int32_t mem);
/* applyLinearOperator: y = J x; x, y FP64 in host or device memory */
int eg_lo_apply(eg_lo* lo, const double* x, double* y, int32_t mem);
/* y = J x with x, y device arrays in the operator's own precision (double
   for EG_F64, float for EG_F32), no conversion; enqueued, no synchronisation */
int eg_lo_apply_native(eg_lo* lo, const void* x, void* y);
/* applyLinearOperatorTranspose (reference LinearSolvers.jl:533,
   lo_petscmat.jl:143-160): y = J^T x; x, y FP64 in host or device memory */
int eg_lo_apply_transpose(eg_lo* lo, const double* x, double* y, int32_t mem);
/* copy the blocks to host FP64 arrays: diag [E][Np nv][Np nv],
   coupling [I][2][S nv][S nv] (either may be NULL) */
int eg_lo_get_blocks(eg_lo* lo, double* diag, double* coupling);

/* calcPC / applyPC of the element block-Jacobi preconditioner (reference
   preconditioning.jl:7-139: LU with partial pivoting per element block).
   The factors are turned into explicit block inverses so applyPC is a
   batched dense matrix-vector product. */
int eg_pc_create(eg_lo* lo, eg_pc** out);
int eg_pc_destroy(eg_pc* pc);
int eg_pc_calc(eg_pc* pc);
int eg_pc_apply(eg_pc* pc, const double* x, double* y, int32_t mem);
/* y = M^-1 x in the operator's own precision on device arrays, enqueued */
int eg_pc_apply_native(eg_pc* pc, const void* x, void* y);
/* applyPCTranspose (reference LinearSolvers.jl:277): y = M^-T x */
int eg_pc_apply_transpose(eg_pc* pc, const double* x, double* y, int32_t mem);

typedef struct {
  int32_t iters;        /* total Krylov iterations                          */
  int32_t restarts;
  int32_t converged;    /* 1 if ||b - A x|| <= max(reltol ||b||, abstol)     */
  int32_t reorth;       /* Arnoldi steps that took a second Gram-Schmidt pass */
  double res0;          /* ||b - A x0||                                     */
  double res_final;     /* final (estimated) residual norm                  */
} eg_ls_stats;

/* GMRES(restart), right preconditioned, classical Gram-Schmidt with one
   re-orthogonalisation (the reference uses PETSc GMRES(30) with modified
   Gram-Schmidt, read_input.jl:559-569).  Vectors are in the operator's
   precision; b and x are FP64 at the interface. */
int eg_ls_create(eg_lo* lo, eg_pc* pc, int32_t restart, eg_ls** out);
int eg_ls_destroy(eg_ls* ls);
/* setTolerances (ls_standard.jl); negative values leave a field unchanged */
int eg_ls_set_tolerances(eg_ls* ls, double reltol, double abstol, double dtol, int32_t itermax);
/* Blocks of the persistent GMRES kernel (one per SM at most, as a
   cooperative grid; 0 restores the automatic choice: one thread-block
   cluster of 16 blocks (8 where 16 cannot be placed) for operators of at
   most 2 MB or systems of at most 16 x 32 elements, else one block per SM,
   at most one per element).  A tuning knob with no reference
   counterpart; the result does not depend on it beyond the order of the FP
   reductions. */
int eg_ls_set_grid(eg_ls* ls, int32_t blocks);
/* Batched persistent GMRES (process-wide switch; no reference counterpart).
   When enabled, the multi-block Krylov solves that threads reach within
   window_us of each other (or as soon as every thread inside eg_newton_solve
   with such a solve has reached one) run as one cooperative launch: each
   solve keeps the blocks it gets alone, solves are packed while their blocks
   fit on the SMs, and barriers cover a solve's own blocks only.  One-block
   solves launch at once (they share the GPU without batching).  Meant for many meshes solved at once on different threads/streams
   (batches, serving).  A solve's result does not depend on the batch it runs
   in.  Off by default. */
int eg_set_gmres_batching(int32_t enable, double window_us);
/* linearSolve: x <- A^-1 b (x is also the initial guess) */
int eg_ls_solve(eg_ls* ls, const double* b, double* x, int32_t mem, eg_ls_stats* stats);
/* linearSolveTranspose (reference ls_standard.jl:230-244, the adjoint solve of
   calcAdjoint): x <- A^-T b by GMRES(restart) right-preconditioned with the
   transposed block-Jacobi inverses, on J^T M^-T = I + C^T D^-T (coupling
   blocks applied transposed, element blocks cancel); same tolerances, device
   Hessenberg and Givens, and restart cycles replayed as CUDA graphs as the
   forward solve's stream path.  x is also the initial guess. */
int eg_ls_solve_transpose(eg_ls* ls, const double* b, double* x, int32_t mem, eg_ls_stats* stats);

/* ---- Newton and RK4 drivers ------------------------------------------- */
typedef struct {
  double res_abstol;        /* opts["res_abstol"]  (read_input.jl:414)      */
  double res_reltol;        /* opts["res_reltol"]                           */
  double step_tol;          /* opts["step_tol"]                             */
  double krylov_reltol;     /* opts["krylov_reltol"] (1e-2)                 */
  int32_t itermax;          /* Newton iterations                            */
  int32_t krylov_itermax;   /* opts["krylov_itermax"]                       */
  int32_t gmres_restart;    /* 30                                           */
  int32_t precision;        /* EG_F64: all FP64; EG_F32: FP32 Jacobian,
                               preconditioner and Krylov, FP64 residual and
                               update (inexact Newton)                      */
  int32_t globalize_euler;  /* opts["newton_globalize_euler"]: pseudo-
                               transient continuation, J - M/tau_vec with
                               tau_vec = tau/(1 + sqrt(jac)) and tau scaled by
                               |R|_{i-1}/|R|_i each iteration (reference
                               globalization.jl:165-320)                    */
  double euler_tau;         /* opts["euler_tau"], initial tau (1.0)          */
} eg_newton_opts;

typedef struct {
  int32_t iters;            /* Newton iterations taken                      */
  int32_t krylov_iters;     /* total GMRES iterations                       */
  int32_t converged;
  int32_t graph_iters;      /* iterations run as CUDA graphs (0: eager path) */
  double res_norm0;         /* calcNorm(R(q0), strongres) (physicsRhs)       */
  double res_norm;          /* final                                        */
  double step_norm;         /* last ||dq||_2                                */
  double t_residual, t_jacobian, t_pc, t_krylov;   /* device ms per phase   */
} eg_newton_stats;

/* newton / newtonInner (reference src/NonlinearSolvers/newton.jl:54-304):
   q <- q + dq until calcNorm(R(q), M^-1) < res_abstol, or the relative
   norm < res_reltol, or ||dq|| <= step_tol.  q is FP64 in host or device
   memory.  The Jacobian, preconditioner, Krylov basis and work vectors are
   kept by the mesh after the first solve (for this precision and restart
   length), so later solves on the mesh allocate nothing.  When the persistent
   GMRES kernel takes the system and the phase timers are off, each iteration
   runs as three CUDA graphs around the GMRES launch with one synchronisation
   (captured on the first solve, on the mesh stream, which must not be the
   legacy default stream; else the same launches run eagerly, with the same
   results); q is then iterated in a copy the mesh owns and written back at
   the end, also when Newton stops unconverged (not after a device error). */
int eg_newton_solve(eg_mesh* mesh, double* q, int32_t mem, const eg_newton_opts* opts,
                    eg_newton_stats* stats);

/*
 * Degree prolongation between two eg_mesh objects on the same elements
 * (p-continuation, the reference's p_homotopy idea): q_hi[e] = T q_lo[e] for
 * every element, T[Np_hi*nv][Np_lo*nv] row-major (host pointer, copied);
 * q_lo, q_hi in host or device memory per `mem`.
 */
int eg_prolong(eg_mesh* lo, const double* q_lo, eg_mesh* hi, double* q_hi, const double* T,
               int32_t mem);

typedef struct {
  int32_t steps;            /* time steps taken                             */
  int32_t reserved;
  double t;                 /* final time                                   */
  double res_norm;          /* last stage-1 norm sqrt(sum (M^-1 R)^2 M)     */
} eg_rk4_stats;

/* New physics parameters for an existing mesh (the reference changes
   eqn.params / opts between solves, e.g. the Mach number of a sweep).  The
   boundary Dirichlet states are re-evaluated; the mesh stream is synchronised.
   The Newton work objects the mesh keeps stay valid. */
int eg_mesh_set_params(eg_mesh* mesh, const eg_params* params);

/*
 * Device-memory estimate from mesh counts (reference src/estimateMem.jl:1-78,
 * which sums the mesh and solution array sizes from numEl, numInterfaces,
 * nodes per element and dofs per node).  Here the sums cover every device
 * array this library allocates for the mesh (eg_mesh_create), the caller's
 * q and res, and, when newton_precision is EG_F64 or EG_F32, the Newton work
 * objects of eg_newton_solve (Jacobian, block-Jacobi inverses, GMRES basis,
 * Newton vectors).  Each array is rounded up to 512 bytes.
 */
typedef struct {
  int32_t dim, num_el, nodes_per_el, nodes_per_face, stencil_size;
  int32_t num_interfaces, num_bndry, num_orient;
  int32_t newton_precision;   /* EG_F64, EG_F32, or -1: mesh and state only   */
  int32_t gmres_restart;      /* restart length of the Newton GMRES (1..31)   */
  int32_t prolong_from_nodes; /* Np of the coarser level this mesh is
                                 prolonged from (eg_prolong), 0: none         */
  int32_t face_diagonal;      /* 1: the face interpolation is the identity
                                 (face nodes are volume nodes, as for the
                                 diagonal-E operators); the coupling blocks
                                 then keep one nv x nv block per stencil node */
} eg_mem_query;

typedef struct {
  uint64_t mesh, eqn, jacobian, pc, krylov, newton, total;  /* bytes          */
  int64_t allocations;        /* device arrays counted                        */
} eg_mem_estimate;

int eg_estimate_mem(const eg_mem_query* query, eg_mem_estimate* out);

/*
 * Launch configuration of the element kernel (no reference counterpart: the
 * reference's element loops are plain Julia).  elements_per_cta: elements a
 * CTA owns (0: built-in choice, 256 / Np for the weak form); volume_mma: 1 runs
 * the weak-form volume contraction Q^T F on the FP64 tensor cores (mma.sync
 * m8n8k4) instead of CUDA cores (weak form only).  Results of the two
 * contraction kinds agree to FP64 round-off.
 */
typedef struct {
  int32_t elements_per_cta;
  int32_t volume_mma;
  int32_t reserved[2];
} eg_launch_config;

typedef struct {
  eg_launch_config config;
  double ms;                 /* mean element-kernel time of the candidate       */
} eg_tune_entry;

int eg_set_launch_config(eg_mesh* mesh, const eg_launch_config* config);
int eg_get_launch_config(eg_mesh* mesh, eg_launch_config* config);
/* Autotuner: times every admissible configuration (elements per CTA 1, 2,
   4, ... up to 1024 threads, times CUDA-core / tensor-core contraction) on
   the state q_dev (device, [E][Np][nv]) over `reps` launches each, with CUDA
   events on the mesh stream, and keeps the fastest on the mesh.  Up to
   max_entries timings go to `table` (n_entries set to their count).
   Synchronises the mesh stream; not allowed during stream capture. */
int eg_autotune(eg_mesh* mesh, const double* q_dev, int32_t reps, eg_tune_entry* table,
                int32_t max_entries, int32_t* n_entries);

/* Frees the work objects a mesh keeps between solves: Newton's operator,
   preconditioner, Krylov basis and vectors, and eg_rk4's work vectors and
   step graphs (the reference frees its linear solver with `free(ls)`,
   LinearSolvers.jl).  Mesh destroy frees them too. */
int eg_newton_release(eg_mesh* mesh);

/* rk4 (reference src/NonlinearSolvers/rk4.jl:144-336, 404-456): classical
   4-stage RK4 on dq/dt = M^-1 R(q) with step h for round(t_max/h) steps
   (fewer if itermax > 0 is reached, or if res_tol > 0 and the stage-1 norm
   drops below it).  The first call on a mesh allocates six state-sized work
   vectors (48 bytes per unknown) that the mesh keeps (eg_newton_release or
   destroy frees them).  With the phase timers off and a mesh stream that can
   be captured (not the legacy default stream), each time step is replayed as
   a CUDA graph captured on first use for this h (one graph per step; with
   res_tol > 0, one for stage 1 with the norm read-back and one for stages
   2-4); otherwise the same kernels launch one by one, with the same results.
   q (host or device per `mem`) is copied in at the start and written back at
   the end, not after a device error. */
int eg_rk4(eg_mesh* mesh, double* q, double h, double t_max, int32_t itermax, double res_tol,
           int32_t mem, eg_rk4_stats* stats);

/* Largest mesh (unknowns) eg_rk4_static accepts. */
#define EG_RK4_STATIC_MAX_DOF 524288

/* eg_rk4 without allocation.  No reference counterpart: the reference's rk4
   allocates its stage vectors in Julia; this entry point exists for callers
   whose device memory is reserved up front (a process whose caching allocator
   holds most of the HBM cannot count on a mid-run cudaMalloc, and cudaFree
   synchronises the whole device).  Same arguments, kernels and results as
   eg_rk4, for meshes of at most EG_RK4_STATIC_MAX_DOF unknowns (larger ones:
   EG_ERR_INVALID); the work vectors live in one static 24 MiB device array
   per device.  The first call on a device resolves that array's address with
   the device current and should come before any stream capture (the address
   is resolved again if the device's context has changed, e.g. after
   cudaDeviceReset).  The mesh must belong to the current device, and its
   stream to that device (EG_ERR_INVALID otherwise, before any device work).
   Phase timers must be off (EG_ERR_INVALID otherwise).  Kernels launch one by
   one (no graphs).  Calls that overlap in time on one device race on the
   shared array. */
int eg_rk4_static(eg_mesh* mesh, double* q, double h, double t_max, int32_t itermax,
                  double res_tol, int32_t mem, eg_rk4_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* EULERGPU_H */
