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

/* boundary condition functors (reference BCDict, src/solver/euler/bc.jl) */
typedef enum { EG_BC_VORTEX = 0, EG_BC_FREESTREAM = 1 } eg_bc;

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

/* ---- streams, asynchronous launch and phase timers ---------------------- */

/* Run this mesh's work on `stream` (a cudaStream_t; NULL is CUDA's default
   stream), or on the library's own stream when use_own != 0.  Lets a caller
   order library work with its own kernels and CUDA events. */
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

#ifdef __cplusplus
}
#endif
#endif /* EULERGPU_H */
