// eg_memory.cu -- device-memory footprint of a mesh and its Newton work
// objects from the mesh counts alone (reference src/estimateMem.jl:1-78,
// which sums the sizes of the mesh and solution arrays from numEl,
// numInterfaces, nodes per element and dofs per node).
//
// The sums below list every device array that eg_mesh_create, eg_lo_create,
// eg_pc_create, eg_ls_create, eg_newton_solve and eg_prolong allocate, with
// the same sizes; each array is rounded up to the allocation granule, so the
// figure bounds what cudaMemGetInfo sees the library take.  A serving loop
// admits a request only if its estimate fits the remaining HBM budget.
#include <algorithm>

#include "eg_internal.h"
#include "eg_linalg.h"

namespace {
constexpr uint64_t kGranule = 512;  // cudaMalloc alignment of every array

struct Sum {
  uint64_t bytes = 0;
  int64_t count = 0;
  void add(uint64_t n) {
    if (!n) return;
    bytes += (n + kGranule - 1) / kGranule * kGranule;
    ++count;
  }
};
}  // namespace

extern "C" int eg_estimate_mem(const eg_mem_query* qy, eg_mem_estimate* out) {
  if (!qy || !out) {
    eg_set_error("eg_estimate_mem: NULL argument");
    return EG_ERR_INVALID;
  }
  const int dim = qy->dim;
  if ((dim != 2 && dim != 3) || qy->num_el <= 0 || qy->nodes_per_el <= 0 ||
      qy->nodes_per_face <= 0 || qy->stencil_size <= 0 || qy->num_interfaces < 0 ||
      qy->num_bndry < 0 || qy->num_orient <= 0 || qy->prolong_from_nodes < 0 ||
      (qy->face_diagonal != 0 && qy->face_diagonal != 1) ||
      (qy->newton_precision != -1 && qy->newton_precision != EG_F64 &&
       qy->newton_precision != EG_F32) ||
      (qy->newton_precision != -1 && (qy->gmres_restart < 1 || qy->gmres_restart > 31))) {
    eg_set_error("eg_estimate_mem: sizes out of range");
    return EG_ERR_INVALID;
  }
  const uint64_t E = qy->num_el, Np = qy->nodes_per_el, Nf = qy->nodes_per_face,
                 S = qy->stencil_size, I = qy->num_interfaces, B = qy->num_bndry,
                 no = qy->num_orient, F = dim + 1, nv = dim + 2, d = dim;
  const uint64_t N = E * Np * nv;
  // mesh and operator (eg_mesh_create)
  Sum mesh;
  mesh.add(8 * d * Np * Np);         // Q
  mesh.add(8 * Np);                  // w
  mesh.add(8 * F * Nf * S);          // interp
  mesh.add(4 * F * S);               // perm
  mesh.add(4 * no * Nf);             // nbrperm
  mesh.add(8 * Nf);                  // wface
  mesh.add(8 * F * Np * Nf);         // lift
  mesh.add(8 * F * Nf * S);          // liftS
  mesh.add(4 * no * Nf);             // nbrinv
  mesh.add(8 * E * Np * d * d);      // dxidx
  mesh.add(8 * E * Np);              // jac
  mesh.add(8 * E * Np);              // Minv
  mesh.add(4 * I * 5);               // interfaces
  mesh.add(8 * I * Nf * d);          // nrm_face
  mesh.add(4 * B * 2);               // bndryfaces
  mesh.add(4 * B);                   // bc of each boundary face
  mesh.add(8 * B * Nf * d);          // coords_bndry
  mesh.add(8 * B * Nf * d);          // nrm_bndry
  mesh.add(8 * B * Nf * nv);         // Dirichlet states
  mesh.add(sizeof(EFace) * E * F);   // element face table
  mesh.add(8 * (I + B) * Nf * nv);   // face fluxes
  mesh.add(8 * N);                   // host-input staging
  mesh.add(8 * N);                   // host-output staging
  mesh.add(4);                       // status word
  mesh.add(8 * 4096);                // reduction scratch
  if (qy->prolong_from_nodes > 0)    // eg_prolong's matrix kept by the fine mesh
    mesh.add(8 * (Np * nv) * ((uint64_t)qy->prolong_from_nodes * nv));
  // the caller's state and residual (EulerData q, res)
  Sum eqn;
  eqn.add(8 * N);
  eqn.add(8 * N);
  Sum jac, pc, kry, newton;
  if (qy->newton_precision != -1) {
    const uint64_t es = qy->newton_precision == EG_F64 ? 8 : 4;
    const uint64_t n = Np * nv, nb = S * nv, m = qy->gmres_restart;
    // explicit Jacobian (eg_lo_create)
    jac.add(es * E * n * n);                    // element blocks
    jac.add(qy->face_diagonal ? es * I * 2 * S * nv * nv   // coupling blocks
                              : es * I * 2 * nb * nb);
    jac.add(es * (I + B) * Nf * 2 * nv * nv);   // point-flux Jacobians
    jac.add(4 * F * Np);                        // stencil positions
    jac.add(es * N);                            // x, y in the operator precision
    jac.add(es * N);
    jac.add(8 * N);                             // x, y in FP64
    jac.add(8 * N);
    jac.add(4 * E * F);                         // face -> coupling block
    // block-Jacobi inverses (eg_pc_create)
    pc.add(es * E * n * n);
    // GMRES(m) (eg_ls_create)
    kry.add(es * (m + 1) * N);                  // Krylov basis
    kry.add(es * N);                            // w
    kry.add(es * N);                            // z
    kry.add(es * I * 2 * nb);                   // pushed coupling products
    kry.add(es * N);                            // x
    kry.add(es * N);                            // b
    kry.add(es * eg_gmres_partials((int)m));     // partial sums
    kry.add(es * 4 * (m + 2));                  // h
    kry.add(es * (m + 1));                      // y
    kry.add(8 * ((m + 1) * m + 4 * (m + 1)));   // Hessenberg, Givens, least squares
    kry.add(4 * 16);                            // flags
    kry.add(8 * 8);                             // scalars
    kry.add(8 * N);                             // x, b in FP64
    kry.add(8 * N);
    // Newton vectors (eg_newton_solve): residual, step, saved state, the
    // state the iteration graphs update
    newton.add(8 * N);
    newton.add(8 * N);
    newton.add(8 * N);
    newton.add(8 * N);
  }
  out->mesh = mesh.bytes;
  out->eqn = eqn.bytes;
  out->jacobian = jac.bytes;
  out->pc = pc.bytes;
  out->krylov = kry.bytes;
  out->newton = newton.bytes;
  out->total = mesh.bytes + eqn.bytes + jac.bytes + pc.bytes + kry.bytes + newton.bytes;
  out->allocations = mesh.count + eqn.count + jac.count + pc.count + kry.count + newton.count;
  return EG_OK;
}
