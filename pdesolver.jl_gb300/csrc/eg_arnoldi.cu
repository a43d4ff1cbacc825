// eg_arnoldi.cu -- the restarted GMRES solve of a Newton system as one
// persistent cooperative kernel (all restart cycles, one launch).
//
// The Krylov vectors of the Newton systems are small (1.5 MB in FP32 for the
// 8192-triangle p=3 problem), so an Arnoldi step is bound by synchronisation
// and by streaming the operator (D^-1 and the coupling blocks), not by the
// vector work.  One launch per solve replaces ~13 launches per iteration and
// a host round trip per restart:
//   * block b owns a contiguous range of elements (and their rows) for the
//     whole solve, so the block-Jacobi apply, the Gram-Schmidt updates, the
//     scaling of the new basis vector and the solution update touch only its
//     own rows;
//   * the face coupling is pushed: the owner of element e computes, for each
//     interface face, the neighbour's coupling block times e's values (held
//     in shared memory) into a face-side buffer, read after one grid barrier
//     by the neighbour's owner; a grid barrier is otherwise needed only for
//     the dot-product partials;
//   * every block reduces the dot-product partials in the same order, so the
//     Hessenberg column, the re-orthogonalisation test (DGKS), the Givens
//     rotation and the convergence decision are bit-identical in every block:
//     no broadcast is needed and all blocks take the same branches (no
//     barrier can be missed).
// Per Arnoldi iteration: 2 grid barriers (3 with the second Gram-Schmidt
// pass); per restart: 2 more (residual push, residual norm).  A system whose
// element blocks take at most 2 MB, or whose grid would have at most 16
// blocks, runs on one thread-block cluster instead (eg_arnoldi_cluster.cu).
// The operator is the right-preconditioned J M^-1 = I + C D^-1 (element blocks
// cancel with their inverses); the Arnoldi vectors are built from K = C D^-1
// and the identity is added to the Hessenberg diagonal.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "eg_arnoldi_body.cuh"

// one multi-block persistent solve in flight per device: two grids that each
// wait in grid barriers must never hold parts of the GPU at the same time
std::mutex& eg_coop_mutex(int dev) {
  static std::mutex mu[64];
  return mu[dev & 63];
}

namespace {

template <typename T>
int launch_T(eg_ls* ls) {
  eg_mesh* m = ls->lo->mesh;
  CoopArgs<T> a;
  coop_args<T>(ls, &a);
  void* fn = nullptr;
  switch (a.n) {
#define EG_CASE(NBV) \
  case NBV: fn = m->dim == 2 ? (void*)k_gmres_coop<2, NBV, T> : (void*)k_gmres_coop<3, NBV, T>; break;
    EG_CASE(12) EG_CASE(24) EG_CASE(28) EG_CASE(40) EG_CASE(48) EG_CASE(60) EG_CASE(72) EG_CASE(30)
    EG_CASE(115)
#undef EG_CASE
    default: fn = m->dim == 2 ? (void*)k_gmres_coop<2, 0, T> : (void*)k_gmres_coop<3, 0, T>;
  }
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // grid: one cluster for a small system (its blocks are co-scheduled, so
  // several run side by side on other streams; one block when no cluster can
  // be placed); otherwise one block per SM (at most one per element), one
  // such grid at a time
  const size_t elem_bytes = (size_t)a.n * sizeof(T);
  const size_t op_bytes = (size_t)m->E * a.n * a.n * sizeof(T);
  if (ls->coop_grid <= 0) {
    // a cluster for a small system, and for one with at most 32 elements
    // per block of a cluster (no device-wide lock needed)
    const int chunks = (m->E + 31) / 32;
    int C = 0;
    if (op_bytes <= kSmallOperatorBytes)
      C = EG_GMRES_CLUSTER_BLOCKS;
    else if (chunks <= EG_GMRES_CLUSTER_BLOCKS)
      C = std::max(2, chunks);
    while (C > 1 && C > m->E) C >>= 1;
    if (C > 1) {
      int rc = eg_gmres_cluster(ls, C);
      if (rc == EG_ERR_UNSUPPORTED && C > 8) rc = eg_gmres_cluster(ls, 8);
      if (rc != EG_ERR_UNSUPPORTED) return rc;
    }
  }
  // a lone multi-block grid (they run one at a time) takes every SM: the
  // full grid was the fastest for every system above the cluster sizes
  int nblk = op_bytes <= kSmallOperatorBytes ? 1 : std::max(2, std::min(sms, m->E));
  if (ls->coop_grid > 0) nblk = std::min(ls->coop_grid, sms);
  if (nblk > m->E) nblk = m->E;
  if (nblk > EG_COOP_MAX_BLOCKS) nblk = EG_COOP_MAX_BLOCKS;
  const int epb = (m->E + nblk - 1) / nblk;
  int ec = (int)((40 * 1024) / elem_bytes);
  if (ec < 1) ec = 1;
  if (ec > epb) ec = epb;
  a.ec = ec;
  const size_t smem = (size_t)ec * elem_bytes;
  // the default dynamic limit is 48 KB minus the kernel's static shared
  // memory (11.6 KB in FP64), below the chunk size above
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, NT, smem);
  if (per_sm < 1 || nblk <= 0) {
    eg_set_error("persistent GMRES kernel cannot be resident");
    return EG_ERR_UNSUPPORTED;
  }
  void* args[] = {&a};
  if (nblk == 1) {
    EG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(1), dim3(NT), args, smem, m->stream));
    m->launches += 1;
    return EG_OK;
  }
  std::lock_guard<std::mutex> lock(eg_coop_mutex(dev));
  EG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(nblk), dim3(NT), args, smem, m->stream));
  m->launches += 1;
  EG_CUDA(cudaStreamSynchronize(m->stream));  // the grid has finished before the next one starts
  return EG_OK;
}

}  // namespace

// the whole GMRES solve (all restart cycles) as one cooperative launch;
// partial sums need 4 * grid * 33 values of ls->part (eg_ls_create sizes
// them for EG_COOP_MAX_BLOCKS blocks)
int eg_gmres_coop(eg_ls* ls) {
  if (eg_gmres_batching() && eg_gmres_wanted_blocks(ls) > 1) return eg_gmres_coop_batched(ls);
  return ls->lo->prec == EG_F64 ? launch_T<double>(ls) : launch_T<float>(ls);
}

bool eg_coop_usable(const eg_ls* ls) {
  const eg_mesh* m = ls->lo->mesh;
  return ls->lo->nb <= NB_MAX && m->F == m->dim + 1 && m->F * m->S <= 64 && m->F * m->Np <= 128 && m->I > 0 &&
         eg_coop_supported();
}

bool eg_coop_supported() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess) return false;
  return v != 0;
}
