// eg_arnoldi_cluster.cu -- the persistent GMRES solve of a small system by
// one thread-block cluster (k_gmres_cluster: the solve body of
// eg_arnoldi_body.cuh with the hardware cluster barrier in place of the grid
// barrier).  A system whose element blocks take at most 2 MB would be
// latency-bound on one SM; C blocks on C SMs of one GPC share the rows, the
// pushes and the reductions, and the cluster needs neither a cooperative
// launch nor the one-grid-at-a-time rule of the multi-block solve, so the
// small solves of concurrent host threads run side by side.
#include "eg_arnoldi_body.cuh"

namespace {

// the solve of a small system by one thread-block cluster of C blocks;
// EG_ERR_UNSUPPORTED when such a cluster cannot be placed on this device
template <typename T>
int launch_cluster(eg_ls* ls, int C) {
  eg_mesh* m = ls->lo->mesh;
  CoopArgs<T> a;
  coop_args<T>(ls, &a);
  void* fn = nullptr;
  switch (a.n) {
#define EG_CASE(NBV) \
  case NBV: fn = m->dim == 2 ? (void*)k_gmres_cluster<2, NBV, T> : (void*)k_gmres_cluster<3, NBV, T>; break;
    EG_CASE(12) EG_CASE(24) EG_CASE(28) EG_CASE(40) EG_CASE(48) EG_CASE(60) EG_CASE(72) EG_CASE(30)
    EG_CASE(115)
#undef EG_CASE
    default: fn = m->dim == 2 ? (void*)k_gmres_cluster<2, 0, T> : (void*)k_gmres_cluster<3, 0, T>;
  }
  const size_t elem_bytes = (size_t)a.n * sizeof(T);
  const int epb = (m->E + C - 1) / C;
  int ec = (int)((40 * 1024) / elem_bytes);
  if (ec < 1) ec = 1;
  if (ec > epb) ec = epb;
  a.ec = ec;
  const size_t smem = (size_t)ec * elem_bytes;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
  if (C > 8) cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)C);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = m->stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) != cudaSuccess || clusters < 1) {
    cudaGetLastError();
    return EG_ERR_UNSUPPORTED;
  }
  void* args[] = {&a};
  EG_CUDA(cudaLaunchKernelExC(&cfg, fn, args));
  m->launches += 1;
  return EG_OK;
}

}  // namespace

int eg_gmres_cluster(eg_ls* ls, int C) {
  return ls->lo->prec == EG_F64 ? launch_cluster<double>(ls, C) : launch_cluster<float>(ls, C);
}
