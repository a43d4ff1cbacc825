// eg_static.cu -- eg_rk4 with its scratch in a fixed static device array:
// the call itself allocates no device or host memory.
//
// eg_rk4 takes 5 (device state) or 6 (host state) state-sized work vectors
// from cudaMalloc on every call and returns them with cudaFree.  Callers whose
// device memory is reserved up front cannot count on that: a process that
// hands a caching allocator (another framework's pool) most of the HBM can see
// the mid-run cudaMalloc fail, and cudaFree synchronises the whole device,
// stalling what other streams have in flight.  eg_rk4_static runs the same
// kernels in the same order (results are bit-identical to eg_rk4) with the
// work vectors carved from g_rk4_scratch, a file-scope device array of
// 6 * EG_RK4_STATIC_MAX_DOF doubles (24 MiB) that exists once per device.
//
// Setup: the first call on a device (with that device current) resolves the
// array's address with cudaGetSymbolAddress, which may load this module;
// make that first call before any stream capture.  Later calls reuse the
// cached address.  Nothing in the scratch has to start at zero: every work
// vector is written before it is read, and the mesh's status word is cleared
// on the stream at the start of each call.  All calls on one device share the
// one array, so calls that overlap in time (other host threads, or other
// streams still running an earlier call) race on it.
#include <mutex>

#include "eg_internal.h"
#include "eg_kernels.cuh"

namespace {

constexpr int kMaxDevices = 64;
constexpr int64_t kScratchDoubles = 6 * (int64_t)EG_RK4_STATIC_MAX_DOF;

static __device__ __align__(256) double g_rk4_scratch[kScratchDoubles];

std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};

// address of this device's scratch array (resolved once per device)
int scratch_of_current_device(double** out) {
  int dev = -1;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return eg_cuda_fail(ce, "eg_rk4_static: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    eg_set_error("eg_rk4_static: device ordinal %d outside 0..%d", dev, kMaxDevices - 1);
    return EG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    ce = cudaGetSymbolAddress(&p, g_rk4_scratch);
    if (ce != cudaSuccess) return eg_cuda_fail(ce, "eg_rk4_static: cudaGetSymbolAddress");
    g_scratch[dev] = static_cast<double*>(p);
  }
  *out = g_scratch[dev];
  return EG_OK;
}

}  // namespace

extern "C" int eg_rk4_static(eg_mesh* m, double* q, double h, double t_max, int32_t itermax,
                             double res_tol, int32_t mem, eg_rk4_stats* stats) {
  if (!m || !q || !(h > 0) || (mem != EG_MEM_HOST && mem != EG_MEM_DEVICE)) {
    eg_set_error("eg_rk4_static: invalid argument");
    return EG_ERR_INVALID;
  }
  const int64_t N = m->ndof;
  if (N > EG_RK4_STATIC_MAX_DOF) {
    eg_set_error("eg_rk4_static: %lld unknowns exceed the static scratch limit of %d "
                 "(EG_RK4_STATIC_MAX_DOF); use eg_rk4",
                 (long long)N, EG_RK4_STATIC_MAX_DOF);
    return EG_ERR_INVALID;
  }
  if (eg_timing_on(m)) {
    eg_set_error("eg_rk4_static: phase timers are on (they create CUDA events); "
                 "disable them with eg_set_timing(mesh, 0)");
    return EG_ERR_INVALID;
  }
  double* buf = nullptr;
  int rc = scratch_of_current_device(&buf);
  if (rc != EG_OK) return rc;
  double* xold = buf;
  double* k1 = buf + N;
  double* k2 = buf + 2 * N;
  double* k3 = buf + 3 * N;
  double* res = buf + 4 * N;
  double* qd = mem == EG_MEM_HOST ? buf + 5 * N : q;
  if (mem == EG_MEM_HOST) cudaMemcpyAsync(qd, q, 8 * N, cudaMemcpyHostToDevice, m->stream);
  cudaMemcpyAsync(xold, qd, 8 * N, cudaMemcpyDeviceToDevice, m->stream);
  const long t_steps = lround(t_max / h);
  double t = 0.0, last_norm = 0.0;
  int steps = 0, st = EG_OK;
  cudaMemsetAsync(m->status, 0, sizeof(unsigned int), m->stream);
  // the step loop of eg_rk4 (reference rk4.jl:201-330)
  for (long i = 2; i <= t_steps + 1; ++i) {
    t = (i - 2) * h;
    st = eg_launch_residual(m, qd, res);
    if (st != EG_OK) break;
    eg_launch_rk4_stage(m, res, xold, h / 2, k1, qd);
    m->launches += 1;
    if (res_tol > 0) {
      eg_launch_norm(m, k1, 0, m->red + 2048);
      cudaMemcpyAsync(m->h_red, m->red + 2048, sizeof(double), cudaMemcpyDeviceToHost, m->stream);
      cudaStreamSynchronize(m->stream);
      last_norm = m->h_red[0];
      if (last_norm < res_tol) break;
    }
    if (itermax > 0 && i > itermax) break;
    eg_launch_residual(m, qd, res);
    eg_launch_rk4_stage(m, res, xold, h / 2, k2, qd);
    eg_launch_residual(m, qd, res);
    eg_launch_rk4_stage(m, res, xold, h, k3, qd);
    eg_launch_residual(m, qd, res);
    eg_launch_rk4_final(m, k1, k2, k3, res, h, xold, qd);
    m->launches += 3;
    ++steps;
  }
  t += h;
  if (st == EG_OK) {
    cudaMemcpyAsync(m->h_status, m->status, sizeof(unsigned int), cudaMemcpyDeviceToHost, m->stream);
    if (mem == EG_MEM_HOST) cudaMemcpyAsync(q, qd, 8 * N, cudaMemcpyDeviceToHost, m->stream);
    cudaError_t ce = cudaStreamSynchronize(m->stream);
    if (ce != cudaSuccess) st = eg_cuda_fail(ce, "eg_rk4_static");
    else st = eg_check_status(m);
  }
  if (stats) {
    stats->steps = steps;
    stats->t = t;
    stats->res_norm = last_norm;
  }
  return st;
}
