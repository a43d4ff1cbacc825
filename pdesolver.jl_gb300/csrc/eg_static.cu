// eg_static.cu -- eg_rk4 with its scratch in a fixed static device array:
// the call itself allocates no device or host memory.
//
// eg_rk4 takes its six state-sized work vectors from cudaMalloc on its first
// call on a mesh and keeps them, with the CUDA graphs of its step (whose
// instantiation may allocate), until the mesh is destroyed or
// eg_newton_release frees them with cudaFree.  Callers whose device memory is
// reserved up front cannot count on that: a process that hands a caching
// allocator (another framework's pool) most of the HBM can see the mid-run
// cudaMalloc fail, and cudaFree synchronises the whole device, stalling what
// other streams have in flight.  eg_rk4_static runs the same kernels in the
// same order (results are bit-identical to eg_rk4), launched one by one, with
// the work vectors carved from g_rk4_scratch, a file-scope device array of
// 6 * EG_RK4_STATIC_MAX_DOF doubles (24 MiB) that exists once per device.
//
// Setup: the first call on a device (with that device current) resolves the
// array's address with cudaGetSymbolAddress, which may load this module;
// make that first call before any stream capture.  The address is cached per
// device together with the identity of the CUDA context it was resolved in,
// and resolved again when that context has changed (after cudaDeviceReset a
// new primary context loads the module at a new address).  The mesh must
// belong to the current device (and its stream to the same device); otherwise
// the call returns EG_ERR_INVALID before any device work.  Nothing in the
// scratch has to start at zero: every work vector is written before it is
// read, and the mesh's status word is cleared on the stream at the start of
// each call.  All calls on one device share the one array, so calls that
// overlap in time (other host threads, or other streams still running an
// earlier call) race on it.
#include <mutex>

#include "eg_internal.h"
#include "eg_kernels.cuh"

namespace {

constexpr int kMaxDevices = 64;
constexpr int64_t kScratchDoubles = 6 * (int64_t)EG_RK4_STATIC_MAX_DOF;

static __device__ __align__(256) double g_rk4_scratch[kScratchDoubles];

std::mutex g_mu;
struct ScratchSlot {
  double* ptr = nullptr;
  unsigned long long ctx = 0;  // context the address was resolved in (0: unknown)
};
ScratchSlot g_scratch[kMaxDevices];

// identity of the calling thread's current CUDA context (driver entry points
// cuCtxGetCurrent / cuCtxGetId through the runtime, no link to libcuda);
// 0 when the driver does not provide them
unsigned long long current_context_id() {
  typedef int (*GetCurrentFn)(void**);
  typedef int (*GetIdFn)(void*, unsigned long long*);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetIdFn>(f);
    cudaGetLastError();
  });
  if (!get_current || !get_id) return 0;
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != 0 || !ctx) return 0;
  if (get_id(ctx, &id) != 0) return 0;
  return id;
}

// address of the mesh device's scratch array (the mesh's device is current)
int scratch_of_current_device(const eg_mesh* m, double** out) {
  const int dev = m->device;
  if (dev < 0 || dev >= kMaxDevices) {
    eg_set_error("eg_rk4_static: device ordinal %d outside 0..%d", dev, kMaxDevices - 1);
    return EG_ERR_INVALID;
  }
  // a runtime call on the mesh stream binds the device's context to this
  // thread before its identity is read
  cudaError_t ce = cudaStreamQuery(m->stream);
  if (ce != cudaSuccess && ce != cudaErrorNotReady) return eg_cuda_fail(ce, "eg_rk4_static");
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_mu);
  ScratchSlot& slot = g_scratch[dev];
  if (!slot.ptr || slot.ctx != ctx) {
    void* p = nullptr;
    ce = cudaGetSymbolAddress(&p, g_rk4_scratch);
    if (ce != cudaSuccess) return eg_cuda_fail(ce, "eg_rk4_static: cudaGetSymbolAddress");
    slot.ptr = static_cast<double*>(p);
    slot.ctx = ctx;
  }
  *out = slot.ptr;
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
  int rc = eg_check_device(m, "eg_rk4_static");
  if (rc != EG_OK) return rc;
  double* buf = nullptr;
  rc = scratch_of_current_device(m, &buf);
  if (rc != EG_OK) return rc;
  // buf[6][N] = x_old, k1, k2, k3, res, q: the loop iterates in the scratch
  // copy of the state and writes it back at the end
  double* qd = buf + 5 * N;
  EG_CUDA(cudaMemcpyAsync(qd, q, 8 * N, mem == EG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                          m->stream));
  EG_CUDA(cudaMemcpyAsync(buf, qd, 8 * N, cudaMemcpyDeviceToDevice, m->stream));
  EG_CUDA(cudaMemsetAsync(m->status, 0, sizeof(unsigned int), m->stream));
  // the kernels and order of eg_rk4, launched one by one (no graphs)
  eg_rk4_stats s;
  int st = eg_rk4_loop(m, buf, h, t_max, itermax, res_tol, false, &s);
  if (st == EG_OK) {
    cudaError_t ce = cudaMemcpyAsync(m->h_status, m->status, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                     m->stream);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(q, qd, 8 * N, mem == EG_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                           m->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(m->stream);
    if (ce != cudaSuccess) {
      cudaStreamSynchronize(m->stream);
      st = eg_cuda_fail(ce, "eg_rk4_static");
    } else {
      st = eg_check_status(m);
    }
  }
  if (stats) *stats = s;
  return st;
}
