// eg_timing.cu -- streams, asynchronous launch and per-phase device timers
// (the CUDA-event counterpart of the reference's Timings buckets,
// src/Utils/Utils.jl:567-626).
#include <vector>

#include "eg_internal.h"
#include "eg_kernels.cuh"

struct TimerState {
  bool enabled = false;
  std::vector<cudaEvent_t> pool;     // free events
  struct Pending { cudaEvent_t a, b; int phase; int n; };
  std::vector<Pending> pending;
  cudaEvent_t open_ev = nullptr;
  double sums[EG_NPHASE] = {0, 0, 0, 0};
  int64_t timed = 0;
};

static cudaEvent_t take_event(TimerState* t) {
  if (!t->pool.empty()) {
    cudaEvent_t e = t->pool.back();
    t->pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

void eg_phase_begin(eg_mesh* m, int phase) {
  (void)phase;
  TimerState* t = m->timer;
  if (!t || !t->enabled || m->capturing) return;
  t->open_ev = take_event(t);
  cudaEventRecord(t->open_ev, m->stream);
}

void eg_phase_end(eg_mesh* m, int phase, int nlaunch) {
  if (m->capturing) return;  // graph nodes are counted per replay
  m->launches += nlaunch;
  TimerState* t = m->timer;
  if (!t || !t->enabled || !t->open_ev) return;
  cudaEvent_t b = take_event(t);
  cudaEventRecord(b, m->stream);
  t->pending.push_back({t->open_ev, b, phase, nlaunch});
  t->open_ev = nullptr;
}

static void collect(eg_mesh* m) {
  TimerState* t = m->timer;
  if (!t) return;
  for (auto& p : t->pending) {
    cudaEventSynchronize(p.b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    t->sums[p.phase] += ms;
    t->timed += p.n;
    t->pool.push_back(p.a);
    t->pool.push_back(p.b);
  }
  t->pending.clear();
}

void eg_timer_free(eg_mesh* m) {
  TimerState* t = m->timer;
  if (!t) return;
  collect(m);
  for (auto e : t->pool) cudaEventDestroy(e);
  delete t;
  m->timer = nullptr;
}

extern "C" int eg_set_timing(eg_mesh* m, int32_t enable) {
  if (!m) return EG_ERR_INVALID;
  if (!m->timer) m->timer = new TimerState();
  m->timer->enabled = enable != 0;
  return EG_OK;
}

extern "C" int eg_get_timings(eg_mesh* m, eg_timings* out) {
  if (!m || !out) return EG_ERR_INVALID;
  EG_CUDA(cudaStreamSynchronize(m->stream));
  collect(m);
  out->launches = m->launches;
  if (m->timer) {
    out->t_face_flux = m->timer->sums[EG_PHASE_FACE];
    out->t_element = m->timer->sums[EG_PHASE_ELEMENT];
    out->t_norm = m->timer->sums[EG_PHASE_NORM];
    out->t_other = m->timer->sums[EG_PHASE_OTHER];
    out->timed = m->timer->timed;
  } else {
    out->t_face_flux = out->t_element = out->t_norm = out->t_other = 0.0;
    out->timed = 0;
  }
  return EG_OK;
}

extern "C" int eg_reset_timings(eg_mesh* m) {
  if (!m) return EG_ERR_INVALID;
  EG_CUDA(cudaStreamSynchronize(m->stream));
  collect(m);
  if (m->timer) {
    for (double& s : m->timer->sums) s = 0.0;
    m->timer->timed = 0;
  }
  return EG_OK;
}

extern "C" int eg_mesh_set_stream(eg_mesh* m, void* stream, int32_t use_own) {
  if (!m) return EG_ERR_INVALID;
  cudaStream_t s = use_own ? m->own_stream : (cudaStream_t)stream;
  if (s != 0 && s != cudaStreamLegacy && s != cudaStreamPerThread) {
    // a stream of another device would run the mesh's kernels there
    int sdev = -1;
    EG_CUDA(cudaStreamGetDevice(s, &sdev));
    if (sdev != m->device) {
      eg_set_error("eg_mesh_set_stream: the stream belongs to device %d, the mesh to device %d",
                   sdev, m->device);
      return EG_ERR_INVALID;
    }
  }
  EG_CUDA(cudaStreamSynchronize(m->stream));
  m->stream = s;
  return EG_OK;
}

int eg_check_device(const eg_mesh* m, const char* who) {
  int dev = -1;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return eg_cuda_fail(ce, who);
  if (dev != m->device) {
    eg_set_error("%s: the current device is %d, the mesh was created on device %d", who, dev,
                 m->device);
    return EG_ERR_INVALID;
  }
  cudaStream_t s = m->stream;
  if (s != 0 && s != cudaStreamLegacy && s != cudaStreamPerThread) {
    int sdev = -1;
    ce = cudaStreamGetDevice(s, &sdev);
    if (ce != cudaSuccess) return eg_cuda_fail(ce, who);
    if (sdev != m->device) {
      eg_set_error("%s: the mesh stream belongs to device %d, the mesh to device %d", who, sdev,
                   m->device);
      return EG_ERR_INVALID;
    }
  }
  return EG_OK;
}

extern "C" int eg_eval_residual_async(eg_mesh* m, const double* q, double* res) {
  if (!m || !q || !res) {
    eg_set_error("eg_eval_residual_async: NULL argument");
    return EG_ERR_INVALID;
  }
  int st = eg_launch_residual(m, q, res);
  if (st != EG_OK) return st;
  EG_CUDA(cudaGetLastError());
  return EG_OK;
}

extern "C" int eg_sync(eg_mesh* m) {
  if (!m) return EG_ERR_INVALID;
  EG_CUDA(cudaMemcpyAsync(m->h_status, m->status, sizeof(unsigned int), cudaMemcpyDeviceToHost, m->stream));
  EG_CUDA(cudaMemsetAsync(m->status, 0, sizeof(unsigned int), m->stream));
  EG_CUDA(cudaStreamSynchronize(m->stream));
  return eg_check_status(m);
}

bool eg_timing_on(const eg_mesh* m) { return m->timer && m->timer->enabled; }
