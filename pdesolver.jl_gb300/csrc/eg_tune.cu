// eg_tune.cu -- launch configuration of the element kernels and the
// autotuner that picks it.
//
// The element kernel (weak form k_element, split form k_split_element) has
// two free choices per operator: the elements a CTA owns (shared-memory
// staging of Q and the face-lift table is paid once per CTA; more elements
// amortise it but lower the number of resident CTAs), and, for the weak form,
// whether the volume contraction Q^T F runs on CUDA cores or on the FP64
// tensor cores (mma.sync m8n8k4).  eg_autotune times every admissible
// candidate on the caller's state with CUDA events on the mesh stream and
// keeps the fastest.  The reference has no counterpart (its loops are plain
// Julia); the result changes only the launch shape and, for the tensor-core
// contraction, the order of the FP64 sums (results agree with the CUDA-core
// path to round-off).
#include <cstring>
#include <vector>

#include "eg_internal.h"
#include "eg_kernels.cuh"

extern "C" int eg_set_launch_config(eg_mesh* m, const eg_launch_config* c) {
  if (!m || !c) {
    eg_set_error("eg_set_launch_config: NULL argument");
    return EG_ERR_INVALID;
  }
  if (c->elements_per_cta < 0 || (c->volume_mma != 0 && c->volume_mma != 1)) {
    eg_set_error("eg_set_launch_config: elements_per_cta >= 0 and volume_mma in {0, 1}");
    return EG_ERR_INVALID;
  }
  int threads;
  size_t smem;
  eg_mesh probe = *m;  // validate against the mesh's sizes before changing it
  probe.elem_epb = c->elements_per_cta;
  probe.vol_mma = c->volume_mma;
  int epb = c->elements_per_cta;
  if (epb > 0) {
    const int st = eg_element_shape(&probe, epb, c->volume_mma, &threads, &smem);
    if (st != EG_OK) return st;
  } else if (c->volume_mma && m->params.volume_integral_type == 2) {
    eg_set_error("eg_set_launch_config: the split form has no tensor-core contraction");
    return EG_ERR_INVALID;
  }
  m->elem_epb = c->elements_per_cta;
  m->vol_mma = c->volume_mma;
  return EG_OK;
}

extern "C" int eg_get_launch_config(eg_mesh* m, eg_launch_config* c) {
  if (!m || !c) {
    eg_set_error("eg_get_launch_config: NULL argument");
    return EG_ERR_INVALID;
  }
  std::memset(c, 0, sizeof(*c));
  c->elements_per_cta = m->elem_epb;
  c->volume_mma = m->vol_mma;
  return EG_OK;
}

extern "C" int eg_autotune(eg_mesh* m, const double* q_dev, int32_t reps, eg_tune_entry* table,
                           int32_t max_entries, int32_t* n_entries) {
  if (!m || !q_dev || reps < 1 || (max_entries > 0 && !table)) {
    eg_set_error("eg_autotune: invalid argument");
    return EG_ERR_INVALID;
  }
  if (m->capturing) {
    eg_set_error("eg_autotune: the mesh stream is being captured");
    return EG_ERR_INVALID;
  }
  // candidates: elements per CTA in powers of two and the built-in choice
  // 256 / Np, times the contraction kind for the weak form
  std::vector<eg_launch_config> cand;
  const bool weak = m->params.volume_integral_type == 1;
  int builtin = 256 / m->Np;
  if (builtin < 1) builtin = 1;
  std::vector<int> sizes;
  for (int epb = 1; epb <= 128; epb *= 2) {
    if (builtin > epb / 2 && builtin < epb) sizes.push_back(builtin);
    sizes.push_back(epb);
  }
  for (int mma = 0; mma <= (weak ? 1 : 0); ++mma)
    for (int epb : sizes) {
      if ((epb - 1) * m->Np >= 1024) break;
      int threads;
      size_t smem;
      eg_mesh probe = *m;
      if (eg_element_shape(&probe, epb, mma, &threads, &smem) != EG_OK) continue;
      eg_launch_config c;
      std::memset(&c, 0, sizeof(c));
      c.elements_per_cta = epb;
      c.volume_mma = mma;
      cand.push_back(c);
    }
  if (cand.empty()) {
    eg_set_error("eg_autotune: no launch configuration fits");
    return EG_ERR_UNSUPPORTED;
  }
  const int save_epb = m->elem_epb, save_mma = m->vol_mma;
  const bool timers = eg_timing_on(m);
  if (timers) eg_set_timing(m, 0);
  double* res = m->res_dev;
  // face fluxes of q once; every candidate then reads the same m->fflux
  m->elem_epb = 0;
  m->vol_mma = 0;
  int st = eg_launch_residual(m, q_dev, res);
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (st == EG_OK) {
    cudaError_t e = cudaEventCreate(&ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ev1);
    if (e != cudaSuccess) st = eg_cuda_fail(e, "eg_autotune: cudaEventCreate");
  }
  int best = -1;
  float best_ms = 0.0f;
  int n_out = 0;
  for (size_t k = 0; k < cand.size() && st == EG_OK; ++k) {
    m->elem_epb = cand[k].elements_per_cta;
    m->vol_mma = cand[k].volume_mma;
    st = eg_launch_element(m, q_dev, res);  // warm-up (instruction cache, attributes)
    if (st != EG_OK) break;
    cudaEventRecord(ev0, m->stream);
    for (int r = 0; r < reps && st == EG_OK; ++r) st = eg_launch_element(m, q_dev, res);
    cudaEventRecord(ev1, m->stream);
    cudaError_t e = cudaEventSynchronize(ev1);
    if (e != cudaSuccess) {
      st = eg_cuda_fail(e, "eg_autotune");
      break;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    ms /= reps;
    if (n_out < max_entries) {
      table[n_out].config = cand[k];
      table[n_out].ms = ms;
      ++n_out;
    }
    if (best < 0 || ms < best_ms) {
      best = (int)k;
      best_ms = ms;
    }
  }
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (timers) eg_set_timing(m, 1);
  if (n_entries) *n_entries = n_out;
  if (st != EG_OK || best < 0) {
    m->elem_epb = save_epb;
    m->vol_mma = save_mma;
    return st != EG_OK ? st : EG_ERR_UNSUPPORTED;
  }
  m->elem_epb = cand[best].elements_per_cta;
  m->vol_mma = cand[best].volume_mma;
  // report (and clear) density/pressure flags of the caller's state
  return eg_sync(m);
}
