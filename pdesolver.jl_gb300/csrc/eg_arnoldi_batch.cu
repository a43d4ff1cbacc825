// eg_arnoldi_batch.cu -- several problems' persistent GMRES solves in one
// cooperative launch (the batched counterpart of eg_arnoldi.cu).
//
// When batching is on (eg_set_gmres_batching), a thread that reaches the
// Krylov solve of its Newton iteration hands the solve to a per-device
// batcher instead of launching it, if the solve runs on several blocks (a
// one-block solve is launched at once: one-block grids of several threads
// already share the GPU without waiting for each other).  The solves handed in within a short
// window (or as soon as every thread inside eg_newton_solve has handed one in)
// go out as one cooperative grid walking a work list: each problem gets a
// contiguous range of blocks (at most one block per SM in total, more blocks
// for larger operators) and runs the same device function as the
// single-problem kernel, with grid barriers replaced by barriers over its own
// blocks.  Several problems then share the GPU inside one launch instead of
// queueing for it one multi-block grid at a time.
//
// Every block of a cooperative launch is resident, so a barrier over some of
// its blocks always completes; each wait is still bounded (kSpinLimit polls),
// after which the block raises the launch's error flag, every block of the
// launch leaves at its next barrier, and the host reports EG_ERR_TIMEOUT.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <mutex>
#include <vector>

#include "eg_arnoldi_body.cuh"

namespace {

constexpr int kMaxBatch = 128;               // problems per launch
constexpr long long kSpinLimit = 1LL << 24;  // polls of one barrier wait

// barrier over the nblk blocks of one problem of a batched launch; returns
// false (in every thread of the block) once the launch's error flag is set
struct SubBarrier {
  unsigned int* count;  // arrivals at the current barrier
  unsigned int* gen;    // generation, bumped by the last arrival
  int* err;             // launch-wide flag: a wait gave up
  int nblk;
  int* s_ok;            // shared-memory broadcast slot
  __device__ bool sync() {
    __syncthreads();
    if (threadIdx.x == 0) {
      int ok = 1;
      if (nblk > 1) {
        const unsigned int g = *(volatile unsigned int*)gen;
        __threadfence();  // the block's writes before its arrival
        if (atomicAdd(count, 1u) == (unsigned int)(nblk - 1)) {
          *(volatile unsigned int*)count = 0u;
          __threadfence();
          atomicAdd(gen, 1u);
        } else {
          long long polls = 0;
          while (*(volatile unsigned int*)gen == g) {
            if (*(volatile int*)err) {
              ok = 0;
              break;
            }
            if (++polls > kSpinLimit) {
              atomicExch(err, 1);
              ok = 0;
              break;
            }
            __nanosleep(64);
          }
        }
        __threadfence();  // the other blocks' writes after the barrier
      }
      if (*(volatile int*)err) ok = 0;
      *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
  }
};

// one work-list entry: the problem's kernel arguments (device copy), its
// block range, its (dimension, block size) case and its chunk size
struct BatchEntry {
  const void* args;
  int b0, nblk, kind, ec;
};
struct BatchList {
  int n;
  BatchEntry e[kMaxBatch];
};

// (dimension, element-block size) cases with a compiled body, the same set
// as the single-problem launcher compiles for these dimensions (the block
// size changes the order of the block-row sums); others run the generic body
int kind_of(int dim, int n) {
  if (dim == 2) {
    switch (n) {
      case 12: return 0;
      case 24: return 1;
      case 28: return 2;
      case 40: return 3;
      case 48: return 4;
      case 60: return 5;
      case 72: return 6;
      default: return 7;
    }
  }
  switch (n) {
    case 30: return 8;
    case 115: return 9;
    default: return 10;
  }
}

template <typename T>
__global__ void __launch_bounds__(NT, 1) k_gmres_batch(BatchList list, unsigned int* bars, int* err) {
  __shared__ GmresShared<T> sm;
  __shared__ CoopArgs<T> sa;
  __shared__ int s_k, s_nblk, s_b0, s_kind, s_ok;
  if (threadIdx.x == 0) {
    int k = 0;
    while (k + 1 < list.n && (int)blockIdx.x >= list.e[k + 1].b0) ++k;
    const BatchEntry en = list.e[k];
    s_k = k;
    s_nblk = en.nblk;
    s_b0 = en.b0;
    s_kind = en.kind;
    sa = *reinterpret_cast<const CoopArgs<T>*>(en.args);
    sa.ec = en.ec;
  }
  __syncthreads();
  const int k = s_k, nblk = s_nblk, b = (int)blockIdx.x - s_b0;
  SubBarrier bar{bars + 2 * k, bars + 2 * k + 1, err, nblk, &s_ok};
  switch (s_kind) {
    case 0: gmres_body<2, 12, T>(sa, b, nblk, bar, sm); break;
    case 1: gmres_body<2, 24, T>(sa, b, nblk, bar, sm); break;
    case 2: gmres_body<2, 28, T>(sa, b, nblk, bar, sm); break;
    case 3: gmres_body<2, 40, T>(sa, b, nblk, bar, sm); break;
    case 4: gmres_body<2, 48, T>(sa, b, nblk, bar, sm); break;
    case 5: gmres_body<2, 60, T>(sa, b, nblk, bar, sm); break;
    case 6: gmres_body<2, 72, T>(sa, b, nblk, bar, sm); break;
    case 7: gmres_body<2, 0, T>(sa, b, nblk, bar, sm); break;
    case 8: gmres_body<3, 30, T>(sa, b, nblk, bar, sm); break;
    case 9: gmres_body<3, 115, T>(sa, b, nblk, bar, sm); break;
    default: gmres_body<3, 0, T>(sa, b, nblk, bar, sm); break;
  }
}

// ------------------------------------------------------------------ batcher
struct Submission {
  eg_ls* ls;
  int rc = EG_OK;
  bool done = false;
};

struct Batcher {
  std::mutex mu;
  std::condition_variable cv;
  std::vector<Submission*> pending;
  std::chrono::steady_clock::time_point first;  // oldest pending hand-in
  bool launching = false;
  cudaStream_t stream = nullptr;  // the batched grids' stream
  unsigned int* bars = nullptr;   // [kMaxBatch][2] barrier counters (device)
  int* err = nullptr;             // device error flag
  int* h_err = nullptr;           // pinned copy
  std::atomic<int> active{0};     // threads inside eg_newton_solve with a
                                  // multi-block Krylov solve
};

Batcher& batcher(int dev) {
  static Batcher b[64];
  return b[dev & 63];
}

std::atomic<int> g_batching{0};
std::atomic<long long> g_window_ns{50000};

int ensure_batcher(Batcher& B) {
  if (B.stream) return EG_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void**)&B.bars, sizeof(unsigned int) * 2 * kMaxBatch);
  if (e == cudaSuccess) e = cudaMalloc((void**)&B.err, sizeof(int));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&B.h_err, sizeof(int));
  if (e != cudaSuccess) return eg_cuda_fail(e, "GMRES batcher");
  return EG_OK;
}

// blocks of one problem: what the single-problem launcher gives it (one block
// for operators of at most 2 MB, else up to one block per SM with at least 32
// elements each).  A batch never shrinks a problem's share: the block
// partition fixes the order of the dot-product reductions, so a solve gives
// the same bits in any batch and alone.
int wanted_blocks_sms(const eg_ls* ls, int sms) {
  const eg_mesh* m = ls->lo->mesh;
  const size_t es = ls->lo->prec == EG_F64 ? 8 : 4;
  const size_t op = (size_t)m->E * ls->lo->n * ls->lo->n * es;
  // the block count of the same solve alone (eg_arnoldi.cu), so a batched
  // solve keeps its partition and gives the same bits: one (a small system,
  // solved by a cluster and never batched), the cluster's blocks for at most
  // 16 x 32 elements, else one block per SM
  const int chunks = (m->E + 31) / 32;
  int nb = op <= (size_t(2) << 20) ? 1
           : chunks <= EG_GMRES_CLUSTER_BLOCKS ? std::max(2, chunks)
                                               : std::max(2, std::min(sms, m->E));
  nb = std::min(nb, m->E);
  return std::min(nb, EG_COOP_MAX_BLOCKS);
}

template <typename T>
int launch_batch(Batcher& B, const std::vector<Submission*>& batch, int dev) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  std::vector<int> nb(batch.size());
  for (size_t i = 0; i < batch.size(); ++i) nb[i] = wanted_blocks_sms(batch[i]->ls, sms);
  BatchList list;
  list.n = (int)batch.size();
  int b0 = 0;
  size_t smem = 0;
  for (size_t i = 0; i < batch.size(); ++i) {
    const eg_ls* ls = batch[i]->ls;
    const eg_mesh* m = ls->lo->mesh;
    const int n = ls->lo->n;
    const int epb = (m->E + nb[i] - 1) / nb[i];
    const size_t elem_bytes = (size_t)n * sizeof(T);
    int ec = (int)((40 * 1024) / elem_bytes);
    ec = std::max(1, std::min(ec, epb));
    smem = std::max(smem, (size_t)ec * elem_bytes);
    list.e[i] = BatchEntry{ls->dargs, b0, nb[i], kind_of(m->dim, n), ec};
    b0 += nb[i];
  }
  const void* fn = (const void*)k_gmres_batch<T>;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, NT, smem);
  if (per_sm < 1 || b0 > sms * per_sm) {
    eg_set_error("batched GMRES kernel cannot be resident");
    return EG_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(eg_coop_mutex(dev));
  for (Submission* s : batch) EG_CUDA(cudaStreamWaitEvent(B.stream, s->ls->ev_in, 0));
  EG_CUDA(cudaMemsetAsync(B.bars, 0, sizeof(unsigned int) * 2 * list.n, B.stream));
  EG_CUDA(cudaMemsetAsync(B.err, 0, sizeof(int), B.stream));
  void* args[] = {&list, &B.bars, &B.err};
  EG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(b0), dim3(NT), args, smem, B.stream));
  EG_CUDA(cudaMemcpyAsync(B.h_err, B.err, sizeof(int), cudaMemcpyDeviceToHost, B.stream));
  EG_CUDA(cudaStreamSynchronize(B.stream));  // the grid has finished before the next one starts
  batch[0]->ls->lo->mesh->launches += 1;
  if (*B.h_err) {
    eg_set_error("batched GMRES: a barrier wait gave up");
    return EG_ERR_TIMEOUT;
  }
  return EG_OK;
}

template <typename T>
int stage_args(eg_ls* ls) {
  eg_mesh* m = ls->lo->mesh;
  if (!ls->dargs) {
    cudaError_t e = cudaMalloc(&ls->dargs, sizeof(CoopArgs<double>));
    if (e == cudaSuccess) e = cudaMallocHost(&ls->hargs, sizeof(CoopArgs<double>));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ls->ev_in, cudaEventDisableTiming);
    if (e != cudaSuccess) return eg_cuda_fail(e, "batched GMRES set-up");
  }
  // the staging buffer is the solver's own and its previous copy has
  // completed (every Newton iteration synchronises the mesh stream)
  coop_args<T>(ls, reinterpret_cast<CoopArgs<T>*>(ls->hargs));
  EG_CUDA(cudaMemcpyAsync(ls->dargs, ls->hargs, sizeof(CoopArgs<T>), cudaMemcpyHostToDevice, m->stream));
  EG_CUDA(cudaEventRecord(ls->ev_in, m->stream));
  return EG_OK;
}

}  // namespace

bool eg_gmres_batching() { return g_batching.load() != 0; }

int eg_gmres_wanted_blocks(const eg_ls* ls) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return wanted_blocks_sms(ls, sms);
}

void eg_batch_enter(int dev) { batcher(dev).active.fetch_add(1); }
void eg_batch_leave(int dev) { batcher(dev).active.fetch_sub(1); }

int eg_gmres_coop_batched(eg_ls* ls) {
  const bool f64 = ls->lo->prec == EG_F64;
  int st = f64 ? stage_args<double>(ls) : stage_args<float>(ls);
  if (st != EG_OK) return st;
  int dev = 0;
  cudaGetDevice(&dev);
  Batcher& B = batcher(dev);
  Submission sub;
  sub.ls = ls;
  std::unique_lock<std::mutex> lk(B.mu);
  st = ensure_batcher(B);
  if (st != EG_OK) return st;
  if (B.pending.empty()) B.first = std::chrono::steady_clock::now();
  B.pending.push_back(&sub);
  B.cv.notify_all();
  while (!sub.done) {
    const auto now = std::chrono::steady_clock::now();
    const bool full = (int)B.pending.size() >= std::max(1, B.active.load()) ||
                      (int)B.pending.size() >= kMaxBatch;
    const bool late = std::chrono::duration_cast<std::chrono::nanoseconds>(now - B.first).count() >=
                      g_window_ns.load();
    if (!B.launching && !B.pending.empty() && (full || late)) {
      // lead: pack pending solves of the first one's precision, in arrival
      // order, while their blocks fit on the SMs (first fit; the others wait
      // for the next launch)
      B.launching = true;
      int sms = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      const int prec = B.pending[0]->ls->lo->prec;
      std::vector<Submission*> batch, rest;
      int used = 0;
      for (Submission* s : B.pending) {
        const int w = wanted_blocks_sms(s->ls, sms);
        if (s->ls->lo->prec == prec && (int)batch.size() < kMaxBatch && used + w <= sms) {
          batch.push_back(s);
          used += w;
        } else {
          rest.push_back(s);
        }
      }
      B.pending.swap(rest);
      if (!B.pending.empty()) B.first = now;
      lk.unlock();
      const int rc = prec == EG_F64 ? launch_batch<double>(B, batch, dev) : launch_batch<float>(B, batch, dev);
      lk.lock();
      for (Submission* s : batch) {
        s->rc = rc;
        s->done = true;
      }
      B.launching = false;
      B.cv.notify_all();
    } else {
      B.cv.wait_for(lk, std::chrono::microseconds(20));
    }
  }
  return sub.rc;
}

extern "C" int eg_set_gmres_batching(int32_t enable, double window_us) {
  if ((enable != 0 && enable != 1) || !(window_us >= 0.0)) {
    eg_set_error("eg_set_gmres_batching: enable in {0, 1}, window_us >= 0");
    return EG_ERR_INVALID;
  }
  g_window_ns.store((long long)(window_us * 1000.0));
  g_batching.store(enable);
  return EG_OK;
}
