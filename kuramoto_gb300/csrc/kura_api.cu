// kura_api.cu -- C ABI of libkura (declared in include/kura.h).
//
// Owns the device buffers of one network and its batch of trajectories, launches
// the persistent DP45 kernel, drains its output rings and calls the observer
// callbacks.  Stands in for dp45_init/dp45_run/dp45_eval/dp45_destroy
// (dp45.h:7-11) and for the device-side parts of the reference main
// (kuramoto.cu:409-457, 552-585, 628-647).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "kura.h"
#include "kura_kernels.cuh"
#include "kura_tensor.h"

using kura::TrajG;

static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
#define CU(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return fail(e_ == cudaErrorMemoryAllocation ? KURA_ERR_NOMEM : KURA_ERR_CUDA,           \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                        \
  } while (0)

struct kura_handle {
  kura_config cfg{};
  int n = 0, ld = 0, B = 0, K = 0, bmax = 1, kmax = 8, coupling = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // device
  float* omega = nullptr;
  float* adj = nullptr;
  int8_t* adj8 = nullptr;  // N*A as int8 (KURA_ADJ_I8), rows of ld8
  int ld8 = 0;
  float* ph_hi = nullptr;
  float* ph_lo = nullptr;
  long long* ph_w = nullptr;
  float* g = nullptr;
  float2* xbuf = nullptr;
  float* part = nullptr;
  unsigned* bar = nullptr;
  int* err = nullptr;
  TrajG* traj = nullptr;
  float* t_eval = nullptr;
  float* out_r = nullptr;
  int* out_idx = nullptr;
  float* out_theta = nullptr;
  float* out_coup = nullptr;
  double* log_t = nullptr;
  double* log_h = nullptr;
  float* fin_theta = nullptr;
  float* fin_coup = nullptr;
  long long* counters = nullptr;
  int ring = 0, ring_alloc = 0, ring_dl = -1, log_cap = 0, n_eval = 0, t_eval_alloc = 0;
  double dt = 1, t1 = 0;
  int grid = 1, rows = 1, xs_smem = 0;
  size_t smem = 0;
  // host
  std::vector<TrajG> htraj;
  std::vector<std::vector<float>> order;
  std::vector<float> c1;
  std::vector<float> t_eval_h;
  std::vector<double> t0;
  std::vector<char> finished;  // the trajectory reached the end of a horizon (a later horizon continues it)
  bool omega_set = false, adj_set = false, horizon_set = false;
  long long launch_attempts = -1;  // step attempts per persistent launch (< 0: unbounded)
  long long budget = -1;           // step attempts of the current kura_advance call (< 0: none)
  // pinned host memory: the trajectory states and error flag of a launch in flight, and the
  // staging area its records are copied to while the next launch runs
  TrajG* traj_pin = nullptr;
  int* err_h = nullptr;
  char* stage = nullptr;
  size_t stage_bytes = 0;
  cudaEvent_t ev_stage = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  kura_stats stats{};
  kura::TensorEngine* te = nullptr;  // the tensor-core ensemble, when selected
};

// KURA_ENGINE_AUTO: tensor cores for a dense network with more than 8 trajectories
static int resolve_engine(const kura_config* c) {
  if (c->engine == KURA_ENGINE_TENSOR) return KURA_ENGINE_TENSOR;
  if (c->engine == KURA_ENGINE_PERSISTENT) return KURA_ENGINE_PERSISTENT;
  // a dense batch of two or more that keeps only the order parameter: the tensor engine reads the
  // BF16 adjacency once per RHS for the whole batch (a batch of 8 at N=65536: 0.95 of HBM against
  // the CUDA-core kernel's 0.34, 4.1x the throughput); per-step records need the persistent kernel
  if (c->coupling == KURA_COUPLING_DENSE && c->adj_storage != KURA_ADJ_I8 &&
      (c->batch > 8 || (c->batch >= 2 && c->dense_level == 0)))
    return KURA_ENGINE_TENSOR;
  return KURA_ENGINE_PERSISTENT;
}

extern "C" const char* kura_last_error(void) { return g_err.c_str(); }
void kura::set_last_error(const char* msg) { g_err = msg; }

static int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

static void plan(const kura_config* c, int* ld, int* bmax, int* kmax) {
  *ld = (int)((c->n + 31) / 32 * 32);
  *bmax = c->batch <= 1 ? 1 : 8;
  *kmax = c->k <= 8 ? 8 : 32;
}

static int validate(const kura_config* c) {
  if (!c) return fail(KURA_ERR_INVALID, "config is NULL");
  if (c->n < 1 || c->n > (1LL << 30)) return fail(KURA_ERR_INVALID, "n must be in [1, 2^30]");
  if (c->batch < 1) return fail(KURA_ERR_INVALID, "batch must be >= 1");
  if (c->engine < 0 || c->engine > 2) return fail(KURA_ERR_INVALID, "unknown engine");
  if (resolve_engine(c) == KURA_ENGINE_TENSOR) {
    if (c->coupling != KURA_COUPLING_DENSE)
      return fail(KURA_ERR_UNSUPPORTED, "the tensor-core ensemble needs a dense adjacency");
    if (c->batch > 128) return fail(KURA_ERR_UNSUPPORTED, "the tensor-core ensemble takes batch <= 128");
    if (c->dense_level != 0)
      return fail(KURA_ERR_UNSUPPORTED, "the tensor-core ensemble keeps the order parameter only (dense level 0)");
  } else if (c->batch > 8) {
    return fail(KURA_ERR_UNSUPPORTED, "batch > 8 needs a dense network on the tensor-core ensemble");
  }
  if (c->k < 0) return fail(KURA_ERR_INVALID, "k must be >= 0");
  if (c->coupling != KURA_COUPLING_DENSE && c->coupling != KURA_COUPLING_VOLCANO)
    return fail(KURA_ERR_INVALID, "unknown coupling");
  if (c->coupling == KURA_COUPLING_VOLCANO && c->k > 32)
    return fail(KURA_ERR_UNSUPPORTED, "regenerated volcano coupling supports k <= 32");
  if (c->coupling == KURA_COUPLING_VOLCANO && (long long)c->k * c->n >= (1LL << 62))
    return fail(KURA_ERR_INVALID, "k*n too large");
  if (!(c->atol > 0) && !c->fixed_step) return fail(KURA_ERR_INVALID, "atol must be > 0");
  if (c->rtol < 0) return fail(KURA_ERR_INVALID, "rtol must be >= 0");
  if (c->adj_storage != KURA_ADJ_F32 && c->adj_storage != KURA_ADJ_I8)
    return fail(KURA_ERR_INVALID, "unknown adjacency storage");
  if (c->adj_storage == KURA_ADJ_I8 && c->coupling == KURA_COUPLING_DENSE && c->k > 127)
    return fail(KURA_ERR_UNSUPPORTED, "int8 adjacency storage holds N*A exactly only for k <= 127");
  return KURA_OK;
}
static bool uses_i8(const kura_config* c) {
  return c->adj_storage == KURA_ADJ_I8 && c->coupling == KURA_COUPLING_DENSE && resolve_engine(c) != KURA_ENGINE_TENSOR;
}

extern "C" int kura_memory_required(const kura_config* c, int64_t* bytes) {
  int rc = validate(c);
  if (rc) return rc;
  if (resolve_engine(c) == KURA_ENGINE_TENSOR) {
    *bytes = (int64_t)kura::TensorEngine::memory_required(c->n, c->batch);
    return KURA_OK;
  }
  int ld, bmax, kmax;
  plan(c, &ld, &bmax, &kmax);
  long long B = c->batch, n = ld;
  long long b = 4 * n;                                   // omega
  if (c->coupling == KURA_COUPLING_DENSE) b += uses_i8(c) ? c->n * ((c->n + 15) / 16 * 16) : 4LL * c->n * n;
  b += 2 * B * n * (4 + 4 + 8);                          // phases
  b += 7 * B * n * 4;                                    // slopes
  b += 2 * B * n * 8;                                    // exchange
  b += B * n * 4 * 3;                                    // end record
  *bytes = b;
  return KURA_OK;
}

extern "C" void kura_destroy(kura_handle* h) {
  if (!h) return;
  cudaSetDevice(h->cfg.device);
  void* ptrs[] = {h->omega, h->adj, h->adj8, h->ph_hi, h->ph_lo, h->ph_w, h->g, h->xbuf, h->part, h->bar, h->err,
                  h->traj, h->t_eval, h->out_r, h->out_idx, h->out_theta, h->out_coup, h->log_t, h->log_h,
                  h->fin_theta, h->fin_coup, h->counters};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->ev_stage) cudaEventDestroy(h->ev_stage);
  if (h->traj_pin) cudaFreeHost(h->traj_pin);
  if (h->err_h) cudaFreeHost(h->err_h);
  if (h->stage) cudaFreeHost(h->stage);
  delete h->te;
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

template <typename T> static cudaError_t dalloc(T** p, size_t count) {
  cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
  if (e == cudaSuccess) e = cudaMemset(*p, 0, std::max<size_t>(count, 1) * sizeof(T));
  // the memset runs on the legacy default stream, which does not order with the non-blocking
  // stream a handle may own: wait for it, so that no later copy on that stream lands first
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  return e;
}

extern "C" int kura_create(const kura_config* cfg, kura_handle** out) {
  if (!out) return fail(KURA_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int rc = validate(cfg);
  if (rc) return rc;
  int ndev = 0;
  CU(cudaGetDeviceCount(&ndev));
  if (cfg->device < 0 || cfg->device >= ndev) return fail(KURA_ERR_INVALID, "device index out of range");
  CU(cudaSetDevice(cfg->device));
  auto* h = new kura_handle();
  h->cfg = *cfg;
  h->n = (int)cfg->n;
  h->B = cfg->batch;
  h->K = cfg->k;
  h->coupling = cfg->coupling;
  plan(cfg, &h->ld, &h->bmax, &h->kmax);
  auto bail = [&](int code) {
    kura_destroy(h);
    return code;
  };
#define CUH(call)                                                                               \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return bail(fail(e_ == cudaErrorMemoryAllocation ? KURA_ERR_NOMEM : KURA_ERR_CUDA,        \
                       std::string(#call) + ": " + cudaGetErrorString(e_)));                    \
  } while (0)
  if (cfg->stream) {
    h->stream = (cudaStream_t)cfg->stream;
  } else {
    CUH(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
  }
  CUH(cudaEventCreate(&h->ev0));
  CUH(cudaEventCreate(&h->ev1));
  h->htraj.assign(h->B, TrajG{});
  for (auto& T : h->htraj) T.status = 1;  // no state yet
  h->c1.assign(h->B, 0.f);
  h->t0.assign(h->B, 0.0);
  h->finished.assign(h->B, 0);
  h->order.assign(h->B, {});
  if (resolve_engine(cfg) == KURA_ENGINE_TENSOR) {
    h->te = new kura::TensorEngine();
    int rc2 = h->te->init(cfg->n, cfg->k, cfg->batch, cfg->seed, cfg->atol, cfg->rtol, cfg->fixed_step,
                          cfg->dense_level, cfg->device, h->stream);
    if (rc2) return bail(fail(rc2, kura::TensorEngine::last_error()));
    h->stats.grid = 0;
    h->stats.block = 160;
    *out = h;
    return KURA_OK;
  }

  // grid: one or more CTAs per SM, all co-resident (cooperative launch)
  int dev = cfg->device, sms = 0, coop = 0;
  CUH(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CUH(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) return bail(fail(KURA_ERR_UNSUPPORTED, "device lacks cooperative launch"));
  int G = sms;
  int rows = ceil_div(h->n, G);
  int bps = 0;
  CUH(kura::persistent_config(uses_i8(cfg) ? kura::COUP_DENSE_I8 : h->coupling, h->bmax, h->kmax, &h->smem, &bps, rows, &h->xs_smem));
  if (bps < 1) return bail(fail(KURA_ERR_UNSUPPORTED, "persistent kernel does not fit on an SM"));
  G = sms * std::min(bps, 1);
  // at least 64 rows per CTA for the regenerated coupling (its cost per CTA is mostly
  // fixed); 16 for the dense one, whose rows are long
  G = std::min(G, std::max(1, ceil_div(h->n, h->coupling == KURA_COUPLING_DENSE ? 16 : 64)));
  rows = ceil_div(h->n, G);
  G = ceil_div(h->n, rows);
  CUH(kura::persistent_config(uses_i8(cfg) ? kura::COUP_DENSE_I8 : h->coupling, h->bmax, h->kmax, &h->smem, &bps, rows, &h->xs_smem));
  if (bps < 1) return bail(fail(KURA_ERR_UNSUPPORTED, "persistent kernel shared memory exceeds an SM"));
  h->grid = G;
  h->rows = rows;

  size_t ld = h->ld, B = h->B;
  CUH(dalloc(&h->omega, ld));
  if (uses_i8(cfg)) {
    h->ld8 = (h->n + 15) / 16 * 16;
    CUH(dalloc(&h->adj8, (size_t)h->n * h->ld8));
  } else if (h->coupling == KURA_COUPLING_DENSE) {
    CUH(dalloc(&h->adj, (size_t)h->n * ld));
  }
  CUH(dalloc(&h->ph_hi, 2 * B * ld));
  CUH(dalloc(&h->ph_lo, 2 * B * ld));
  CUH(dalloc(&h->ph_w, 2 * B * ld));
  CUH(dalloc(&h->g, 7 * B * ld));
  CUH(dalloc(&h->xbuf, 2 * B * ld));
  CUH(dalloc(&h->part, 2 * (size_t)G * B * kura::PW_MAX));
  CUH(dalloc(&h->bar, 4));
  CUH(dalloc(&h->err, 4));
  CUH(dalloc(&h->traj, B));
  CUH(dalloc(&h->fin_theta, B * ld));
  CUH(dalloc(&h->fin_coup, 2 * B * ld));
  CUH(dalloc(&h->counters, 4));
  h->log_cap = 4096;
  CUH(dalloc(&h->log_t, B * (size_t)h->log_cap));
  CUH(dalloc(&h->log_h, B * (size_t)h->log_cap));
  CUH(cudaMallocHost((void**)&h->traj_pin, sizeof(TrajG) * B));
  CUH(cudaMallocHost((void**)&h->err_h, sizeof(int)));
  CUH(cudaEventCreateWithFlags(&h->ev_stage, cudaEventDisableTiming));
  h->htraj.assign(B, TrajG{});
  for (auto& T : h->htraj) {
    T.status = 1;  // no state yet
    T.c1 = 0.f;
  }
  h->c1.assign(B, 0.f);
  h->t0.assign(B, 0.0);
  h->finished.assign(B, 0);
  h->order.assign(B, {});
  h->stats.grid = G;
  h->stats.block = kura::KT;
  *out = h;
  return KURA_OK;
#undef CUH
}

static int check_traj(kura_handle* h, int traj) {
  if (!h) return fail(KURA_ERR_INVALID, "handle is NULL");
  if (traj < 0 || traj >= h->B) return fail(KURA_ERR_INVALID, "trajectory index out of range");
  return KURA_OK;
}

extern "C" int kura_set_frequencies(kura_handle* h, const float* omega, int64_t n) {
  if (!h || !omega) return fail(KURA_ERR_INVALID, "NULL argument");
  if (n != h->n) return fail(KURA_ERR_INVALID, "frequency count differs from n");
  CU(cudaSetDevice(h->cfg.device));
  if (h->te) {
    int rc = h->te->set_frequencies(omega);
    if (rc) return fail(rc, kura::TensorEngine::last_error());
    h->omega_set = true;
    return KURA_OK;
  }
  CU(cudaMemcpyAsync(h->omega, omega, sizeof(float) * n, cudaMemcpyHostToDevice, h->stream));
  CU(cudaStreamSynchronize(h->stream));
  h->omega_set = true;
  return KURA_OK;
}

extern "C" int kura_set_adjacency(kura_handle* h, const float* adj, int64_t n) {
  if (!h || !adj) return fail(KURA_ERR_INVALID, "NULL argument");
  if (h->coupling != KURA_COUPLING_DENSE) return fail(KURA_ERR_INVALID, "adjacency is regenerated (volcano coupling)");
  if (n != h->n) return fail(KURA_ERR_INVALID, "adjacency size differs from n");
  CU(cudaSetDevice(h->cfg.device));
  if (h->te) {
    int rc = h->te->set_adjacency(adj);
    if (rc) return fail(rc, kura::TensorEngine::last_error());
    h->adj_set = true;
    return KURA_OK;
  }
  if (h->adj8) {
    // integers N*A_ij in [-127, 127] that reproduce A_ij exactly as float(k) * float(1/N)
    const float invn = 1.0f / (float)n;
    std::vector<int8_t> q((size_t)n * h->ld8, 0);
    for (int64_t i = 0; i < n; ++i)
      for (int64_t j = 0; j < n; ++j) {
        const float a = adj[i * n + j];
        const double k = std::rint((double)a * (double)n);
        if (!(std::fabs(k) <= 127.0) || (float)k * invn != a)
          return fail(KURA_ERR_UNSUPPORTED, "adjacency entry (" + std::to_string(i) + ", " + std::to_string(j) +
                                                ") is not an integer multiple of 1/N in [-127, 127]: store it as "
                                                "float32 (KURA_ADJ_F32)");
        q[(size_t)i * h->ld8 + j] = (int8_t)k;
      }
    CU(cudaMemcpyAsync(h->adj8, q.data(), q.size(), cudaMemcpyHostToDevice, h->stream));
  } else {
    CU(cudaMemcpy2DAsync(h->adj, sizeof(float) * h->ld, adj, sizeof(float) * n, sizeof(float) * n, n,
                         cudaMemcpyHostToDevice, h->stream));
  }
  CU(cudaStreamSynchronize(h->stream));
  h->adj_set = true;
  return KURA_OK;
}

extern "C" int kura_generate_adjacency(kura_handle* h) {
  if (!h) return fail(KURA_ERR_INVALID, "handle is NULL");
  if (h->coupling != KURA_COUPLING_DENSE) return fail(KURA_ERR_INVALID, "adjacency is regenerated (volcano coupling)");
  CU(cudaSetDevice(h->cfg.device));
  if (h->te) {
    int rc = h->te->generate_adjacency();
    if (rc) return fail(rc, kura::TensorEngine::last_error());
    h->adj_set = true;
    return KURA_OK;
  }
  int words = (h->K + 31) / 32;
  uint32_t* bits = nullptr;
  if (words > 0) {
    CU(cudaMallocAsync((void**)&bits, sizeof(uint32_t) * (size_t)words * h->n, h->stream));
    CU(kura::launch_volcano_words(h->cfg.seed, h->n, h->K, words, bits, h->stream));
  }
  if (h->adj8)
    CU(kura::launch_volcano_adjacency_i8(bits, h->n, h->K, words, h->ld8, h->adj8, h->stream));
  else
    CU(kura::launch_volcano_adjacency(bits, h->n, h->K, words, h->ld, h->adj, h->stream));
  if (bits) CU(cudaFreeAsync(bits, h->stream));
  CU(cudaStreamSynchronize(h->stream));
  h->adj_set = true;
  return KURA_OK;
}

extern "C" int kura_get_adjacency(kura_handle* h, float* adj, int64_t n) {
  if (!h || !adj) return fail(KURA_ERR_INVALID, "NULL argument");
  if (h->coupling != KURA_COUPLING_DENSE || !h->adj_set) return fail(KURA_ERR_INVALID, "no stored adjacency");
  if (n != h->n) return fail(KURA_ERR_INVALID, "adjacency size differs from n");
  CU(cudaSetDevice(h->cfg.device));
  if (h->te) {
    int rc = h->te->get_adjacency(adj);
    return rc ? fail(rc, kura::TensorEngine::last_error()) : KURA_OK;
  }
  if (h->adj8) {
    std::vector<int8_t> q((size_t)n * h->ld8);
    CU(cudaMemcpyAsync(q.data(), h->adj8, q.size(), cudaMemcpyDeviceToHost, h->stream));
    CU(cudaStreamSynchronize(h->stream));
    const float invn = 1.0f / (float)n;
    for (int64_t i = 0; i < n; ++i)
      for (int64_t j = 0; j < n; ++j) adj[i * n + j] = (float)q[(size_t)i * h->ld8 + j] * invn;
    return KURA_OK;
  }
  CU(cudaMemcpy2DAsync(adj, sizeof(float) * n, h->adj, sizeof(float) * h->ld, sizeof(float) * n, n,
                       cudaMemcpyDeviceToHost, h->stream));
  CU(cudaStreamSynchronize(h->stream));
  return KURA_OK;
}

extern "C" int kura_set_coupling(kura_handle* h, int32_t traj, float c) {
  int rc = check_traj(h, traj);
  if (rc) return rc;
  h->c1[traj] = c;
  h->htraj[traj].c1 = c;
  return KURA_OK;
}

static int set_state_common(kura_handle* h, int traj, const float* dev_theta, double t, double step) {
  if (!h->te) {
    size_t off = (size_t)traj * h->ld;  // physical buffer 0
    CU(kura::launch_init_state(dev_theta, h->n, h->ld, h->ph_hi + off, h->ph_lo + off, h->ph_w + off, h->stream));
    CU(cudaStreamSynchronize(h->stream));
  }
  h->finished[traj] = 0;
  TrajG& T = h->htraj[traj];
  float c = T.c1;
  T = TrajG{};
  T.c1 = c;
  T.t = t;
  T.h = step;
  T.t_last = t;
  T.t1 = t;
  T.status = 0;
  T.need_k1 = 1;
  T.need_init = 0;
  h->horizon_set = false;
  if (h->te) {
    int rc = h->te->set_state(traj, dev_theta, T);
    if (rc) return fail(rc, kura::TensorEngine::last_error());
  }
  return KURA_OK;
}

extern "C" int kura_set_state(kura_handle* h, int32_t traj, const float* theta, double t, double step) {
  int rc = check_traj(h, traj);
  if (rc) return rc;
  if (!theta) return fail(KURA_ERR_INVALID, "theta is NULL");
  if (!(step > 0)) return fail(KURA_ERR_INVALID, "step must be > 0");
  CU(cudaSetDevice(h->cfg.device));
  float* tmp = h->te ? h->te->staging(traj) : h->fin_theta + (size_t)traj * h->ld;
  CU(cudaMemcpyAsync(tmp, theta, sizeof(float) * h->n, cudaMemcpyHostToDevice, h->stream));
  return set_state_common(h, traj, tmp, t, step);
}

extern "C" int kura_set_state_device(kura_handle* h, int32_t traj, const float* theta_device, double t,
                                     double step) {
  int rc = check_traj(h, traj);
  if (rc) return rc;
  if (!theta_device) return fail(KURA_ERR_INVALID, "theta is NULL");
  if (!(step > 0)) return fail(KURA_ERR_INVALID, "step must be > 0");
  CU(cudaSetDevice(h->cfg.device));
  return set_state_common(h, traj, theta_device, t, step);
}

extern "C" int kura_set_horizon(kura_handle* h, double t1, double dt, int32_t initial_record) {
  if (!h) return fail(KURA_ERR_INVALID, "handle is NULL");
  if (!(dt > 0)) return fail(KURA_ERR_INVALID, "dt must be > 0");
  // either every trajectory has a fresh state (kura_set_state) or every one finished the
  // previous horizon, which this one then continues from where it stopped
  int fresh = 0, cont = 0;
  for (int b = 0; b < h->B; ++b) {
    const TrajG& T = h->htraj[b];
    if (T.status == 0 && T.need_k1 == 1) fresh++;
    else if (T.status == 1 && h->finished[b]) cont++;
  }
  if (fresh != h->B && cont != h->B)
    return fail(KURA_ERR_INVALID, "set the state of every trajectory (or finish a run) before the horizon");
  const bool continuing = cont == h->B;
  double tmin = h->htraj[0].t;
  for (int b = 1; b < h->B; ++b) tmin = std::min(tmin, h->htraj[b].t);
  CU(cudaSetDevice(h->cfg.device));
  // t_eval = dt*n for n = int(t0/dt)+1 .. int(t1/dt), in float like the reference (a resumed
  // run rebuilds it the same way from its start time, kuramoto.cu:543-550)
  float t0f = (float)tmin, dtf = (float)dt, t1f = (float)t1;
  int n0 = int(t0f / dtf) + 1, n1 = int(t1f / dtf) + 1;
  h->t_eval_h.clear();
  for (int n = n0; n < n1; ++n) h->t_eval_h.push_back(dtf * n);
  h->n_eval = (int)h->t_eval_h.size();
  // A trajectory that starts (or continues) after the earliest one owes no output at or
  // before its own time.  A continued trajectory keeps its slopes (FSAL) and step size as
  // after an accepted step.  Trajectories that start at the earliest time take the grid as
  // the reference builds it, from its first point.
  auto first_eval = [&](const TrajG& T) {
    int e = 0;
    if (continuing || T.t > tmin)
      while (e < h->n_eval && T.t >= (double)h->t_eval_h[e]) e++;
    return e;
  };
  for (int b = 0; b < h->B; ++b) {
    if (continuing) h->htraj[b].status = 0;
    h->finished[b] = 0;
  }
  h->dt = dt;
  h->t1 = t1;
  if (h->te) {
    for (int b = 0; b < h->B; ++b) {
      TrajG& T = h->htraj[b];
      T.t1 = t1;
      T.eval_i = T.eval_end = first_eval(T);
      T.need_init = initial_record ? 1 : 0;
      T.out_count = 0;
      T.log_count = 0;
      h->order[b].clear();
      h->t0[b] = T.t;
    }
    h->ring = h->n_eval + 2;
    int rc = h->te->set_horizon(h->t_eval_h, h->ring, h->htraj);
    if (rc) return fail(rc, kura::TensorEngine::last_error());
    h->horizon_set = true;
    return KURA_OK;
  }
  if (h->n_eval > h->t_eval_alloc || !h->t_eval) {
    if (h->t_eval) cudaFree(h->t_eval);
    h->t_eval = nullptr;
    CU(dalloc(&h->t_eval, h->t_eval_h.size()));
    h->t_eval_alloc = h->n_eval;
  }
  if (h->n_eval)
    CU(cudaMemcpyAsync(h->t_eval, h->t_eval_h.data(), sizeof(float) * h->n_eval, cudaMemcpyHostToDevice, h->stream));
  // output ring: every record when only r is kept, else bounded by a 2 GiB budget
  int dl = h->cfg.dense_level;
  long long per = (long long)h->B * h->ld * 4 * ((dl >= 1 ? 1 : 0) + (dl >= 2 ? 2 : 0));
  long long want = (long long)h->n_eval + 2;
  long long ring = want;
  if (per > 0) ring = std::min<long long>(want, std::max<long long>(4, (2LL << 30) / per));
  if (ring > h->ring_alloc || dl != h->ring_dl) {
    for (void* p : {(void*)h->out_r, (void*)h->out_idx, (void*)h->out_theta, (void*)h->out_coup})
      if (p) cudaFree(p);
    h->out_r = nullptr; h->out_idx = nullptr; h->out_theta = nullptr; h->out_coup = nullptr;
    CU(dalloc(&h->out_r, (size_t)h->B * ring));
    CU(dalloc(&h->out_idx, (size_t)h->B * ring));
    if (dl >= 1) CU(dalloc(&h->out_theta, (size_t)h->B * ring * h->ld));
    if (dl >= 2) CU(dalloc(&h->out_coup, (size_t)h->B * ring * 2 * h->ld));
    h->ring_alloc = (int)ring;
    h->ring_dl = dl;
  }
  h->ring = h->ring_alloc;
  for (int b = 0; b < h->B; ++b) {
    TrajG& T = h->htraj[b];
    T.t1 = t1;
    T.eval_i = T.eval_end = first_eval(T);
    T.need_init = initial_record ? 1 : 0;
    T.out_count = 0;
    T.log_count = 0;
    h->order[b].clear();
    h->t0[b] = T.t;
  }
  h->horizon_set = true;
  return KURA_OK;
}

// enqueues one persistent launch (state upload, kernel, error flag and state download)
static int launch_begin(kura_handle* h, int mode, bool log_steps) {
  kura::KParams p{};
  p.n = h->n; p.ld = h->ld; p.batch = h->B; p.k = h->K; p.coupling = h->adj8 ? kura::COUP_DENSE_I8 : h->coupling;
  p.dense_level = h->cfg.dense_level; p.fixed = h->cfg.fixed_step; p.rows = h->rows; p.seed = h->cfg.seed;
  p.mode = mode;
  p.omega = h->omega; p.adj = h->adj;
  p.ph_hi = h->ph_hi; p.ph_lo = h->ph_lo; p.ph_w = h->ph_w; p.g = h->g; p.xbuf = h->xbuf; p.part = h->part;
  p.bar = h->bar; p.err = h->err; p.traj = h->traj;
  p.t_eval = h->t_eval; p.n_eval = h->n_eval;
  p.atol = h->cfg.atol; p.rtol = h->cfg.rtol; p.dt = h->dt;
  p.out_r = h->out_r; p.out_idx = h->out_idx; p.out_theta = h->out_theta; p.out_coup = h->out_coup;
  p.ring = h->ring;
  p.log_t = h->log_t; p.log_h = h->log_h; p.log_cap = log_steps ? h->log_cap : 0;
  p.max_attempts = h->launch_attempts > 0 ? h->launch_attempts : -1;
  if (h->budget > 0) p.max_attempts = h->budget;  // kura_advance: one launch of at most that many
  const char* to = getenv("KURA_BARRIER_TIMEOUT_MS");
  double ms = to ? atof(to) : 20000.0;
  p.timeout_ns = (unsigned long long)(ms * 1e6);
  const char* extra = getenv("KURA_TEST_BARRIER_EXTRA");
  p.bar_extra = extra ? (unsigned)atoi(extra) : 0u;
  p.fin_theta = h->fin_theta; p.fin_coup = h->fin_coup;
  p.xs_smem = h->xs_smem;
  p.counters = h->counters;
  p.adj8 = h->adj8;
  p.ld8 = h->ld8;
  p.invn = 1.0f / (float)h->n;
  std::memcpy(h->traj_pin, h->htraj.data(), sizeof(TrajG) * h->B);
  CU(cudaMemcpyAsync(h->traj, h->traj_pin, sizeof(TrajG) * h->B, cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemsetAsync(h->bar, 0, sizeof(unsigned), h->stream));
  CU(cudaMemsetAsync(h->err, 0, sizeof(int), h->stream));
  CU(cudaEventRecord(h->ev0, h->stream));
  CU(kura::launch_persistent(p, h->grid, h->bmax, h->kmax, h->smem, h->stream));
  CU(cudaEventRecord(h->ev1, h->stream));
  CU(cudaMemcpyAsync(h->err_h, h->err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(h->traj_pin, h->traj, sizeof(TrajG) * h->B, cudaMemcpyDeviceToHost, h->stream));
  return KURA_OK;
}
// waits for the launch enqueued by launch_begin
static int launch_end(kura_handle* h) {
  CU(cudaStreamSynchronize(h->stream));
  std::memcpy(h->htraj.data(), h->traj_pin, sizeof(TrajG) * h->B);
  float ms_k = 0;
  CU(cudaEventElapsedTime(&ms_k, h->ev0, h->ev1));
  h->stats.kernel_ms += ms_k;
  h->stats.launches++;
  const int err = *h->err_h;
  if (err) return fail(err, err == KURA_ERR_BARRIER_TIMEOUT ? "grid barrier timed out" : "persistent kernel aborted");
  return KURA_OK;
}
static int launch(kura_handle* h, int mode, bool log_steps) {
  int rc = launch_begin(h, mode, log_steps);
  return rc ? rc : launch_end(h);
}

extern "C" int kura_run(kura_handle* h, const kura_callbacks* cb) {
  if (!h) return fail(KURA_ERR_INVALID, "handle is NULL");
  if (!h->omega_set) return fail(KURA_ERR_INVALID, "frequencies not set");
  if (h->coupling == KURA_COUPLING_DENSE && !h->adj_set) return fail(KURA_ERR_INVALID, "adjacency not set");
  if (!h->horizon_set) return fail(KURA_ERR_INVALID, "horizon not set (kura_set_horizon after kura_set_state)");
  CU(cudaSetDevice(h->cfg.device));
  if (h->te) {
    int rc = h->te->run(h->htraj, h->stats, h->budget);
    if (rc) return fail(rc, kura::TensorEngine::last_error());
    long long acc = 0, rej = 0;
    int errc = 0;
    std::vector<float> rbuf;
    std::vector<int> ibuf;
    for (int b = 0; b < h->B; ++b) {
      TrajG& T = h->htraj[b];
      acc += T.accepted;
      rej += T.rejected;
      if (T.status < 0 && !errc) errc = T.status;
      rbuf.resize(std::max(T.out_count, 1));
      ibuf.resize(std::max(T.out_count, 1));
      if (T.out_count > 0) {
        rc = h->te->read_order(b, T.out_count, rbuf.data(), ibuf.data());
        if (rc) return fail(rc, kura::TensorEngine::last_error());
      }
      for (int q = 0; q < T.out_count; ++q) {
        h->order[b].push_back(rbuf[q]);
        if (cb && cb->on_output) {
          const int idx = ibuf[q];
          const double te = idx < 0 ? h->t0[b] : (double)h->t_eval_h[idx];
          if (cb->on_output(cb->user, b, idx, te, rbuf[q], nullptr, nullptr))
            return fail(KURA_ERR_CALLBACK, "on_output aborted");
        }
      }
    }
    h->stats.accepted = acc;
    h->stats.rejected = rej;
    if (errc) {
      std::string m = errc == KURA_ERR_STEP_UNDERFLOW ? "step size underflow"
                      : errc == KURA_ERR_UNSUPPORTED ? "more than 32 output times crossed in one step"
                                                      : "non-finite error norm";
      for (int b = 0; b < h->B; ++b) {
        const TrajG& T = h->htraj[b];
        if (T.status == errc) {
          char buf[200];
          snprintf(buf, sizeof buf, " (trajectory %d: t %.9g, h %.3g, t_last %.9g, outputs %d..%d of %d)", b, T.t,
                   T.h, T.t_last, T.eval_i, T.eval_end, h->n_eval);
          m += buf;
          break;
        }
      }
      return fail(errc, m);
    }
    for (int b = 0; b < h->B; ++b) h->finished[b] = h->htraj[b].status == 1;
    if (h->budget > 0) {  // the records were read: the next advance writes its own from slot 0
      for (auto& T : h->htraj) T.out_count = 0;
      rc = h->te->sync_traj(h->htraj, true);
      if (rc) return fail(rc, kura::TensorEngine::last_error());
    }
    return KURA_OK;
  }
  const bool log_steps = cb && cb->on_step;
  const bool want_out = cb && cb->on_output, want_chunk = cb && cb->on_chunk;
  const int dl = h->cfg.dense_level;
  std::vector<long long> step_no(h->B, 0);
  for (int b = 0; b < h->B; ++b) step_no[b] = h->htraj[b].accepted;
  // Records of launch k are copied into pinned staging memory on the stream, launch k+1 is
  // enqueued behind the copies, and the observers consume launch k's records while k+1 runs.
  struct Seg {
    size_t r, idx, th, cp, lt, lh, chunk;
    int cnt, logs;
  };
  std::vector<Seg> seg(h->B);
  auto progress = [&]() {
    long long v = 0;
    for (auto& T : h->htraj) v += T.accepted + T.rejected + T.eval_i;
    return v;
  };
  int rc = launch(h, kura::MODE_INTEGRATE, log_steps);
  if (rc) return rc;
  long long before = 0;
  int stall = 0;
  while (true) {
    // ---- stage the records of the launch that just ended
    size_t need = 0;
    auto take = [&](size_t bytes) {
      size_t o = need;
      need += (bytes + 255) / 256 * 256;
      return o;
    };
    for (int b = 0; b < h->B; ++b) {
      const TrajG& T = h->htraj[b];
      Seg& S = seg[b];
      S.cnt = T.out_count;
      S.logs = log_steps ? std::min(T.log_count, h->log_cap) : 0;
      S.r = take(sizeof(float) * S.cnt);
      S.idx = take(sizeof(int) * S.cnt);
      S.th = take(want_out && dl >= 1 ? sizeof(float) * S.cnt * h->ld : 0);
      S.cp = take(want_out && dl >= 2 ? sizeof(float) * S.cnt * 2 * h->ld : 0);
      S.lt = take(sizeof(double) * S.logs);
      S.lh = take(sizeof(double) * S.logs);
      S.chunk = take(want_chunk ? sizeof(float) * h->n : 0);
    }
    if (need > h->stage_bytes) {
      if (h->stage) CU(cudaFreeHost(h->stage));
      h->stage = nullptr;
      h->stage_bytes = 0;
      CU(cudaMallocHost((void**)&h->stage, need));
      h->stage_bytes = need;
    }
    char* st = h->stage;
    for (int b = 0; b < h->B; ++b) {
      const TrajG& T = h->htraj[b];
      const Seg& S = seg[b];
      if (S.cnt > 0) {
        CU(cudaMemcpyAsync(st + S.r, h->out_r + (size_t)b * h->ring, sizeof(float) * S.cnt, cudaMemcpyDeviceToHost,
                           h->stream));
        CU(cudaMemcpyAsync(st + S.idx, h->out_idx + (size_t)b * h->ring, sizeof(int) * S.cnt, cudaMemcpyDeviceToHost,
                           h->stream));
        if (want_out && dl >= 1)
          CU(cudaMemcpyAsync(st + S.th, h->out_theta + (size_t)b * h->ring * h->ld, sizeof(float) * S.cnt * h->ld,
                             cudaMemcpyDeviceToHost, h->stream));
        if (want_out && dl >= 2)
          CU(cudaMemcpyAsync(st + S.cp, h->out_coup + (size_t)b * h->ring * 2 * h->ld,
                             sizeof(float) * S.cnt * 2 * h->ld, cudaMemcpyDeviceToHost, h->stream));
      }
      if (S.logs > 0) {
        CU(cudaMemcpyAsync(st + S.lt, h->log_t + (size_t)b * h->log_cap, sizeof(double) * S.logs,
                           cudaMemcpyDeviceToHost, h->stream));
        CU(cudaMemcpyAsync(st + S.lh, h->log_h + (size_t)b * h->log_cap, sizeof(double) * S.logs,
                           cudaMemcpyDeviceToHost, h->stream));
      }
      if (want_chunk) {
        size_t off = ((size_t)T.rot_y * h->B + b) * h->ld;
        CU(kura::launch_unwrap(h->ph_hi + off, h->ph_lo + off, h->ph_w + off, h->n, h->fin_theta + (size_t)b * h->ld,
                               h->stream));
        CU(cudaMemcpyAsync(st + S.chunk, h->fin_theta + (size_t)b * h->ld, sizeof(float) * h->n,
                           cudaMemcpyDeviceToHost, h->stream));
      }
    }
    CU(cudaEventRecord(h->ev_stage, h->stream));
    std::vector<double> chunk_t(h->B), chunk_h(h->B);
    bool done = true;
    int errc = 0;
    for (int b = 0; b < h->B; ++b) {
      TrajG& T = h->htraj[b];
      chunk_t[b] = T.t;
      chunk_h[b] = T.h;
      T.out_count = 0;
      T.log_count = 0;
      if (T.status == 0 || T.eval_i < T.eval_end) done = false;
      if (T.status < 0 && !errc) errc = T.status;
    }
    const long long after = progress();
    stall = (after == before) ? stall + 1 : 0;
    before = after;
    // ---- the next launch runs while the observers read the staged records
    bool running = false;
    if (!done && !errc && stall <= 2 && h->budget <= 0) {
      rc = launch_begin(h, kura::MODE_INTEGRATE, log_steps);
      if (rc) return rc;
      running = true;
    }
    CU(cudaEventSynchronize(h->ev_stage));
    int abort = 0;
    for (int b = 0; b < h->B && !abort; ++b) {
      const Seg& S = seg[b];
      const float* r = (const float*)(st + S.r);
      const int* idx = (const int*)(st + S.idx);
      for (int q = 0; q < S.cnt; ++q) h->order[b].push_back(r[q]);
      if (want_out) {
        for (int q = 0; q < S.cnt && !abort; ++q) {
          const double te = idx[q] < 0 ? h->t0[b] : (double)h->t_eval_h[idx[q]];
          const float* th = dl >= 1 ? (const float*)(st + S.th) + (size_t)q * h->ld : nullptr;
          const float* cp = dl >= 2 ? (const float*)(st + S.cp) + (size_t)q * 2 * h->ld : nullptr;
          if (cb->on_output(cb->user, b, idx[q], te, r[q], th, cp)) abort = 1;
        }
      }
      const double* lt = (const double*)(st + S.lt);
      const double* lh = (const double*)(st + S.lh);
      for (int q = 0; q < S.logs && !abort; ++q)
        if (cb->on_step(cb->user, b, lt[q], lh[q], ++step_no[b])) abort = 2;
    }
    if (want_chunk)
      for (int b = 0; b < h->B && !abort; ++b)
        if (cb->on_chunk(cb->user, b, chunk_t[b], chunk_h[b], (const float*)(st + seg[b].chunk))) abort = 3;
    if (running) {
      rc = launch_end(h);
      if (rc) return rc;
    }
    if (abort) return fail(KURA_ERR_CALLBACK, abort == 1 ? "on_output aborted" : abort == 2 ? "on_step aborted"
                                                                                          : "on_chunk aborted");
    if (errc) {
      const char* m = errc == KURA_ERR_STEP_UNDERFLOW ? "step size underflow" : "non-finite error norm";
      return fail(errc, m);
    }
    if (done || h->budget > 0) break;
    if (!running) return fail(KURA_ERR_INVALID, "integration made no progress");
  }
  long long acc = 0, rej = 0, bars = 0;
  for (auto& T : h->htraj) { acc += T.accepted; rej += T.rejected; }
  CU(cudaMemcpy(&bars, h->counters, sizeof(long long), cudaMemcpyDeviceToHost));
  h->stats.accepted = acc;
  h->stats.rejected = rej;
  h->stats.barriers = bars;
  for (int b = 0; b < h->B; ++b) h->finished[b] = h->htraj[b].status == 1;
  return KURA_OK;
}

extern "C" int kura_advance(kura_handle* h, const kura_callbacks* cb, int64_t attempts, int32_t* running) {
  if (!h) return fail(KURA_ERR_INVALID, "handle is NULL");
  if (attempts < 1) return fail(KURA_ERR_INVALID, "attempts must be >= 1");
  h->budget = attempts;
  int rc = kura_run(h, cb);
  h->budget = -1;
  if (rc) return rc;
  if (running) {
    int r = 0;
    for (const auto& T : h->htraj) r += T.status == 0 ? 1 : 0;
    *running = r;
  }
  return KURA_OK;
}

extern "C" int kura_get_state(kura_handle* h, int32_t traj, float* theta, double* t, double* step) {
  int rc = check_traj(h, traj);
  if (rc) return rc;
  CU(cudaSetDevice(h->cfg.device));
  const TrajG& T = h->htraj[traj];
  if (theta && h->te) {
    int rc2 = h->te->get_state(traj, T.rot_y, theta);
    if (rc2) return fail(rc2, kura::TensorEngine::last_error());
  } else if (theta) {
    size_t off = ((size_t)T.rot_y * h->B + traj) * h->ld;
    float* tmp = h->fin_theta + (size_t)traj * h->ld;
    CU(kura::launch_unwrap(h->ph_hi + off, h->ph_lo + off, h->ph_w + off, h->n, tmp, h->stream));
    CU(cudaMemcpyAsync(theta, tmp, sizeof(float) * h->n, cudaMemcpyDeviceToHost, h->stream));
    CU(cudaStreamSynchronize(h->stream));
  }
  if (t) *t = T.t;
  if (step) *step = T.h;
  return KURA_OK;
}

extern "C" int kura_get_order(kura_handle* h, int32_t traj, float* r, int64_t cap, int64_t* count) {
  int rc = check_traj(h, traj);
  if (rc) return rc;
  const auto& v = h->order[traj];
  if (count) *count = (int64_t)v.size();
  if (r) std::memcpy(r, v.data(), sizeof(float) * std::min<size_t>(v.size(), (size_t)std::max<int64_t>(cap, 0)));
  return KURA_OK;
}

extern "C" int kura_final_record(kura_handle* h, int32_t traj, float* theta, float* couplings, double* t,
                                 double* step) {
  int rc = check_traj(h, traj);
  if (rc) return rc;
  if (!h->horizon_set) return fail(KURA_ERR_INVALID, "no run to report");
  CU(cudaSetDevice(h->cfg.device));
  if (h->te) {
    rc = h->te->evaluate(1, traj, theta, couplings);
    if (rc) return fail(rc, kura::TensorEngine::last_error());
    if (t) *t = h->htraj[traj].t;
    if (step) *step = h->htraj[traj].h;
    return KURA_OK;
  }
  rc = launch(h, kura::MODE_FINAL, false);
  if (rc) return rc;
  if (theta) CU(cudaMemcpy(theta, h->fin_theta + (size_t)traj * h->ld, sizeof(float) * h->n, cudaMemcpyDeviceToHost));
  if (couplings)
    CU(cudaMemcpy(couplings, h->fin_coup + (size_t)traj * 2 * h->ld, sizeof(float) * 2 * h->n, cudaMemcpyDeviceToHost));
  if (t) *t = h->htraj[traj].t;
  if (step) *step = h->htraj[traj].h;
  return KURA_OK;
}

extern "C" int kura_rhs(kura_handle* h, int32_t traj, const float* theta, float* dtheta, float* couplings) {
  int rc = check_traj(h, traj);
  if (rc) return rc;
  if (!theta) return fail(KURA_ERR_INVALID, "theta is NULL");
  if (!h->omega_set) return fail(KURA_ERR_INVALID, "frequencies not set");
  if (h->coupling == KURA_COUPLING_DENSE && !h->adj_set) return fail(KURA_ERR_INVALID, "adjacency not set");
  CU(cudaSetDevice(h->cfg.device));
  // the batch is evaluated at its current phases; this trajectory is first set to theta
  rc = kura_set_state(h, traj, theta, 0.0, 1.0);
  if (rc) return rc;
  if (h->te) {
    rc = h->te->evaluate(2, traj, dtheta, couplings);
    return rc ? fail(rc, kura::TensorEngine::last_error()) : KURA_OK;
  }
  rc = launch(h, kura::MODE_RHS, false);
  if (rc) return rc;
  if (dtheta) CU(cudaMemcpy(dtheta, h->fin_theta + (size_t)traj * h->ld, sizeof(float) * h->n, cudaMemcpyDeviceToHost));
  if (couplings)
    CU(cudaMemcpy(couplings, h->fin_coup + (size_t)traj * 2 * h->ld, sizeof(float) * 2 * h->n, cudaMemcpyDeviceToHost));
  return KURA_OK;
}

extern "C" int kura_set_launch_attempts(kura_handle* h, int64_t attempts) {
  if (!h) return fail(KURA_ERR_INVALID, "handle is NULL");
  if (h->te) return fail(KURA_ERR_UNSUPPORTED, "the tensor-core engine has no checkpoint launches");
  h->launch_attempts = attempts > 0 ? attempts : -1;
  return KURA_OK;
}

extern "C" int kura_get_stats(kura_handle* h, kura_stats* st) {
  if (!h || !st) return fail(KURA_ERR_INVALID, "NULL argument");
  *st = h->stats;
  return KURA_OK;
}

extern "C" int kura_volcano_factor(int32_t seed, int64_t n, int32_t k, int8_t* u) {
  if (n < 1 || k < 0 || !u) return fail(KURA_ERR_INVALID, "bad argument");
  if (k == 0) return KURA_OK;
  int words = (k + 31) / 32;
  uint32_t* d = nullptr;
  CU(cudaMalloc((void**)&d, sizeof(uint32_t) * (size_t)words * n));
  cudaError_t e = kura::launch_volcano_words(seed, (int)n, k, words, d, 0);
  std::vector<uint32_t> hb((size_t)words * n);
  if (e == cudaSuccess) e = cudaMemcpy(hb.data(), d, sizeof(uint32_t) * hb.size(), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(KURA_ERR_CUDA, cudaGetErrorString(e));
  for (int m = 0; m < k; ++m)
    for (int64_t i = 0; i < n; ++i) u[(size_t)m * n + i] = ((hb[(size_t)(m / 32) * n + i] >> (m % 32)) & 1u) ? 1 : -1;
  return KURA_OK;
}
