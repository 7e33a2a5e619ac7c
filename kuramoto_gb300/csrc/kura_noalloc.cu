// kura_noalloc.cu -- an integration entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code running inside a framework that owns
// the device allocator (a memory pool that must see every allocation, so a private
// cudaMalloc would fragment or overrun its budget), or a host process that runs
// under a fixed device-memory budget set before it starts.
// kura_integrate_volcano_noalloc serves them.  The caller
// passes device buffers for its inputs and outputs; all scratch the persistent
// kernel needs (phases, slopes, partial sums, the barrier counter, trajectory
// state) lives in one file-scope __device__ array, g_noalloc_scratch, of TOTAL
// bytes (about 6.7 MiB).  Every GPU that loads libkura holds that array until the
// process exits.
//
// Limits (checked; larger requests return KURA_ERR_INVALID with a message):
//   round_up(n, 32) * batch <= MAX_SLOTS (65536), batch <= 8, k <= 32,
//   order_cap <= MAX_RECORDS (4096), int(t1/dt)+1 <= order_cap.
//
// The array is shared by every call on a device and keeps the last call's
// contents; each call clears what must start at zero.  Calls whose work overlaps
// on the GPU (concurrent streams, or host threads calling at once) race on the
// array and corrupt each other's results: serialize them.  The first call on a
// device looks up the array's device address (cudaGetSymbolAddress) with that
// device current; make that first call before any stream capture.  The call makes
// `device` current while it works and restores the caller's current device on
// every return.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include "kura.h"
#include "kura_kernels.cuh"

namespace {

using kura::TrajG;

constexpr long long MAX_SLOTS = 65536;  // padded oscillators times trajectories
constexpr int MAX_RECORDS = 4096;       // order-parameter records per trajectory
constexpr int MAX_GRID = 256;           // CTAs of the persistent kernel
constexpr int MAX_BATCH = 8;

constexpr size_t al(size_t b) { return (b + 255) & ~(size_t)255; }
// byte offsets of the scratch regions
constexpr size_t O_HI = 0;
constexpr size_t O_LO = O_HI + al(2 * MAX_SLOTS * 4);
constexpr size_t O_W = O_LO + al(2 * MAX_SLOTS * 4);
constexpr size_t O_G = O_W + al(2 * MAX_SLOTS * 8);
constexpr size_t O_X = O_G + al(7 * MAX_SLOTS * 4);
constexpr size_t O_PART = O_X + al(2 * MAX_SLOTS * 8);
constexpr size_t O_BAR = O_PART + al((size_t)2 * MAX_GRID * MAX_BATCH * kura::PW_MAX * 4);
constexpr size_t O_ERR = O_BAR + al(4);
constexpr size_t O_CNT = O_ERR + al(4);
constexpr size_t O_TRAJ = O_CNT + al(16);
constexpr size_t O_TEVAL = O_TRAJ + al(MAX_BATCH * sizeof(TrajG));
constexpr size_t O_IDX = O_TEVAL + al(MAX_RECORDS * 4);
constexpr size_t O_FIN = O_IDX + al((size_t)MAX_BATCH * MAX_RECORDS * 4);
constexpr size_t O_FINC = O_FIN + al(MAX_SLOTS * 4);
constexpr size_t TOTAL = O_FINC + al(2 * MAX_SLOTS * 4);

__device__ __align__(256) unsigned char g_noalloc_scratch[TOTAL];

std::mutex g_mu;
void* g_addr[256];  // device address of g_noalloc_scratch per device ordinal

// restores the caller's current device when the entry point returns
struct DeviceRestore {
  int dev = -1;
  DeviceRestore() {
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
  }
  ~DeviceRestore() {
    if (dev >= 0) cudaSetDevice(dev);
  }
};

int fail(int code, const std::string& m) {
  kura::set_last_error(m.c_str());  // read back with kura_last_error()
  return code;
}

struct TrajInit {
  float c[MAX_BATCH];
  double h0, t1;
  int batch;
};

// trajectory state of a fresh start at t = 0 (the reference's !reloaded path)
__global__ void k_noalloc_setup(TrajG* traj, TrajInit in, float* t_eval, int n0, int n_eval, float dtf) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < in.batch) {
    TrajG T = {};
    T.t = 0.0;
    T.h = in.h0;
    T.t_last = 0.0;
    T.t1 = in.t1;
    T.status = 0;
    T.need_k1 = 1;
    T.need_init = 1;
    T.c1 = in.c[t];
    traj[t] = T;
  }
  for (int i = t; i < n_eval; i += gridDim.x * blockDim.x) t_eval[i] = dtf * (float)(n0 + i);
}

}  // namespace

extern "C" int kura_integrate_volcano_noalloc(int64_t n, int32_t k, int32_t batch, int32_t seed, const float* c,
                                              const float* omega_dev, float* theta_dev, double t1, double dt,
                                              double h0, double atol, double rtol, int32_t device, void* stream,
                                              float* order_dev, int64_t order_cap, int64_t* accepted) {
  if (n < 1 || k < 0 || k > 32 || batch < 1 || batch > MAX_BATCH)
    return fail(KURA_ERR_INVALID, "need n >= 1, 0 <= k <= 32, 1 <= batch <= 8");
  if (!c || !omega_dev || !theta_dev || !order_dev) return fail(KURA_ERR_INVALID, "NULL argument");
  const long long ld = (n + 31) / 32 * 32;
  if (ld * batch > MAX_SLOTS)
    return fail(KURA_ERR_INVALID, "round_up(n,32)*batch exceeds the scratch limit of 65536");
  // every double must be finite (a NaN passes any ordered comparison's negation)
  if (!std::isfinite(t1) || !std::isfinite(dt) || !std::isfinite(h0) || !std::isfinite(atol) ||
      !std::isfinite(rtol))
    return fail(KURA_ERR_INVALID, "t1, dt, h0, atol and rtol must be finite");
  if (!(dt > 0) || !(h0 > 0) || !(atol > 0) || !(rtol >= 0) || !(t1 >= 0))
    return fail(KURA_ERR_INVALID, "need dt, h0, atol > 0 and t1, rtol >= 0");
  if (order_cap < 1 || order_cap > MAX_RECORDS) return fail(KURA_ERR_INVALID, "order_cap must be in [1, 4096]");
  // output grid t_eval = dt*n, n = 1 .. int(t1/dt) in float, as a fresh start of the reference;
  // the record count is bounded in floating point before any conversion to int
  const float dtf = (float)dt, t1f = (float)t1;
  if (!(dtf > 0) || !std::isfinite(t1f) || !std::isfinite(t1f / dtf))
    return fail(KURA_ERR_INVALID, "t1 and dt must be representable in float with dt > 0");
  if (!((double)(t1f / dtf) < (double)order_cap))  // int(t1/dt) + 1 <= order_cap
    return fail(KURA_ERR_INVALID, "order_cap smaller than the int(t1/dt)+1 records");
  const int n0 = 1, n1 = int(t1f / dtf) + 1;
  const int n_eval = n1 > n0 ? n1 - n0 : 0;
  if (n_eval + 1 > order_cap) return fail(KURA_ERR_INVALID, "order_cap smaller than the int(t1/dt)+1 records");

  cudaError_t e;
  if (device < 0 || device >= 256) return fail(KURA_ERR_INVALID, "device index out of range");
  DeviceRestore restore;
  if ((e = cudaSetDevice(device)) != cudaSuccess) return fail(KURA_ERR_CUDA, cudaGetErrorString(e));
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[device]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return fail(KURA_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_addr[device] = p;
    }
    base = (unsigned char*)g_addr[device];
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int B = batch, N = (int)n, LD = (int)ld;
  const int bmax = B <= 1 ? 1 : 8, kmax = k <= 8 ? 8 : 32;

  int sms = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
    return fail(KURA_ERR_CUDA, cudaGetErrorString(e));
  int G = std::min(std::min(sms, MAX_GRID), std::max(1, (N + 63) / 64));
  int rows = (N + G - 1) / G;
  G = (N + rows - 1) / rows;
  size_t smem = 0;
  int bps = 0, xs = 0;
  if ((e = kura::persistent_config(KURA_COUPLING_VOLCANO, bmax, kmax, &smem, &bps, rows, &xs)) != cudaSuccess)
    return fail(KURA_ERR_CUDA, cudaGetErrorString(e));
  if (bps < 1) return fail(KURA_ERR_UNSUPPORTED, "persistent kernel does not fit on an SM");

  kura::KParams p;
  std::memset(&p, 0, sizeof(p));
  p.n = N; p.ld = LD; p.batch = B; p.k = k; p.coupling = KURA_COUPLING_VOLCANO; p.dense_level = 0;
  p.fixed = 0; p.rows = rows; p.seed = seed; p.mode = kura::MODE_INTEGRATE;
  p.omega = omega_dev; p.adj = nullptr;
  p.ph_hi = (float*)(base + O_HI); p.ph_lo = (float*)(base + O_LO); p.ph_w = (long long*)(base + O_W);
  p.g = (float*)(base + O_G); p.xbuf = (float2*)(base + O_X); p.part = (float*)(base + O_PART);
  p.bar = (unsigned*)(base + O_BAR); p.err = (int*)(base + O_ERR); p.traj = (TrajG*)(base + O_TRAJ);
  p.t_eval = (const float*)(base + O_TEVAL); p.n_eval = n_eval;
  p.atol = atol; p.rtol = rtol; p.dt = dt;
  p.out_r = order_dev; p.out_idx = (int*)(base + O_IDX); p.out_theta = nullptr; p.out_coup = nullptr;
  p.ring = (int)order_cap;
  p.log_t = nullptr; p.log_h = nullptr; p.log_cap = 0;
  p.max_attempts = -1;
  p.timeout_ns = 20000ull * 1000000ull;
  p.xs_smem = xs;
  p.bar_extra = 0;
  p.fin_theta = (float*)(base + O_FIN); p.fin_coup = (float*)(base + O_FINC);
  p.counters = (long long*)(base + O_CNT);

  // clear what must start at zero, then the trajectories and the phases
  if ((e = cudaMemsetAsync(base + O_BAR, 0, O_TRAJ - O_BAR, st)) != cudaSuccess)
    return fail(KURA_ERR_CUDA, cudaGetErrorString(e));
  TrajInit in;
  std::memset(&in, 0, sizeof(in));
  for (int b = 0; b < B; ++b) in.c[b] = c[b];
  in.h0 = h0;
  in.t1 = t1;
  in.batch = B;
  k_noalloc_setup<<<(std::max(n_eval, B) + 255) / 256, 256, 0, st>>>(p.traj, in, (float*)p.t_eval, n0, n_eval, dtf);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(KURA_ERR_CUDA, cudaGetErrorString(e));
  for (int b = 0; b < B; ++b) {
    size_t off = (size_t)b * LD;  // phase buffer 0
    if ((e = kura::launch_init_state(theta_dev + (size_t)b * N, N, LD, p.ph_hi + off, p.ph_lo + off, p.ph_w + off,
                                     st)) != cudaSuccess)
      return fail(KURA_ERR_CUDA, cudaGetErrorString(e));
  }
  if ((e = kura::launch_persistent(p, G, bmax, kmax, smem, st)) != cudaSuccess)
    return fail(KURA_ERR_CUDA, cudaGetErrorString(e));
  int err = 0;
  TrajG tr[MAX_BATCH];
  if ((e = cudaMemcpyAsync(&err, p.err, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(tr, p.traj, sizeof(TrajG) * B, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return fail(KURA_ERR_CUDA, cudaGetErrorString(e));
  if (err) return fail(err, "persistent kernel aborted (grid barrier time limit)");
  long long acc = 0;
  for (int b = 0; b < B; ++b) {
    if (tr[b].status < 0) return fail(tr[b].status, "integration failed (step underflow or non-finite norm)");
    acc += tr[b].accepted;
  }
  // final phases, unwrapped, back into the caller's buffer
  for (int b = 0; b < B; ++b) {
    size_t off = ((size_t)tr[b].rot_y * B + b) * LD;
    if ((e = kura::launch_unwrap(p.ph_hi + off, p.ph_lo + off, p.ph_w + off, N, theta_dev + (size_t)b * N, st)) !=
        cudaSuccess)
      return fail(KURA_ERR_CUDA, cudaGetErrorString(e));
  }
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(KURA_ERR_CUDA, cudaGetErrorString(e));
  if (accepted) *accepted = acc;
  return KURA_OK;
}
