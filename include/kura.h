/* kura.h -- C ABI of the GB300 Kuramoto DP45 integrator (libkura.so).
 *
 * The reference program (znicolaou/kuramoto) has no library interface: its
 * integrator is the static-state C ABI of dp45.h, driven by host callbacks
 * (dydt once per stage, step_eval once per accepted step), and its user-facing
 * surface is the `kuramoto` command line plus the FILEBASE files.  This header
 * replaces that internal ABI with explicit handles.  Each entry point names the
 * reference code it stands in for.
 *
 * Conventions: every call returns KURA_OK (0) or a negative KURA_ERR_* code;
 * kura_last_error() gives a message for the calling thread.  All pointers are
 * host pointers unless the name ends in _device.  Calls on one handle are not
 * thread-safe.  Oscillator arrays are float32; adjacency rows are contiguous
 * (row i at adj + i*n), which is the buffer the reference hands to cuBLAS
 * (column-major with OP_T, kuramoto.cu:113-114).
 */
#ifndef KURA_H
#define KURA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KURA_OK 0
#define KURA_ERR_INVALID (-1)         /* bad argument or call order */
#define KURA_ERR_CUDA (-2)            /* CUDA runtime error */
#define KURA_ERR_NOMEM (-3)           /* device allocation failed */
#define KURA_ERR_BARRIER_TIMEOUT (-4) /* a grid barrier of the persistent kernel gave up */
#define KURA_ERR_STEP_UNDERFLOW (-5)  /* step size fell below 1e-14 * max(1,|t|) */
#define KURA_ERR_NONFINITE (-6)       /* error norm became NaN or infinite */
#define KURA_ERR_UNSUPPORTED (-7)     /* configuration outside the built kernels */
#define KURA_ERR_CALLBACK (-8)        /* an observer callback returned non-zero */

#define KURA_COUPLING_DENSE 0   /* adjacency stored in HBM (reference default) */
#define KURA_COUPLING_VOLCANO 1 /* rank-K volcano factor regenerated from Philox (reference -A) */

/* KURA_ENGINE_AUTO picks the tensor-core ensemble for a dense network with batch > 8, or with
 * batch >= 2 at dense level 0, and the CUDA-core persistent kernel otherwise.  The persistent kernel takes batch <= 8 (dense
 * or volcano coupling, every dense level); the tensor-core ensemble takes a dense network
 * with batch <= 128, keeps only the order parameter (dense level 0) and reports no per-step
 * records.  The reference has neither: it integrates one trajectory per process. */
/* Storage of a dense adjacency on the persistent engine.  KURA_ADJ_I8 keeps N*A as int8,
 * a quarter of the bytes the coupling streams per RHS; it holds the reference's volcano rule
 * exactly (N*A_ij is an integer in [-K, K], K <= 127) and any adjacency whose entries are
 * integer multiples of 1/N within that range.  The reference stores float32. */
#define KURA_ADJ_F32 0
#define KURA_ADJ_I8 1

#define KURA_ENGINE_AUTO 0
#define KURA_ENGINE_PERSISTENT 1
#define KURA_ENGINE_TENSOR 2

typedef struct kura_handle kura_handle;

/* Network and integrator settings; the reference flag each field replaces is given. */
typedef struct kura_config {
  int64_t n;           /* -N oscillators */
  int32_t k;           /* -K volcano rank */
  int32_t coupling;    /* KURA_COUPLING_DENSE or KURA_COUPLING_VOLCANO (-A) */
  int32_t batch;       /* trajectories sharing omega and the adjacency (1 = the reference) */
  int32_t seed;        /* -s Philox seed of the volcano factor */
  double atol;         /* -a */
  double rtol;         /* -r */
  int32_t fixed_step;  /* -F */
  int32_t device;      /* -g */
  int32_t dense_level; /* -D: 0 order only; >=1 adds phases and step times; >=2 adds couplings */
  int32_t engine;      /* KURA_ENGINE_*: which kernels integrate the batch */
  void* stream;        /* cudaStream_t for every launch and copy (NULL: a stream owned by the handle) */
  int32_t adj_storage; /* KURA_ADJ_F32 (default) or KURA_ADJ_I8, dense coupling on the persistent engine */
} kura_config;

typedef struct kura_stats {
  int64_t accepted;    /* accepted steps, summed over trajectories */
  int64_t rejected;    /* rejected attempts, summed over trajectories */
  int64_t launches;    /* persistent-kernel launches */
  int64_t barriers;    /* grid barriers executed (all launches) */
  double kernel_ms;    /* device time of the persistent launches (CUDA events) */
  int32_t grid;        /* CTAs of the persistent kernel */
  int32_t block;       /* threads per CTA */
  double coupling_ms;  /* device time of the timed coupling-GEMM launches (tensor engine, environment
                          KURA_TIME_COUPLING=1: the six GEMMs of one attempt in every four, CUDA events) */
  int64_t coupling_launches; /* launches that coupling_ms covers */
} kura_stats;

/* Per-record observer callbacks, called from kura_run on the calling thread, in
 * order, after each persistent launch is drained.  Return non-zero to abort.
 * on_step mirrors step_eval's per-step work (kuramoto.cu:169-188); on_output the
 * per-t_eval work (kuramoto.cu:212-234); theta / couplings are NULL when the
 * dense level does not ask for them.  on_chunk is called after each launch with
 * the current phases (for checkpoint files such as fs.dat). */
typedef struct kura_callbacks {
  void* user;
  int (*on_step)(void* user, int32_t traj, double t, double h, int64_t step);
  int (*on_output)(void* user, int32_t traj, int64_t index, double t_eval, float r, const float* theta,
                   const float* couplings);
  int (*on_chunk)(void* user, int32_t traj, double t, double h, const float* theta);
} kura_callbacks;

/* replaces dp45_init (dp45.h:8) and the allocations of main (kuramoto.cu:442-457) */
int kura_create(const kura_config* cfg, kura_handle** out);
/* replaces dp45_destroy (dp45.h:10) and main's frees (kuramoto.cu:659-675) */
void kura_destroy(kura_handle* h);
const char* kura_last_error(void);
/* device memory the handle holds, in bytes (the reference prints its estimate, kuramoto.cu:424-433) */
int kura_memory_required(const kura_config* cfg, int64_t* bytes);

/* omega upload (kuramoto.cu:552) */
int kura_set_frequencies(kura_handle* h, const float* omega, int64_t n);
/* adjacency from a file (-R, kuramoto.cu:559-566); row-major n x n */
int kura_set_adjacency(kura_handle* h, const float* adj, int64_t n);
/* volcano adjacency A = (1/N) sum_m (-1)^m u_m u_m^T (getadj, kuramoto.cu:128-161) */
int kura_generate_adjacency(kura_handle* h);
/* adjacency download for adj.dat (kuramoto.cu:573-578) */
int kura_get_adjacency(kura_handle* h, float* adj, int64_t n);
/* coupling constant of one trajectory (-c, tot_kuramoto's c1, kuramoto.cu:42-47) */
int kura_set_coupling(kura_handle* h, int32_t traj, float c);
/* phases, time and step of one trajectory (random start or -R reload, kuramoto.cu:459-506) */
int kura_set_state(kura_handle* h, int32_t traj, const float* theta, double t, double step);
int kura_set_state_device(kura_handle* h, int32_t traj, const float* theta_device, double t, double step);
/* output grid t_eval = dt*n, n = int(t0/dt)+1 .. int(t1/dt), and the end time
 * (kuramoto.cu:543-550); initial_record = 1 writes r(theta0) (and theta0,
 * couplings) first, as a fresh start does (kuramoto.cu:587-626).  After a kura_run that
 * brought every trajectory to its end time, a new horizon continues the integration from
 * where each trajectory stopped (phases, FSAL slope and step size kept on the device): the
 * reference's -R resume (kuramoto.cu:466-494, 543) without the round trip through fs.dat.
 * Trajectories of a batch may start (or continue) at different times: the grid then starts
 * after the earliest one's time, and each trajectory records only the output times after
 * its own. */
int kura_set_horizon(kura_handle* h, double t1, double dt, int32_t initial_record);

/* integrate every trajectory to t1 (dp45_run with step_eval, dp45.cu:148-164) */
int kura_run(kura_handle* h, const kura_callbacks* cb);
/* integrate for at most `attempts` step attempts of every unfinished trajectory (the tensor
 * engine takes them in groups of four), then return with the state kept on the device;
 * *running (may be NULL) receives the trajectories still short of t1.  A later kura_advance or
 * kura_run continues exactly where this one stopped.  The reference's counterpart is a run cut
 * short by its job's time limit and resumed with -R (job1.sh:3 ckpt partition; kuramoto.cu:466-494),
 * here without losing the FSAL slope or the step size.  Records reach the observers as in
 * kura_run. */
int kura_advance(kura_handle* h, const kura_callbacks* cb, int64_t attempts, int32_t* running);

/* current phases (unwrapped), time and step of one trajectory */
int kura_get_state(kura_handle* h, int32_t traj, float* theta, double* t, double* step);
/* order parameter records of one trajectory since kura_set_horizon (order.dat) */
int kura_get_order(kura_handle* h, int32_t traj, float* r, int64_t cap, int64_t* count);
/* end-of-run record of fs.dat: phases at the last output time, evaluated after the
 * FSAL copy as the reference does (kuramoto.cu:630-647), and the couplings there */
int kura_final_record(kura_handle* h, int32_t traj, float* theta, float* couplings, double* t, double* step);
/* right-hand side dtheta/dt and couplings [A cos, A sin] interleaved at theta (dydt, kuramoto.cu:118-126) */
int kura_rhs(kura_handle* h, int32_t traj, const float* theta, float* dtheta, float* couplings);
int kura_get_stats(kura_handle* h, kura_stats* st);
/* checkpoint grain: at most `attempts` step attempts per persistent launch (<= 0: unbounded,
 * the default), so that on_chunk sees the phases, t and h at least that often.  The
 * reference rewrites fs.dat after every accepted step for preemption (kuramoto.cu:251-264);
 * this is the same checkpoint at a coarser, chosen grain.  Persistent engine only. */
int kura_set_launch_attempts(kura_handle* h, int64_t attempts);

/* host random inputs with glibc rand(): theta0 uniform in [-init/2, init/2] then
 * Cauchy or normal frequencies (kuramoto.cu:416, 495-541) */
int kura_random_inputs(int32_t seed, int64_t n, float init, float freq, int32_t normal, int32_t gen_theta,
                       int32_t gen_omega, float* theta0, float* omega);
/* Philox4x32-10 volcano factor bits as +/-1 int8 at m*n+i (kuramoto.cu:62-101, 128-135), on the device */
int kura_volcano_factor(int32_t seed, int64_t n, int32_t k, int8_t* u);

/* Integrates `batch` trajectories of one volcano network with the factor
 * regenerated from Philox (the reference's -A mode) from t = 0 to t1, without
 * allocating any device memory.  No counterpart in the reference.  For callers
 * that cannot call cudaMalloc: a framework that owns the device allocator (its pool
 * must account for every byte), or a process held to a fixed device-memory budget.
 * Inputs and outputs are the caller's device buffers: omega_dev[n];
 * theta_dev[batch][n] holds theta0 on entry and the final phases on success;
 * order_dev[batch][order_cap] receives r(0) and r at t = dt, 2dt, .., int(t1/dt)*dt.
 * c[batch] (coupling constants) is a host array; accepted (optional, host) gets the
 * accepted steps summed over the batch.  t1, dt, h0, atol and rtol must be finite.
 * Scratch is one static __device__ array of about 6.7 MiB held by every GPU that
 * loads the library; it limits round_up(n,32)*batch <= 65536, batch <= 8, k <= 32 and
 * order_cap <= 4096, and larger requests return KURA_ERR_INVALID.  All calls share that
 * array: calls that overlap on the GPU race.  The first call on a device looks up the
 * array's address; make it before any stream capture.  The call waits for its work on
 * `stream` before it returns (NULL: the legacy default stream) and leaves the caller's
 * current device as it found it.  On an error return theta_dev still holds theta0,
 * order_dev holds whatever records were written before the failure (not meaningful),
 * and *accepted is not written. */
int kura_integrate_volcano_noalloc(int64_t n, int32_t k, int32_t batch, int32_t seed, const float* c,
                                   const float* omega_dev, float* theta_dev, double t1, double dt, double h0,
                                   double atol, double rtol, int32_t device, void* stream, float* order_dev,
                                   int64_t order_cap, int64_t* accepted);

/* ---- many independent networks of uneven size in one persistent launch
 *
 * The reference integrates one network per `kuramoto -A` process (kuramoto.cu:380-640,
 * regenerated volcano coupling kuramoto.cu:62-135, integrator dp45.cu:148-164).  A
 * kura_multi handle holds a set of such networks, each with its own N, rank K, Philox seed
 * and coupling constant, all integrated from t = 0 to the same t1 with the same atol/rtol
 * and output interval dt, each with its own adaptive step, by one launch in which a
 * thread-block cluster integrates one network at a time from a work queue. */
typedef struct kura_instance {
  int64_t n;    /* oscillators, 1 .. 16 x 22755 */
  int32_t k;    /* volcano rank 0..8 (-K) */
  int32_t seed; /* Philox seed of the factor (-s) */
  float c;      /* coupling constant (-c) */
  int32_t reserved;
} kura_instance;

typedef struct kura_multi_stats {
  double kernel_ms;     /* device time of the last integration launch */
  double osc_steps;     /* sum over networks of accepted steps x n */
  double tune_ms;       /* device time of the autotuner's chosen trial */
  int64_t accepted;     /* accepted steps, all networks */
  int64_t rejected;     /* rejected attempts, all networks */
  int32_t cluster_size; /* CTAs per network */
  int32_t block_threads;
  int32_t grid;  /* CTAs of the main launch */
  int32_t heavy; /* networks run in large clusters beside the main launch */
} kura_multi_stats;

typedef struct kura_multi kura_multi;

/* Allocates the device state of `count` networks (about 72 bytes per oscillator plus
 * 4 bytes per record).  Records: r at t = 0 and at dt*m, m = 1 .. int(t1/dt) in float,
 * as the reference's order.dat (kuramoto.cu:543-626).  h0 is the first trial step of every
 * network.  cluster_size (1, 2, 4, 8, 16) and block_threads (256, 512, 1024) fix the launch
 * shape; 0 lets the autotuner choose it at the first integration, as the shape with the
 * shortest predicted time for the whole integration (environment KURA_MULTI_TUNE_LOG=1
 * prints its trials).  Later integrations on the handle keep the shape and give bitwise
 * identical results for the same inputs. */
int kura_multi_create(const kura_instance* inst, int32_t count, double t1, double dt, double h0, double atol,
                      double rtol, int32_t device, int32_t cluster_size, int32_t block_threads, kura_multi** out);
void kura_multi_destroy(kura_multi* m);
/* Integrates every network from the given start.  omega and theta0 hold the networks'
 * oscillators back to back in the order of creation (host pointers, sum of n floats each).
 * order receives count x (int(t1/dt) + 1) floats, network by network; theta_final (may be
 * NULL) the unwrapped phases at each network's final time (the first step end >= t1);
 * accepted (may be NULL) the accepted steps per network.  Synchronous.  A network whose
 * step underflows or whose error norm is NaN fails the call with that code. */
int kura_multi_integrate(kura_multi* m, const float* omega, const float* theta0, float* order, float* theta_final,
                         int64_t* accepted);
int kura_multi_get_stats(const kura_multi* m, kura_multi_stats* stats);

/* ---- the order-parameter surrogate (a learned model; the reference has no counterpart)
 *
 * A 4-layer perceptron in_dim -> hidden -> hidden -> hidden -> out_dim with SiLU between
 * layers, BF16 weights and activations, FP32 accumulation, FP32 master weights and biases.
 * Its forward and backward GEMMs run on the tensor cores; training is Adam with a linear
 * learning-rate ramp, on minibatches of `batch` rows, one CUDA graph per step.  Loss: mean
 * squared error over the out_dim outputs. */
typedef struct kura_mlp kura_mlp;

/* in_dim, out_dim 1..64; hidden 64, 128 or 256; batch a multiple of 128 up to 4096.  Weights
 * are Glorot-uniform from a splitmix64 stream of `seed`, biases zero. */
int kura_mlp_create(int32_t in_dim, int32_t hidden, int32_t out_dim, int32_t batch, uint64_t seed, int32_t device,
                    kura_mlp** out);
void kura_mlp_destroy(kura_mlp* m);
/* Parameters in this order, layer by layer: W [out][in] row-major, then b [out]. */
int kura_mlp_param_count(const kura_mlp* m, int64_t* count);
int kura_mlp_get_params(kura_mlp* m, float* params, int64_t count);
int kura_mlp_set_params(kura_mlp* m, const float* params, int64_t count);
/* y[n][out_dim] = f(x[n][in_dim]), host arrays, any n. */
int kura_mlp_forward(kura_mlp* m, const float* x, int64_t n, float* y);
/* Loss and its gradient (parameter order above) on one minibatch of n <= batch rows. */
int kura_mlp_gradients(kura_mlp* m, const float* x, const float* target, int64_t n, float* grads, float* loss);
/* Trains on n_samples rows (at least one batch): `epochs` passes, each a fresh shuffle from
 * `shuffle_seed` that drops the last partial batch; Adam (0.9, 0.999, 1e-8) restarted at the
 * call, learning rate from lr to lr_final.  epoch_loss[epochs] (may be NULL) receives the mean
 * minibatch loss of each epoch, device_ms (may be NULL) the device time of the steps. */
int kura_mlp_train(kura_mlp* m, const float* x, const float* target, int64_t n_samples, int32_t epochs, float lr,
                   float lr_final, uint64_t shuffle_seed, float* epoch_loss, double* device_ms);

#ifdef __cplusplus
}
#endif
#endif
