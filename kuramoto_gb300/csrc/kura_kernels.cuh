// kura_kernels.cuh -- device-side data structures shared by the kernels and the
// C ABI implementation of libkura.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace kura {

constexpr int KT = 512;       // threads per CTA of the persistent integrator
constexpr int KW = KT / 32;   // warps per CTA
constexpr int CT = 1024;      // columns per staged x tile of the dense coupling
constexpr int CT_I8 = 4096;   // the same for int8 rows and one trajectory (8 steps of 16 bytes per lane per tile)
constexpr int I8_SLOTS = 16;  // 16-byte chunk slots per lane in the int8 product's cp.async ring (8 rows x 2 steps)
constexpr int CT_F1 = 8192;   // the same for float rows and one trajectory
constexpr int A_ROWS = 4;     // rows per warp and pass of the dense float product
constexpr int A_STAGES = 3;   // 16-byte chunks per row and lane in flight (cp.async ring) in that product
constexpr int I8_CHUNK4 = 17; // x tile stride of the int8 product per 16 columns, in (cos, cos, sin, sin) float4
constexpr int I8_CHUNK = 18;  // the same for a batch, in (cos, sin) pairs
constexpr int F_CHUNK = 6;    // the same for the float product per 4 columns
constexpr int PW_MAX = 2 * 32 + 2;  // partial sums per trajectory and CTA: 2K projections + (sum cos, sum sin)

// Per-trajectory scalars.  Every CTA keeps an identical copy in shared memory
// and takes identical decisions from identical data; CTA 0 writes it back.
struct TrajG {
  double t, h, t_last, t1;
  long long accepted, rejected;
  int status;      // 0 running, 1 finished, < 0 a KURA_ERR_* code
  int eval_i;      // next output index into t_eval
  int eval_end;    // one past the last output owed by the last accepted step
  int rot_y;       // physical phase buffer holding y (the other holds ylast / y7)
  int rot_g;       // FSAL: 0 -> k1 in g slot 0 and k7 in slot 6; 1 -> swapped
  int need_k1;     // the first RHS of a run is still to be evaluated
  int need_init;   // fresh start: record r(theta0) (and theta0, couplings) first
  int out_count;   // output records written in this launch
  int log_count;   // accepted steps logged in this launch
  float c1;        // coupling constant
  int pad[2];
};

struct KParams {
  int n, ld, batch, k, coupling, dense_level, fixed, rows, seed, mode;
  const float* omega;  // [ld]
  const float* adj;    // [n][ld] dense coupling
  float* ph_hi;        // [2][B][ld] wrapped phase, high part
  float* ph_lo;        // [2][B][ld] low part
  long long* ph_w;     // [2][B][ld] 2*pi windings
  float* g;            // [7][B][ld] coupling part of the stage slopes k_j - omega
  float2* xbuf;        // [2][B][ld] (cos, sin) exchanged between CTAs
  float* part;         // [2][grid][B][PW_MAX] per-CTA partial sums
  unsigned* bar;       // grid barrier arrival counter (zeroed before each launch)
  int* err;            // launch-wide abort code
  TrajG* traj;         // [B]
  const float* t_eval; // output grid
  int n_eval;
  double atol, rtol, dt;
  float* out_r;        // [B][ring] order parameter records
  int* out_idx;        // [B][ring] output index (-1: the record at t0)
  float* out_theta;    // [B][ring][ld] unwrapped phases (dense_level >= 1)
  float* out_coup;     // [B][ring][2*ld] couplings (dense_level >= 2)
  int ring;
  double* log_t;       // [B][log_cap] accepted step times
  double* log_h;       // [B][log_cap] step size after each accepted step
  int log_cap;
  long long max_attempts;       // per launch, < 0: unlimited
  unsigned long long timeout_ns;
  int xs_smem;         // 1: the CTA's (cos, sin) live in shared memory (volcano coupling)
  unsigned bar_extra;  // arrivals a barrier waits for beyond the grid (tests of the time limit)
  float* fin_theta;    // [B][ld] end-of-run phases / RHS output
  float* fin_coup;     // [B][2*ld]
  long long* counters; // [0] barriers executed (CTA 0 adds)
  const int8_t* adj8;  // [n][ld8] N*A as int8 (dense coupling stored as integers), or null
  int ld8;             // row stride of adj8 (a multiple of 16)
  float invn;          // 1/N in float, the scale of adj8
};

// kernel selector for a dense adjacency stored as the integers N*A (int8); the public
// coupling stays KURA_COUPLING_DENSE
constexpr int COUP_DENSE_I8 = 2;

enum Mode { MODE_INTEGRATE = 0, MODE_FINAL = 1, MODE_RHS = 2 };

// The persistent kernel instantiations; bmax/kmax select the template.
cudaError_t persistent_config(int coupling, int bmax, int kmax, size_t* smem_bytes, int* blocks_per_sm,
                              int rows_per_cta, int* xs_smem);
cudaError_t launch_persistent(const KParams& p, int grid, int bmax, int kmax, size_t smem, cudaStream_t st);
cudaError_t launch_init_state(const float* theta, int n, int ld, float* hi, float* lo, long long* w,
                              cudaStream_t st);
cudaError_t launch_volcano_words(int seed, int n, int k, int words, uint32_t* bits, cudaStream_t st);
cudaError_t launch_volcano_adjacency_i8(const uint32_t* bits, int n, int k, int words, int ld8, int8_t* adj8,
                                        cudaStream_t st);
cudaError_t launch_volcano_adjacency(const uint32_t* bits, int n, int k, int words, int ld, float* adj,
                                     cudaStream_t st);
// sets the message returned by kura_last_error() for the calling thread
void set_last_error(const char* msg);
cudaError_t launch_unwrap(const float* hi, const float* lo, const long long* w, int n, float* out,
                          cudaStream_t st);

}  // namespace kura
