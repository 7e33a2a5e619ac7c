// kura_multi.cu -- many independent volcano networks of uneven size in one persistent launch.
//
// Each network (its own N, rank K <= 8, coupling c, Philox seed, frequencies and initial
// phases) is integrated from t = 0 to t1 with its own adaptive DP45 step (dp45_run,
// dp45.cu:148-164; the reference runs one `kuramoto -A` process per network) by one
// thread-block cluster.  Clusters pull networks from a work queue (largest first in the
// pilot launch, then by predicted remaining work), so nothing synchronises the grid: a network's reductions (the K-mode projections of the
// regenerated volcano coupling, kuramoto.cu:62-101, the error norm, dp45.cu:116-119, and
// the order parameter, kuramoto.cu:587-600) go through distributed shared memory between
// the CTAs of its cluster, with hardware cluster barriers.  The factor bits of a CTA's rows
// are regenerated from the network's Philox stream into shared memory when the cluster
// takes the network, so neither A nor the factor is stored.
//
// Per network the state lives in HBM and stays in L2 while the network is in flight:
// phases as a wrapped float pair plus an int64 winding count (two buffers, y and y7) and
// the seven slopes minus omega.  The controller runs on thread 0 of every CTA of the
// cluster on bitwise identical sums, so all CTAs take the same decisions without
// exchanging them, and every cluster barrier is reached by all of them.
//
// The launch shape (cluster size, block size) comes from an autotuner that runs a
// stratified sample of the networks at every candidate shape and predicts the time of the
// whole integration from it.  An integration is a pilot launch (a CUDA graph replayed every
// time) followed by the rest of the work in the order of predicted cost, the heaviest
// networks in large clusters beside the others.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "kura.h"
#include "kura_device.cuh"
#include "kura_kernels.cuh"

namespace cg = cooperative_groups;

namespace kura {
namespace {

constexpr int M_KMAX = 8;             // volcano rank of the multi-network kernel
constexpr int M_NV = 2 * M_KMAX + 2;  // reduction slots: 16 projections, sum cos, sum sin
constexpr int M_RX = 2 * M_KMAX;      // slot of sum cos (sum sin follows)
constexpr int M_ROW_BYTES = 9;        // shared memory per row: (cos, sin) + factor bits
constexpr int M_SMEM_CAP = 200 * 1024;
constexpr int M_MAX_CLUSTER = 16;
constexpr int MU = 2;  // rows per thread whose loads are issued together in the row loop

struct MInst {
  int n, k, seed, id;  // id: index of the network in the caller's order
  float c, pad;
  long long off;    // first oscillator of the network in the packed arrays
  long long order;  // first record of the network in the order output
};

struct MParams {
  const MInst* inst;
  int count;
  int rows_max;  // rows per CTA the dynamic shared memory is sized for
  int* queue;
  const float* omega;
  const float* theta0;
  float* ph_hi;  // [2][total]: y and y7
  float* ph_lo;
  long long* ph_w;
  float* g;  // [7][total]: slopes minus omega
  long long total;
  double t1, h0, atol, rtol;
  int n_eval;  // records at dtf*1 .. dtf*n_eval after the one at t = 0
  float dtf;
  float* out_r;         // (n_eval + 1) per network, at MInst::order
  float* theta_out;     // total (final unwrapped phases), may be null
  long long* accepted;  // by MInst::id
  long long* rejected;
  int* status;             // by MInst::id: 1 done, < 0 a KURA_ERR_* code
  long long max_attempts;  // per network and launch, < 0: unbounded
  struct MNet* state;      // by MInst::id: the controller state between launches
};

// A network's controller between launches: a launch that stops a network after
// max_attempts leaves it here, and the next launch resumes it (the phases and slopes stay
// in HBM).  stage: 0 not started, 1 resumable, 2 finished.
struct MNet {
  double t, h, t_last;
  long long acc, rej;
  int rot_y, rot_g, eval_i, eval_end, status, stage;
  unsigned long long ns;  // time the network has spent in its clusters (the autotuner reads it)
};

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

struct MSmem {
  float red[32][M_NV];
  float part[2][M_MAX_CLUSTER][M_NV];  // every CTA's totals by reduction parity and rank
  float rsum[M_NV];
  float f3[2 * M_KMAX];  // (-1)^m / N times the projection totals
  float2 tab[256];  // sum_m +-f3_m for every sign pattern of the K factor bits
  float E[8];           // error weights of the attempt
  float Wst[7][8];      // rows 0..5: weights h a_sj of stages 2..7; row 6: dense output
  float mhs[7], mls[7];  // the time offset of each row as a float pair
  int idx;
  double t, h, t_last;
  long long acc, rej;
  int rot_y, rot_g, eval_i, eval_end, status;
  unsigned long long t_start;  // when the cluster took the network (rank 0)
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// 16 values per lane -> v[0] of lane L holds the warp total of value L >> 1 (recursive halving)
__device__ __forceinline__ void reduce_scatter16(float (&v)[16], int lane) {
#pragma unroll
  for (int half = 8, bit = 16; half >= 1; half >>= 1, bit >>= 1) {
    const bool upper = lane & bit;
#pragma unroll
    for (int j = 0; j < half; ++j) {
      const float send = upper ? v[j] : v[j + half];
      const float keep = upper ? v[j + half] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, bit);
    }
  }
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
}

// slot of slope j (0-based) when k1 of the attempt sits in slot g1 (0 or 6) and k7 in 6 - g1
__device__ __forceinline__ int slot_of(int j, int g1) { return j == 0 ? g1 : (j == 6 ? 6 - g1 : j); }

template <int NT>
struct Multi {
  static constexpr int NW = NT / 32;
  const MParams& p;
  MSmem& S;
  float2* xs;
  uint8_t* ubits;
  cg::cluster_group cl;
  int CS, rank, tid, lane, warp;
  int n, k, r0, r1;
  long long off;
  float c1;
  int par;

  __device__ Multi(const MParams& pp, MSmem& s, unsigned char* dyn)
      : p(pp), S(s), cl(cg::this_cluster()) {
    xs = reinterpret_cast<float2*>(dyn);
    ubits = dyn + 8 * (size_t)pp.rows_max;
    CS = (int)cl.num_blocks();
    rank = (int)cl.block_rank();
    tid = threadIdx.x;
    lane = tid & 31;
    warp = tid >> 5;
    par = 0;
  }

  // totals over the cluster, in a fixed order, of the projections (slots 0..nproj-1) and /
  // or the r sums (slots M_RX, M_RX+1) -> S.rsum, identical on every CTA
  __device__ void cluster_reduce(float (&acc)[M_NV], int nproj, bool want_r) {
    if (nproj > 1) {
      float v16[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) v16[j] = acc[j];
      reduce_scatter16(v16, lane);
      if (!(lane & 1) && (lane >> 1) < nproj) S.red[warp][lane >> 1] = v16[0];
    } else if (nproj == 1) {
      const float t = warp_sum(acc[0]);
      if (lane == 0) S.red[warp][0] = t;
    }
    if (want_r) {
      const float x = warp_sum(acc[M_RX]), y = warp_sum(acc[M_RX + 1]);
      if (lane == 0) {
        S.red[warp][M_RX] = x;
        S.red[warp][M_RX + 1] = y;
      }
    }
    __syncthreads();
    const bool mine = tid < M_NV && (tid < nproj || (want_r && tid >= M_RX));
    if (mine) {
      float s = 0.f;
      for (int q = 0; q < NW; ++q) s += S.red[q][tid];
      // pushed into slot `rank` of every CTA of the cluster, so that the totals are read
      // from local shared memory after the barrier
      for (int r = 0; r < CS; ++r) cl.map_shared_rank(&S.part[par][0][0], r)[rank * M_NV + tid] = s;
    }
    cl.sync();  // every CTA's totals are visible
    if (mine) {
      float s = 0.f;
      for (int r = 0; r < CS; ++r) s += S.part[par][r][tid];
      S.rsum[tid] = s;
      if (tid < nproj) S.f3[tid] = (((tid >> 1) & 1) ? -s : s) / (float)n;
    }
    // a CTA writes into this parity's slots again two reductions later, after the barrier
    // of the next one, which every CTA reaches only after reading these totals
    par ^= 1;
    __syncthreads();
  }

  // one coupling evaluation at theta = y[base] + omega*(mh+ml) + sum_j W_j g_j with the
  // weights of row si (a stage argument, dp45.cu:90-106, or the dense output,
  // dp45.cu:70-76).  Writes g[gout] =
  // c (sin F_c - cos F_s) (kuramoto.cu:104-126) when gout >= 0 and the r sums when
  // want_r; store_y7 keeps the stage-7 argument (FSAL) as the next y
  __device__ void coupling(int base, int si, int nW, int g1, int gout, bool want_r, bool store_y7) {
    float acc[M_NV];
#pragma unroll
    for (int v = 0; v < M_NV; ++v) acc[v] = 0.f;
    const long long T = p.total;
    const bool proj = gout >= 0;
    // MU rows per thread and pass: every load of the MU rows is issued before any of their
    // arithmetic, so that their L2 latencies overlap (the shared-memory and y7 stores of a row
    // keep the compiler from hoisting the next row's loads itself).  Only the r sums are
    // accumulated here; the projections follow in a second pass over the rows' (cos, sin)
    // in shared memory, which keeps the registers of this loop free for the batch.  Each
    // thread visits its rows in the same order in both passes.
    float Wr[7];
#pragma unroll
    for (int j = 0; j < 7; ++j) Wr[j] = S.Wst[si][j];
    const float mh = S.mhs[si], ml = S.mls[si];
    for (int i0 = r0 + tid; i0 < r1; i0 += MU * NT) {
      float om[MU], yh[MU], yl[MU], gs[MU];
#pragma unroll
      for (int q = 0; q < MU; ++q) {
        const int i = i0 + q * NT;
        const bool ok = i < r1;
        const long long gi = off + i;
        om[q] = ok ? p.omega[gi] : 0.f;
        yh[q] = ok ? p.ph_hi[base * T + gi] : 0.f;
        yl[q] = ok ? p.ph_lo[base * T + gi] : 0.f;
        gs[q] = 0.f;
#pragma unroll
        for (int j = 0; j < 7; ++j)
          if (j < nW) gs[q] = __fmaf_rn(Wr[j], ok ? p.g[(long long)slot_of(j, g1) * T + gi] : 0.f, gs[q]);
      }
#pragma unroll
      for (int q = 0; q < MU; ++q) {
        const int i = i0 + q * NT;
        if (i >= r1) break;
        const long long gi = off + i;
        const f2 pr = two_prod(om[q], mh);
        const f2 s1 = two_sum(yh[q], pr.hi);
        const f2 s2 = two_sum(s1.hi, gs[q]);
        const float lo = yl[q] + ((s1.lo + s2.lo) + __fmaf_rn(om[q], ml, pr.lo));
        float sn, cs;
        sincos_pair(s2.hi, lo, &sn, &cs);
        xs[i - r0] = make_float2(cs, sn);
        if (store_y7) {
          const f2 y = two_sum(s2.hi, lo);
          float hi7 = y.hi, lo7 = y.lo;
          long long w7 = p.ph_w[base * T + gi];
          wrap_phase(hi7, lo7, w7);
          p.ph_hi[(base ^ 1) * T + gi] = hi7;
          p.ph_lo[(base ^ 1) * T + gi] = lo7;
          p.ph_w[(base ^ 1) * T + gi] = w7;
        }
        acc[M_RX] += cs;
        acc[M_RX + 1] += sn;
      }
    }
    if (proj) {
      // sum over the rows with u_mn = +1 (the factor bits above k are zero)
      for (int i = r0 + tid; i < r1; i += NT) {
        const float2 x = xs[i - r0];
        const uint32_t u = ubits[i - r0];
#pragma unroll
        for (int m = 0; m < M_KMAX; ++m) {
          if (u & (1u << m)) {
            acc[2 * m] += x.x;
            acc[2 * m + 1] += x.y;
          }
        }
      }
    }
    // sum_n u_mn x_n = 2 (sum over u_mn = +1) - sum_n x_n
    if (proj) {
#pragma unroll
      for (int m = 0; m < M_KMAX; ++m) {
        acc[2 * m] = 2.f * acc[2 * m] - acc[M_RX];
        acc[2 * m + 1] = 2.f * acc[2 * m + 1] - acc[M_RX + 1];
      }
    }
    if (proj || want_r) cluster_reduce(acc, proj ? 2 * k : 0, want_r);
    if (!proj) return;
    // f3_m = (-1)^m / N sum_n u_mn (cos_n, sin_n) (m1), F_n = sum_m u_mn f3_m in order of
    // m (m2), tabulated once per sign pattern
    for (int pat = tid; pat < (1 << k); pat += NT) {
      float Fc = 0.f, Fs = 0.f;
      for (int m = 0; m < k; ++m) {
        const float fc = S.f3[2 * m], fs = S.f3[2 * m + 1];
        const bool pos = (pat >> m) & 1;
        Fc += pos ? fc : -fc;
        Fs += pos ? fs : -fs;
      }
      S.tab[pat] = make_float2(Fc, Fs);
    }
    __syncthreads();
    float* gdst = p.g + (long long)gout * T + off;
    for (int i = r0 + tid; i < r1; i += NT) {
      const float2 F = S.tab[ubits[i - r0]];
      const float2 x = xs[i - r0];
      gdst[i] = c1 * (x.y * F.x - x.x * F.y);
    }
  }

  // the stage and error weights of the next attempt from S.h (dp45.cu:90-106, 116), by
  // the lanes of warp 0 in parallel
  __device__ void fill_stage_tables() {
    const double h = S.h;
    for (int e = lane; e < 6 * 8 + 6 + 7; e += 32) {
      if (e < 48) {
        const int s = 2 + e / 8, j = e % 8;
        S.Wst[s - 2][j] = (j < s - 1) ? (float)(h * A_TAB[s - 1][j]) : 0.f;
      } else if (e < 54) {
        const int s = 2 + (e - 48);
        const double mh = C_TAB[s - 1] * h;
        const float hi = (float)mh;
        S.mhs[s - 2] = hi;
        S.mls[s - 2] = (float)(mh - (double)hi);
      } else {
        S.E[e - 54] = (float)(h * E_TAB[e - 54]);
      }
    }
  }

  __device__ void record(const MInst& I, int slot) {
    if (rank == 0 && tid == 0) {
      const float xn = S.rsum[M_RX] / (float)n, yn = S.rsum[M_RX + 1] / (float)n;
      p.out_r[I.order + slot] = sqrtf(xn * xn + yn * yn);
    }
  }

  __device__ void run_network(const MInst& I) {
    n = I.n;
    k = I.k;
    off = I.off;
    c1 = I.c;
    const int R = (n + CS - 1) / CS;
    r0 = min(n, rank * R);
    r1 = min(n, r0 + R);
    MNet& G = p.state[I.id];
    const int stage = G.stage;  // the same on every CTA of the cluster
    if (stage == 2) return;     // finished by an earlier launch
    if (rank == 0 && tid == 0) S.t_start = now_ns();
    // factor bits (low bit of Philox element m*N + i, kuramoto.cu:128-135) and, on a fresh
    // start, y(0)
    for (int i = r0 + tid; i < r1; i += NT) {
      uint32_t w = 0;
      for (int m = 0; m < k; ++m)
        w |= (stream_word(I.seed, (unsigned long long)m * (unsigned long long)n + (unsigned long long)i) & 1u) << m;
      ubits[i - r0] = (uint8_t)w;
      if (stage == 0) {
        const double th = (double)p.theta0[off + i];
        const double kk = rint(th / TWO_PI_D);
        const double rr = th - kk * TWO_PI_D;
        const float hi = (float)rr;
        p.ph_hi[off + i] = hi;
        p.ph_lo[off + i] = (float)(rr - (double)hi);
        p.ph_w[off + i] = (long long)kk;
      }
    }
    if (tid == 0) {
      if (stage == 0) {
        S.t = 0.0;
        S.h = p.h0;
        S.t_last = 0.0;
        S.acc = S.rej = 0;
        S.rot_y = S.rot_g = 0;
        S.eval_i = S.eval_end = 0;
        S.status = 0;
      } else {
        S.t = G.t;
        S.h = G.h;
        S.t_last = G.t_last;
        S.acc = G.acc;
        S.rej = G.rej;
        S.rot_y = G.rot_y;
        S.rot_g = G.rot_g;
        S.eval_i = G.eval_i;
        S.eval_end = G.eval_end;
        S.status = G.status;
      }
      S.mhs[6] = S.mls[6] = 0.f;
    }
    if (warp == 0) {
      __syncwarp();
      fill_stage_tables();
    }
    __syncthreads();
    if (stage == 0) {
      // first slope of the run (dp45.cu:151) and the record at t = 0
      coupling(0, 6, 0, 0, 0, true, false);
      record(I, 0);
    }
    long long attempts = 0;
    const long long T = p.total;
    while (true) {
      if (S.eval_i < S.eval_end) {
        // dense output at the next record time inside the last step (dp45.cu:70-76);
        // after the accept, k1 of the step sits in the k7 slot and vice versa
        if (tid == 0) {
          const double te = (double)(p.dtf * (float)(S.eval_i + 1));
          const double hs = S.t - S.t_last, dl = te - S.t_last, x = dl / hs;
          for (int j = 0; j < 7; ++j) {
            const double cc = ((P_TAB[j][3] * x + P_TAB[j][2]) * x + P_TAB[j][1]) * x * x + P_TAB[j][0] * x;
            S.Wst[6][j] = (float)(hs * cc);
          }
          S.mhs[6] = (float)dl;
          S.mls[6] = (float)(dl - (double)S.mhs[6]);
        }
        __syncthreads();
        coupling(S.rot_y ^ 1, 6, 7, S.rot_g ? 0 : 6, -1, true, false);
        record(I, 1 + S.eval_i);
        __syncthreads();  // every thread has read eval_i
        if (tid == 0) S.eval_i++;
        __syncthreads();
        continue;
      }
      if (!(S.t < p.t1) || S.status != 0) break;
      if (p.max_attempts >= 0 && attempts >= p.max_attempts) break;
      attempts++;
      // one attempt (dp45_step, dp45.cu:87-141).  The weights were filled after the last
      // controller decision; stage s + 1 needs no barrier of its own after stage s, because
      // every thread reads and writes the same rows in every stage and the shared buffers
      // of the reduction and the table are ordered by the barriers inside the reduction
      const int g1 = S.rot_g ? 6 : 0;
      for (int s = 2; s <= 7; ++s)
        coupling(S.rot_y, s - 2, s - 1, g1, s < 7 ? s - 1 : 6 - g1, false, s == 7);
      // error norm sqrt(sum (err_i / tol_i)^2 / N) (dp45.cu:79-84, 116-119); the omega
      // parts of the slopes cancel in the error weights
      float e2[M_NV];
#pragma unroll
      for (int v = 0; v < M_NV; ++v) e2[v] = 0.f;
      for (int i = r0 + tid; i < r1; i += NT) {
        const long long gi = off + i;
        float e = 0.f;
#pragma unroll
        for (int j = 0; j < 7; ++j) e = __fmaf_rn(S.E[j], p.g[(long long)slot_of(j, g1) * T + gi], e);
        float tol = (float)p.atol;
        if (p.rtol != 0.0) {
          const long long a = S.rot_y * T + gi, b = (S.rot_y ^ 1) * T + gi;
          const float a0 = fabsf(__fmaf_rn((float)p.ph_w[a], P2_1, p.ph_hi[a]));
          const float a1 = fabsf(__fmaf_rn((float)p.ph_w[b], P2_1, p.ph_hi[b]));
          tol = (float)p.atol + (float)p.rtol * fmaxf(a0, a1);
        }
        const float ye = e / tol;
        e2[0] = __fmaf_rn(ye, ye, e2[0]);
      }
      cluster_reduce(e2, 1, false);
      // controller (dp45.cu:109-139)
      if (tid == 0) {
        const double norm = sqrt((double)S.rsum[0]) / sqrt((double)n);
        const double h = S.h;
        if (isnan(norm)) {
          S.status = KURA_ERR_NONFINITE;
        } else {
          // 0.9 norm^(-1/5); norm = +inf gives 0: a rejection with the 0.2 floor
          const double factor = (double)(0.9f * exp2f(-0.2f * log2f((float)norm)));
          if (norm < 1.0) {
            S.t_last = S.t;
            S.t = S.t + h;
            S.rot_y ^= 1;
            S.rot_g ^= 1;
            S.acc++;
            S.h = h * fmin(factor, 10.0);
            int e = S.eval_i;
            while (e < p.n_eval && S.t >= (double)(p.dtf * (float)(e + 1))) e++;
            S.eval_end = e;
          } else {
            S.rej++;
            if (factor < 1.0) S.h = h * fmax(factor, 0.2);
            if (!(S.h >= 1e-14 * fmax(1.0, fabs(S.t)))) S.status = KURA_ERR_STEP_UNDERFLOW;
          }
        }
      }
      if (warp == 0) {
        __syncwarp();
        fill_stage_tables();
      }
      __syncthreads();
    }
    const bool finished = !(S.t < p.t1) || S.status != 0;
    if (p.theta_out && finished)
      for (int i = r0 + tid; i < r1; i += NT) {
        const long long a = S.rot_y * T + off + i;
        p.theta_out[off + i] = (float)((double)p.ph_w[a] * TWO_PI_D + (double)p.ph_hi[a] + (double)p.ph_lo[a]);
      }
    // every CTA has read G.stage and S before rank 0 rewrites the state
    cl.sync();
    if (rank == 0 && tid == 0) {
      G.t = S.t;
      G.h = S.h;
      G.t_last = S.t_last;
      G.acc = S.acc;
      G.rej = S.rej;
      G.rot_y = S.rot_y;
      G.rot_g = S.rot_g;
      G.eval_i = S.eval_i;
      G.eval_end = S.eval_end;
      G.status = S.status;
      G.stage = finished ? 2 : 1;
      G.ns += now_ns() - S.t_start;
      p.accepted[I.id] = S.acc;
      p.rejected[I.id] = S.rej;
      p.status[I.id] = finished ? (S.status == 0 ? 1 : S.status) : 0;
    }
  }

  __device__ void run() {
    while (true) {
      if (rank == 0 && tid == 0) S.idx = atomicAdd(p.queue, 1);
      cl.sync();
      const int idx = *cl.map_shared_rank(&S.idx, 0);
      cl.sync();  // rank 0 overwrites its slot only after every CTA has read it
      if (idx >= p.count) break;
      run_network(p.inst[idx]);
      // the next network reuses shared memory that other CTAs may still read remotely
      cl.sync();
    }
  }
};

template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_multi(const MParams p) {
  __shared__ MSmem S;
  extern __shared__ __align__(16) unsigned char dyn[];
  Multi<NT> m(p, S, dyn);
  m.run();
}

size_t dyn_smem(int rows) { return ((size_t)rows * M_ROW_BYTES + 15) / 16 * 16; }

template <int NT>
cudaError_t launch_multi_t(const MParams& p, int cs, cudaStream_t st, int* grid_out) {
  auto f = k_multi<NT>;
  const size_t smem = dyn_smem(p.rows_max);
  cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (cs > 8) {
    e = cudaFuncSetAttribute(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3(cs);
  int clusters = 0;
  e = cudaOccupancyMaxActiveClusters(&clusters, (void*)f, &cfg);
  if (e != cudaSuccess) return e;
  if (clusters < 1) return cudaErrorInvalidConfiguration;
  clusters = std::min(clusters, std::max(1, p.count));
  cfg.gridDim = dim3(clusters * cs);
  if (grid_out) *grid_out = clusters * cs;
  return cudaLaunchKernelEx(&cfg, f, p);
}

template <int NT>
cudaError_t clusters_t(int cs, int rows, int* out) {
  auto f = k_multi<NT>;
  const size_t smem = dyn_smem(rows);
  cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (cs > 8) {
    e = cudaFuncSetAttribute(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = smem;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3(cs);
  return cudaOccupancyMaxActiveClusters(out, (void*)f, &cfg);
}

// clusters of `cs` CTAs of `nt` threads with `rows` rows each that fit on the GPU at once
cudaError_t clusters_of(int cs, int nt, int rows, int* out) {
  switch (nt) {
    case 256: return clusters_t<256>(cs, rows, out);
    case 512: return clusters_t<512>(cs, rows, out);
    case 1024: return clusters_t<1024>(cs, rows, out);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_multi(const MParams& p, int cs, int nt, cudaStream_t st, int* grid) {
  switch (nt) {
    case 256: return launch_multi_t<256>(p, cs, st, grid);
    case 512: return launch_multi_t<512>(p, cs, st, grid);
    case 1024: return launch_multi_t<1024>(p, cs, st, grid);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace
}  // namespace kura

using kura::MInst;
using kura::MParams;

struct kura_multi {
  int device = 0, count = 0, n_eval = 0, maxn = 0;
  long long total = 0;
  double t1 = 0, dt = 0, h0 = 0, atol = 0, rtol = 0;
  int want_cs = 0, want_nt = 0, cs = 0, nt = 0, grid = 0, csmin = 1;
  bool tuned = false;
  std::vector<MInst> queue;  // largest network first
  cudaStream_t st = nullptr;
  cudaStream_t st2 = nullptr;  // the heavy networks' launch, beside the main one
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaEvent_t evf = nullptr, evj = nullptr;  // fork after the pilot, join of the heavy launch
  MInst* d_instH = nullptr;
  int heavy = 0;
  MInst* d_inst = nullptr;
  int *d_queue = nullptr, *d_status = nullptr;
  float *d_om = nullptr, *d_th = nullptr, *d_hi = nullptr, *d_lo = nullptr, *d_g = nullptr, *d_r = nullptr,
        *d_theta = nullptr;
  long long *d_w = nullptr, *d_acc = nullptr, *d_rej = nullptr;
  cudaGraphExec_t graph = nullptr;   // pilot: every network's first attempts, in size order
  kura::MNet* d_state = nullptr;
  MInst* d_inst2 = nullptr;
  int pilot_attempts = 32;
  kura_multi_stats stats = {};
};

namespace {

int mfail(int code, const std::string& msg) {
  kura::set_last_error(msg.c_str());
  return code;
}
#define MCU(x)                                                                                    \
  do {                                                                                            \
    cudaError_t e_ = (x);                                                                         \
    if (e_ != cudaSuccess)                                                                        \
      return mfail(e_ == cudaErrorMemoryAllocation ? KURA_ERR_NOMEM : KURA_ERR_CUDA,              \
                   std::string(#x) + ": " + cudaGetErrorString(e_));                             \
  } while (0)

MParams base_params(kura_multi* m) {
  MParams p;
  std::memset(&p, 0, sizeof(p));
  p.inst = m->d_inst;
  p.count = m->count;
  p.queue = m->d_queue;
  p.omega = m->d_om;
  p.theta0 = m->d_th;
  p.ph_hi = m->d_hi;
  p.ph_lo = m->d_lo;
  p.ph_w = m->d_w;
  p.g = m->d_g;
  p.total = m->total;
  p.t1 = m->t1;
  p.h0 = m->h0;
  p.atol = m->atol;
  p.rtol = m->rtol;
  p.n_eval = m->n_eval;
  p.dtf = (float)m->dt;
  p.out_r = m->d_r;
  p.theta_out = m->d_theta;
  p.accepted = m->d_acc;
  p.rejected = m->d_rej;
  p.status = m->d_status;
  p.max_attempts = -1;
  p.state = m->d_state;
  return p;
}

// Runs a stratified sample of the networks for a few attempts at every candidate shape and
// keeps the one with the shortest predicted integration.  A network's predicted time is its
// predicted step count, (t1 - t) / h after the trial, times the time per attempt it took in
// this shape.  The prediction for the shape is the trial's time scaled to all networks (the
// first attempts of every network) plus the larger of the balanced total (the sum over the
// networks, scaled to all of them, over the clusters) and twice the longest network.
// Step counts are heavy-tailed (they grow with a network's fastest oscillator and with its
// coupling as it synchronises), so the latency of one network's step often decides; the
// factor 2 is there because the first attempts underestimate the longest networks the most
// (on 512 networks with Cauchy frequencies they predicted 1/5 of the total step count and
// 1/11 of the longest network's).  KURA_MULTI_TUNE_LOG=1 prints every trial's figures.
int autotune(kura_multi* m) {
  const int S = std::min(m->count, 2 * 152);
  std::vector<MInst> sample(S);
  for (int i = 0; i < S; ++i) {
    sample[i] = m->queue[(size_t)i * m->count / S];
    sample[i].id = i;
    sample[i].order = (long long)i * (m->n_eval + 1);
  }
  int maxn = 0;
  for (const MInst& q : sample) maxn = std::max(maxn, q.n);
  MCU(cudaMemcpyAsync(m->d_inst, sample.data(), sizeof(MInst) * S, cudaMemcpyHostToDevice, m->st));
  MParams q = base_params(m);
  q.count = S;
  q.theta_out = nullptr;
  q.max_attempts = 24;
  double best = -1;
  float best_ms = 0;
  std::vector<kura::MNet> st(S);
  const char* env = std::getenv("KURA_MULTI_TUNE_LOG");  // "1": print every trial's prediction
  const bool tune_log = env && env[0] == '1';
  const int css[] = {1, 2, 4, 8, 16};
  const int nts[] = {256, 512, 1024};
  for (int c : css) {
    if ((m->want_cs > 0 && c != m->want_cs) || c < m->csmin) continue;
    q.rows_max = (maxn + c - 1) / c;
    for (int t : nts) {
      if (m->want_nt > 0 && t != m->want_nt) continue;
      MCU(cudaMemsetAsync(m->d_queue, 0, sizeof(int), m->st));
      MCU(cudaMemsetAsync(m->d_state, 0, sizeof(kura::MNet) * S, m->st));
      MCU(cudaEventRecord(m->ev[0], m->st));
      cudaError_t e = kura::launch_multi(q, c, t, m->st, nullptr);
      if (e != cudaSuccess) {
        cudaGetLastError();  // an unlaunchable shape (cluster too large for a GPC): skip it
        continue;
      }
      MCU(cudaEventRecord(m->ev[1], m->st));
      MCU(cudaStreamSynchronize(m->st));
      float ms = 0;
      MCU(cudaEventElapsedTime(&ms, m->ev[0], m->ev[1]));
      MCU(cudaMemcpy(st.data(), m->d_state, sizeof(kura::MNet) * S, cudaMemcpyDeviceToHost));
      int fit = 0;
      if (kura::clusters_of(c, t, q.rows_max, &fit) != cudaSuccess || fit < 1) {
        cudaGetLastError();
        continue;
      }
      double total = 0, longest = 0;
      for (int i = 0; i < S; ++i) {
        const kura::MNet& G = st[i];
        const long long att = G.acc + G.rej;
        if (att < 1) continue;
        const double per = (double)G.ns / (double)att;
        const double steps = G.stage == 2 ? 0.0 : std::max(0.0, m->t1 - G.t) / std::max(G.h, 1e-300);
        total += steps * per;
        longest = std::max(longest, steps * per);
      }
      const double balanced = total * ((double)m->count / S) / std::min(fit, m->count);
      const double first = (double)ms * 1e6 * ((double)m->count / S);  // the trial's attempts for all
      const double est = first + std::max(balanced, 2.0 * longest);
      if (tune_log)
        std::fprintf(stderr, "kura_multi autotune: cluster %d x %d threads, %d clusters, trial %.3f ms, "
                     "balanced %.3f s, longest %.3f s, predicted %.3f s\n", c, t, fit, ms, balanced * 1e-9,
                     longest * 1e-9, est * 1e-9);
      if (best < 0 || est < best) {
        best = est;
        best_ms = ms;
        m->cs = c;
        m->nt = t;
      }
    }
  }
  if (best < 0) return mfail(KURA_ERR_UNSUPPORTED, "no launchable cluster shape for these networks");
  m->stats.tune_ms = best_ms;
  return KURA_OK;
}

cudaError_t capture(kura_multi* m, const MParams& p, bool reset_state, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(m->st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaError_t e1 = cudaMemsetAsync(m->d_queue, 0, sizeof(int), m->st);
  if (e1 == cudaSuccess && reset_state) e1 = cudaMemsetAsync(m->d_state, 0, sizeof(kura::MNet) * m->count, m->st);
  cudaError_t e2 = e1 == cudaSuccess ? kura::launch_multi(p, m->cs, m->nt, m->st, &m->grid) : e1;
  cudaError_t e3 = cudaStreamEndCapture(m->st, &g);
  if (e2 != cudaSuccess || e3 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return e2 != cudaSuccess ? e2 : e3;
  }
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  return e;
}

// The pilot launch runs the first attempts of every network (largest first) and is
// captured in a CUDA graph.  The host then orders the unfinished networks by their
// predicted remaining work, (t1 - t) / h steps of (N + 2048) row-equivalents each, and
// launches the rest in that order (longest-processing-time first): the few networks whose
// work alone exceeds a cluster's fair share go to large clusters on a second stream, the
// others to the autotuned shape.
int build_graph(kura_multi* m) {
  MParams p = base_params(m);
  p.rows_max = (m->maxn + m->cs - 1) / m->cs;
  MCU(cudaMemcpyAsync(m->d_inst, m->queue.data(), sizeof(MInst) * m->count, cudaMemcpyHostToDevice, m->st));
  MCU(cudaStreamSynchronize(m->st));
  p.max_attempts = m->pilot_attempts;
  cudaError_t e = capture(m, p, true, &m->graph);
  if (e != cudaSuccess)
    return mfail(KURA_ERR_CUDA, std::string("capturing the multi-network launches: ") + cudaGetErrorString(e));
  return KURA_OK;
}

}  // namespace

extern "C" int kura_multi_create(const kura_instance* inst, int32_t count, double t1, double dt, double h0,
                                 double atol, double rtol, int32_t device, int32_t cluster_size,
                                 int32_t block_threads, kura_multi** out) {
  if (!out) return mfail(KURA_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (!inst || count < 1) return mfail(KURA_ERR_INVALID, "no networks");
  if (!(dt > 0) || !(h0 > 0) || !(atol > 0) || !(t1 >= 0) || !(rtol >= 0))
    return mfail(KURA_ERR_INVALID, "need dt > 0, h0 > 0, atol > 0, rtol >= 0, t1 >= 0");
  if (cluster_size != 0 && (cluster_size < 1 || cluster_size > kura::M_MAX_CLUSTER ||
                            (cluster_size & (cluster_size - 1))))
    return mfail(KURA_ERR_INVALID, "cluster_size must be 0 (autotune) or a power of two <= 16");
  if (block_threads != 0 && block_threads != 256 && block_threads != 512 && block_threads != 1024)
    return mfail(KURA_ERR_INVALID, "block_threads must be 0 (autotune), 256, 512 or 1024");
  kura_multi* m = new kura_multi();
  m->device = device;
  m->count = count;
  m->t1 = t1;
  m->dt = dt;
  m->h0 = h0;
  m->atol = atol;
  m->rtol = rtol;
  m->want_cs = cluster_size;
  m->want_nt = block_threads;
  // records at t = 0 and dt*n, n = 1 .. int(t1/dt), in float like the reference (kuramoto.cu:543-550)
  const float dtf = (float)dt, t1f = (float)t1;
  m->n_eval = int(t1f / dtf);
  m->queue.resize(count);
  for (int i = 0; i < count; ++i) {
    const kura_instance& q = inst[i];
    if (q.n < 1 || q.n > (int64_t)kura::M_MAX_CLUSTER * (kura::M_SMEM_CAP / kura::M_ROW_BYTES)) {
      delete m;
      return mfail(KURA_ERR_UNSUPPORTED, "network " + std::to_string(i) + ": n outside 1.." +
                                             std::to_string(kura::M_MAX_CLUSTER * (kura::M_SMEM_CAP / kura::M_ROW_BYTES)));
    }
    if (q.k < 0 || q.k > 8) {
      delete m;
      return mfail(KURA_ERR_UNSUPPORTED, "network " + std::to_string(i) + ": k outside 0..8");
    }
    MInst& I = m->queue[i];
    I.n = (int)q.n;
    I.k = q.k;
    I.seed = q.seed;
    I.id = i;
    I.c = q.c;
    I.pad = 0.f;
    I.off = m->total;
    I.order = (long long)i * (m->n_eval + 1);
    m->total += q.n;
    m->maxn = std::max(m->maxn, (int)q.n);
  }
  std::stable_sort(m->queue.begin(), m->queue.end(), [](const MInst& a, const MInst& b) { return a.n > b.n; });
  while ((size_t)((m->maxn + m->csmin - 1) / m->csmin) * kura::M_ROW_BYTES > (size_t)kura::M_SMEM_CAP) m->csmin *= 2;
  if (cluster_size > 0 && cluster_size < m->csmin) {
    delete m;
    return mfail(KURA_ERR_UNSUPPORTED, "cluster_size too small for the largest network (needs >= " +
                                           std::to_string(m->csmin) + ")");
  }
  auto fail_free = [&](int rc) {
    kura_multi_destroy(m);
    return rc;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail_free(mfail(KURA_ERR_CUDA, cudaGetErrorString(e)));
  const long long T = m->total;
  const size_t rec = (size_t)count * (m->n_eval + 1);
  struct A {
    void** p;
    size_t bytes;
  } allocs[] = {
      {(void**)&m->d_inst, sizeof(MInst) * count}, {(void**)&m->d_queue, 2 * sizeof(int)},
      {(void**)&m->d_status, sizeof(int) * count}, {(void**)&m->d_om, sizeof(float) * T},
      {(void**)&m->d_th, sizeof(float) * T},       {(void**)&m->d_hi, sizeof(float) * 2 * T},
      {(void**)&m->d_lo, sizeof(float) * 2 * T},   {(void**)&m->d_w, sizeof(long long) * 2 * T},
      {(void**)&m->d_g, sizeof(float) * 7 * T},    {(void**)&m->d_r, sizeof(float) * rec},
      {(void**)&m->d_theta, sizeof(float) * T},    {(void**)&m->d_acc, sizeof(long long) * count},
      {(void**)&m->d_rej, sizeof(long long) * count},
      {(void**)&m->d_state, sizeof(kura::MNet) * count}, {(void**)&m->d_inst2, sizeof(MInst) * count},
      {(void**)&m->d_instH, sizeof(MInst) * count},
  };
  for (auto& a : allocs) {
    e = cudaMalloc(a.p, a.bytes);
    if (e != cudaSuccess)
      return fail_free(mfail(e == cudaErrorMemoryAllocation ? KURA_ERR_NOMEM : KURA_ERR_CUDA,
                             std::string("device allocation: ") + cudaGetErrorString(e)));
  }
  e = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->st2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&m->evf, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&m->evj, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreate(&m->ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&m->ev[1]);
  if (e != cudaSuccess) return fail_free(mfail(KURA_ERR_CUDA, cudaGetErrorString(e)));
  *out = m;
  return KURA_OK;
}

extern "C" void kura_multi_destroy(kura_multi* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  if (m->st) cudaStreamSynchronize(m->st);
  if (m->graph) cudaGraphExecDestroy(m->graph);
  void* ptrs[] = {m->d_inst, m->d_queue, m->d_status, m->d_om,    m->d_th,    m->d_hi,    m->d_lo,
                  m->d_w,    m->d_g,     m->d_r,      m->d_theta, m->d_acc,   m->d_rej,   m->d_state,
                  m->d_inst2, m->d_instH};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  for (cudaEvent_t v : m->ev)
    if (v) cudaEventDestroy(v);
  if (m->evf) cudaEventDestroy(m->evf);
  if (m->evj) cudaEventDestroy(m->evj);
  if (m->st2) {
    cudaStreamSynchronize(m->st2);
    cudaStreamDestroy(m->st2);
  }
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
}

extern "C" int kura_multi_integrate(kura_multi* m, const float* omega, const float* theta0, float* order,
                                    float* theta_final, int64_t* accepted) {
  if (!m) return mfail(KURA_ERR_INVALID, "handle is NULL");
  if (!omega || !theta0 || !order) return mfail(KURA_ERR_INVALID, "omega, theta0 and order are required");
  MCU(cudaSetDevice(m->device));
  const long long T = m->total;
  MCU(cudaMemcpyAsync(m->d_om, omega, sizeof(float) * T, cudaMemcpyHostToDevice, m->st));
  MCU(cudaMemcpyAsync(m->d_th, theta0, sizeof(float) * T, cudaMemcpyHostToDevice, m->st));
  MCU(cudaMemsetAsync(m->d_status, 0, sizeof(int) * m->count, m->st));
  if (!m->tuned) {
    if (m->want_cs > 0 && m->want_nt > 0) {
      m->cs = m->want_cs;
      m->nt = m->want_nt;
    } else {
      int rc = autotune(m);
      if (rc != KURA_OK) return rc;
      MCU(cudaMemsetAsync(m->d_status, 0, sizeof(int) * m->count, m->st));
    }
    int rc = build_graph(m);
    if (rc != KURA_OK) return rc;
    m->tuned = true;
  }
  MCU(cudaEventRecord(m->ev[0], m->st));
  MCU(cudaGraphLaunch(m->graph, m->st));
  std::vector<kura::MNet> state(m->count);
  MCU(cudaMemcpyAsync(state.data(), m->d_state, sizeof(kura::MNet) * m->count, cudaMemcpyDeviceToHost, m->st));
  MCU(cudaStreamSynchronize(m->st));
  std::vector<std::pair<double, int>> cost;
  cost.reserve(m->count);
  for (int q = 0; q < m->count; ++q) {
    const MInst& I = m->queue[q];
    const kura::MNet& G = state[I.id];
    const double steps = G.stage == 2 ? 0.0 : std::max(0.0, m->t1 - G.t) / std::max(G.h, 1e-300);
    cost.push_back({steps * ((double)I.n + 2048.0), q});
  }
  std::stable_sort(cost.begin(), cost.end(), [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
    return a.first > b.first;
  });
  std::vector<MInst> order2(m->count);
  for (int q = 0; q < m->count; ++q) order2[q] = m->queue[cost[q].second];
  // Networks whose predicted work alone exceeds a cluster's fair share of the main launch
  // (at most 4) run in a launch of their own with clusters of 1024-thread CTAs, started
  // first on a second stream so that its CTAs take whole SMs; the main launch fills the
  // rest.  Such a network sets the end of the run, and its time is bound by the latency of
  // one step rather than by the SMs it holds.
  double total = 0;
  for (const auto& c : cost) total += c.first;
  const double share = total / std::max(1, m->grid / m->cs);
  int nh = 0;
  while (nh < m->count && nh < 4 && cost[nh].first > share) ++nh;
  int hcs = 0;
  if (nh > 0) {
    int maxnH = 0;
    for (int q = 0; q < nh; ++q) maxnH = std::max(maxnH, order2[q].n);
    int want = 2;
    while (want < 16 && want * 2048 < maxnH) want *= 2;
    MCU(cudaMemcpyAsync(m->d_instH, order2.data(), sizeof(MInst) * nh, cudaMemcpyHostToDevice, m->st));
    MCU(cudaEventRecord(m->evf, m->st));
    MCU(cudaStreamWaitEvent(m->st2, m->evf, 0));
    MCU(cudaMemsetAsync(m->d_queue + 1, 0, sizeof(int), m->st2));
    MParams ph = base_params(m);
    ph.inst = m->d_instH;
    ph.count = nh;
    ph.queue = m->d_queue + 1;
    for (int c = want; c >= 2 && !hcs; c /= 2) {
      ph.rows_max = (maxnH + c - 1) / c;
      if ((size_t)ph.rows_max * kura::M_ROW_BYTES > (size_t)kura::M_SMEM_CAP) break;
      if (kura::launch_multi(ph, c, 1024, m->st2, nullptr) == cudaSuccess)
        hcs = c;
      else
        cudaGetLastError();  // cluster shape not available: try a smaller one
    }
    if (hcs) {
      MCU(cudaEventRecord(m->evj, m->st2));
    } else {
      nh = 0;
    }
  }
  m->heavy = nh;
  MCU(cudaMemcpyAsync(m->d_inst2, order2.data() + nh, sizeof(MInst) * (m->count - nh), cudaMemcpyHostToDevice,
                      m->st));
  {
    MParams p2 = base_params(m);
    p2.inst = m->d_inst2;
    p2.count = m->count - nh;
    p2.rows_max = (m->maxn + m->cs - 1) / m->cs;
    MCU(cudaMemsetAsync(m->d_queue, 0, sizeof(int), m->st));
    if (p2.count > 0) MCU(kura::launch_multi(p2, m->cs, m->nt, m->st, nullptr));
  }
  if (nh > 0) MCU(cudaStreamWaitEvent(m->st, m->evj, 0));
  MCU(cudaEventRecord(m->ev[1], m->st));
  const size_t rec = (size_t)m->count * (m->n_eval + 1);
  MCU(cudaMemcpyAsync(order, m->d_r, sizeof(float) * rec, cudaMemcpyDeviceToHost, m->st));
  if (theta_final)
    MCU(cudaMemcpyAsync(theta_final, m->d_theta, sizeof(float) * T, cudaMemcpyDeviceToHost, m->st));
  std::vector<long long> acc(m->count), rej(m->count);
  std::vector<int> status(m->count);
  MCU(cudaMemcpyAsync(acc.data(), m->d_acc, sizeof(long long) * m->count, cudaMemcpyDeviceToHost, m->st));
  MCU(cudaMemcpyAsync(rej.data(), m->d_rej, sizeof(long long) * m->count, cudaMemcpyDeviceToHost, m->st));
  MCU(cudaMemcpyAsync(status.data(), m->d_status, sizeof(int) * m->count, cudaMemcpyDeviceToHost, m->st));
  MCU(cudaStreamSynchronize(m->st));
  float ms = 0;
  MCU(cudaEventElapsedTime(&ms, m->ev[0], m->ev[1]));
  kura_multi_stats& s = m->stats;
  s.kernel_ms = ms;
  s.cluster_size = m->cs;
  s.block_threads = m->nt;
  s.grid = m->grid;
  s.heavy = m->heavy;
  s.accepted = s.rejected = 0;
  s.osc_steps = 0;
  int bad = -1;
  for (const MInst& I : m->queue) {
    s.accepted += acc[I.id];
    s.rejected += rej[I.id];
    s.osc_steps += (double)acc[I.id] * I.n;
    if (accepted) accepted[I.id] = acc[I.id];
    if (status[I.id] != 1 && bad < 0) bad = I.id;
  }
  if (bad >= 0) {
    const int st = status[bad];
    return mfail(st < 0 ? st : KURA_ERR_CUDA,
                 "network " + std::to_string(bad) + (st < 0 ? " failed" : " was not integrated"));
  }
  return KURA_OK;
}

extern "C" int kura_multi_get_stats(const kura_multi* m, kura_multi_stats* s) {
  if (!m || !s) return mfail(KURA_ERR_INVALID, "NULL argument");
  *s = m->stats;
  return KURA_OK;
}
