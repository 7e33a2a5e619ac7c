// kura_tensor.cu -- the shared-adjacency ensemble on tcgen05 tensor cores.
//
// B trajectories (up to 128) share one dense adjacency A and the frequencies, with
// their own phases, coupling constants and adaptive steps.  Each RHS of the batch is
// one GEMM over A:
//   F[i][(cos|sin), b] = sum_j A_ij (cos, sin)(theta_jb)
// computed as (N A) x [X_hi | X_lo] with X = [cos | sin] split into BF16 hi + lo and FP32
// accumulation in TMEM; the GEMM epilogue forms g = c_b (sin F_c - cos F_s) / N directly.
// For the reference's volcano rule N*A_ij is an integer in [-K, K], exact in BF16, so the
// product carries the precision of the hi+lo split of X (about 2^-16).  A general
// adjacency is split as N A = A_hi + A_lo and the term A_lo X_hi comes from a second GEMM
// pass (split-BF16 hi + lo operands, FP32 accumulation).
//
// The DP45 attempt (dp45_step, dp45.cu:87-141) is a fixed sequence of launches --
// coefficients, 6 x (stage, GEMM), error norm, controller, outputs -- captured once in a
// CUDA graph and replayed; every per-trajectory decision (accept/reject, step size, t,
// output crossings) stays on the device.  The host only polls a completion flag.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>
#include "kura.h"
#include "kura_device.cuh"
#include "kura_kernels.cuh"
#include "kura_tensor.h"
#include "kura_tensor_gemm.cuh"

namespace kura {

namespace {

constexpr int T_MAXC = 32;  // output crossings handled per step
// K per pipeline stage of the coupling GEMM (32: 64-byte swizzle rows; 64: 128-byte rows).
// 64 (three 64 KB stages, eight MMAs per stage handshake) measured 7 % faster per launch at
// N=65536, B=128 than 32 (seven 32 KB stages, four MMAs per handshake)
#ifndef KURA_GEMM_BK
#define KURA_GEMM_BK 64
#endif
constexpr int TE_BK = KURA_GEMM_BK;
constexpr int T_RBLK = 256; // rows per block of the reduction kernels

struct TCoef {
  float W[7];
  float E[7];
  float m_hi, m_lo;
  int slot[7];
  int base, gout, active, store_y7, rec, nW;
  float c1;
  int pad;
};

struct TView {
  int n, np, bp, B, mode;
  const float* omega;
  float* ph_hi;
  float* ph_lo;
  long long* ph_w;
  float* g;
  __nv_bfloat16* X;
  float2* x32;
  float* fin_theta;
  float* fin_coup;
  float* Flo;  // [2][bp][np] partial couplings of the A_lo pass (general adjacency)
};

// row of X holding column q (0 hi cos, 1 hi sin, 2 lo cos, 3 lo sin) of trajectory b: the
// trajectories are grouped by 64 so that each group's 4 x 64 columns are one contiguous
// block, the column block of one GEMM work unit
__host__ __device__ __forceinline__ int x_bph(int bp) { return bp > 64 ? 64 : bp; }
__device__ __forceinline__ size_t xrow(int q, int b, int bp) {
  const int g = x_bph(bp);
  return (size_t)(b / g) * 4 * g + (size_t)q * g + (b % g);
}
__device__ __forceinline__ int slot_k1(int rot_g) { return rot_g ? 6 : 0; }
__device__ __forceinline__ int slot_k7(int rot_g) { return rot_g ? 0 : 6; }

// ---------------------------------------------------------------- coefficients
// Per-trajectory sources: src[0] = phases y (first slope, RHS), src[1..6] = stages 2..7
// of the next attempt (dp45.cu:90-106), src[7] = dense output (set by the output kernels).
__global__ void k_t_coef(TrajG* traj, TCoef* src, int B, int bp, int fixed, int* any_active) {
  if (threadIdx.x == 0) {
    int a0 = 0, a1 = 0;
    for (int b = 0; b < B; ++b) {
      const TrajG& T = traj[b];
      a0 |= (T.status == 0 && T.need_k1);
      a1 |= (T.status == 0 && T.eval_i >= T.eval_end && T.t < T.t1);
    }
    any_active[0] = a0;
    any_active[1] = a1;
    any_active[2] = 1;
  }
  for (int t = threadIdx.x; t < 7 * B * 16; t += blockDim.x) {
    const int j = t & 15, b = (t >> 4) % B, sidx = (t >> 4) / B;  // sidx 0: y; 1..6: stage s = sidx + 1
    TCoef& S = src[sidx * bp + b];
    const TrajG& T = traj[b];
    const double h = T.h;
    const bool act = (T.status == 0 && T.eval_i >= T.eval_end && T.t < T.t1);
    if (sidx == 0) {
      if (j < 7) S.W[j] = 0.f;
      else if (j == 14) { S.m_hi = 0.f; S.m_lo = 0.f; }
      else if (j == 15) {
        S.nW = 0;
        for (int q = 0; q < 7; ++q) S.slot[q] = q;
        S.base = T.rot_y;
        S.gout = slot_k1(T.rot_g);
        S.active = (T.status == 0 && T.need_k1);
        S.store_y7 = 0;
        S.rec = 0;
        S.c1 = T.c1;
      }
      continue;
    }
    const int s = sidx + 1;
    if (j < 7) {
      S.W[j] = (j < s - 1) ? (float)(h * A_TAB[s - 1][j]) : 0.f;
    } else if (j < 14) {
      if (s == 7) S.E[j - 7] = (float)(h * E_TAB[j - 7]);
    } else if (j == 14) {
      double mh = C_TAB[s - 1] * h;
      float hi = (float)mh;
      S.m_hi = hi;
      S.m_lo = (float)(mh - (double)hi);
    } else {
      S.nW = s - 1;
      S.slot[0] = slot_k1(T.rot_g);
      for (int q = 1; q < 6; ++q) S.slot[q] = q;
      S.slot[6] = slot_k7(T.rot_g);
      S.base = T.rot_y;
      S.gout = (s < 7) ? s - 1 : slot_k7(T.rot_g);
      S.store_y7 = (s == 7);
      S.rec = 0;
      S.active = act;
      S.c1 = T.c1;
    }
  }
  (void)fixed;
}

// source for the end-of-run record (interpolation with k1 replaced by k7, as after the
// reference's FSAL copy, kuramoto.cu:632) or the current phases (RHS, no step taken)
__global__ void k_t_coef_final(TrajG* traj, TCoef* src, int B, const float* t_eval, int n_eval, int use_eval) {
  const int b = threadIdx.x;
  if (b >= B) return;
  TCoef& S = src[b];
  const TrajG& T = traj[b];
  for (int q = 0; q < 7; ++q) { S.W[q] = 0.f; S.slot[q] = q; }
  S.m_hi = S.m_lo = 0.f;
  S.nW = 0;
  S.base = T.rot_y;
  if (use_eval && n_eval > 0 && T.accepted > 0) {
    const double hs = T.t - T.t_last, dl = (double)t_eval[n_eval - 1] - T.t_last, x = dl / hs;
    for (int j = 0; j < 7; ++j) {
      const double c = ((P_TAB[j][3] * x + P_TAB[j][2]) * x + P_TAB[j][1]) * x * x + P_TAB[j][0] * x;
      S.W[j] = (float)(hs * c);
    }
    S.nW = 7;
    S.m_hi = (float)dl;
    S.m_lo = (float)(dl - (double)S.m_hi);
    const int ks = slot_k1(T.rot_g);
    S.slot[0] = ks;
    S.slot[6] = ks;
    S.base = T.rot_y ^ 1;
  }
  S.gout = -1;
  S.active = 1;
  S.store_y7 = 0;
  S.rec = 1;
  S.c1 = T.c1;
}

// ---------------------------------------------------------------- stage (elementwise)
// theta = phase[base] + omega*(m_hi+m_lo) + sum_j W_j g_j for (trajectory b, oscillator i);
// writes the BF16 hi/lo operand columns (cos, sin) and the FP32 (cos, sin) for the epilogue
__global__ void k_t_stage(TView v, const TCoef* src) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const TCoef& s = src[b];
  if (!s.active || i >= v.n) return;
  const size_t boff = ((size_t)s.base * v.bp + b) * v.np;
  const float om = v.omega[i];
  float gsum = 0.f;
  for (int j = 0; j < s.nW; ++j) gsum = __fmaf_rn(s.W[j], v.g[((size_t)s.slot[j] * v.bp + b) * v.np + i], gsum);
  const f2 pr = two_prod(om, s.m_hi);
  const f2 s1 = two_sum(v.ph_hi[boff + i], pr.hi);
  const f2 s2 = two_sum(s1.hi, gsum);
  const float lo = v.ph_lo[boff + i] + ((s1.lo + s2.lo) + __fmaf_rn(om, s.m_lo, pr.lo));
  float sn, cs;
  sincos_pair(s2.hi, lo, &sn, &cs);
  v.x32[(size_t)b * v.np + i] = make_float2(cs, sn);
  const __nv_bfloat16 ch = __float2bfloat16_rn(cs), sh = __float2bfloat16_rn(sn);
  const __nv_bfloat16 cl = __float2bfloat16_rn(cs - __bfloat162float(ch));
  const __nv_bfloat16 sl = __float2bfloat16_rn(sn - __bfloat162float(sh));
  v.X[xrow(0, b, v.bp) * v.np + i] = ch;
  v.X[xrow(1, b, v.bp) * v.np + i] = sh;
  v.X[xrow(2, b, v.bp) * v.np + i] = cl;
  v.X[xrow(3, b, v.bp) * v.np + i] = sl;
  if (s.store_y7 || s.rec) {
    f2 y = two_sum(s2.hi, lo);
    long long w = v.ph_w[boff + i];
    if (s.store_y7) {
      float hi7 = y.hi, lo7 = y.lo;
      long long w7 = w;
      wrap_phase(hi7, lo7, w7);
      const size_t o = ((size_t)(s.base ^ 1) * v.bp + b) * v.np + i;
      v.ph_hi[o] = hi7;
      v.ph_lo[o] = lo7;
      v.ph_w[o] = w7;
    } else if (v.fin_theta) {
      v.fin_theta[(size_t)b * v.np + i] = (float)((double)w * TWO_PI_D + (double)y.hi + (double)y.lo);
    }
  }
}

// ---------------------------------------------------------------- GEMM epilogues
// accumulator columns of work unit sp: [hi cos | hi sin | lo cos | lo sin] of trajectories
// sp*BP .. sp*BP + BP - 1, BP columns each
template <int BP> struct KuraEpi {
  TView v;
  const TCoef* src;
  float invn;
  int has_lo;
  __device__ void row(uint32_t taddr, int row, int m0, int sp) {
    const int i = m0 + row;
#pragma unroll 1
    for (int b0 = 0; b0 < BP; b0 += 16) {
      float hc[16], hs[16], lc[16], ls[16];
      umma::tmem_ld16(taddr + 0 * BP + b0, hc);
      umma::tmem_ld16(taddr + 1 * BP + b0, hs);
      umma::tmem_ld16(taddr + 2 * BP + b0, lc);
      umma::tmem_ld16(taddr + 3 * BP + b0, ls);
      umma::tmem_ld_wait();
      if (i >= v.n) continue;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int b = sp * BP + b0 + j;
        if (b >= v.B) break;
        const TCoef& s = src[b];
        if (!s.active) continue;
        float Fc = hc[j] + lc[j], Fs = hs[j] + ls[j];
        if (has_lo) {
          Fc += v.Flo[((size_t)0 * v.bp + b) * v.np + i];
          Fs += v.Flo[((size_t)1 * v.bp + b) * v.np + i];
        }
        Fc *= invn;
        Fs *= invn;
        const float2 x = v.x32[(size_t)b * v.np + i];
        const float gv = s.c1 * (x.y * Fc - x.x * Fs);
        if (s.gout >= 0) v.g[((size_t)s.gout * v.bp + b) * v.np + i] = gv;
        if (v.mode != 0 && s.rec) {
          v.fin_coup[((size_t)b * v.np + i) * 2] = Fc;
          v.fin_coup[((size_t)b * v.np + i) * 2 + 1] = Fs;
          if (v.mode == 2) v.fin_theta[(size_t)b * v.np + i] = v.omega[i] + gv;
        }
      }
    }
  }
};
// the A_lo pass: columns [hi cos | hi sin]; stores the partial couplings
template <int BP> struct LoEpi {
  TView v;
  const TCoef* src;
  __device__ void row(uint32_t taddr, int row, int m0, int sp) {
    const int i = m0 + row;
#pragma unroll 1
    for (int b0 = 0; b0 < BP; b0 += 16) {
      float hc[16], hs[16];
      umma::tmem_ld16(taddr + 0 * BP + b0, hc);
      umma::tmem_ld16(taddr + 1 * BP + b0, hs);
      umma::tmem_ld_wait();
      if (i >= v.n) continue;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int b = sp * BP + b0 + j;
        if (b >= v.B) break;
        v.Flo[((size_t)0 * v.bp + b) * v.np + i] = hc[j];
        v.Flo[((size_t)1 * v.bp + b) * v.np + i] = hs[j];
      }
    }
  }
};

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ float block_sum(float v, float* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  float t = 0.f;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q];
  return t;  // valid on thread 0
}

// sum of squared scaled errors of stage 7 (dp45.cu:79-84) -> part[b][blk]
__global__ void k_t_error(TView v, const TCoef* src7, double atol, double rtol, float* part, int nblk) {
  __shared__ float sh[32];
  const int b = blockIdx.y;
  const TCoef& s = src7[b];
  float acc = 0.f;
  if (s.active) {
    const size_t yb = ((size_t)s.base * v.bp + b) * v.np, y7b = ((size_t)(s.base ^ 1) * v.bp + b) * v.np;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.n; i += gridDim.x * blockDim.x) {
      float e = 0.f;
#pragma unroll
      for (int j = 0; j < 7; ++j) e = __fmaf_rn(s.E[j], v.g[((size_t)s.slot[j] * v.bp + b) * v.np + i], e);
      float tol = (float)atol;
      if (rtol != 0.0) {
        float a0 = fabsf(__fmaf_rn((float)v.ph_w[yb + i], P2_1, v.ph_hi[yb + i]));
        float a1 = fabsf(__fmaf_rn((float)v.ph_w[y7b + i], P2_1, v.ph_hi[y7b + i]));
        tol = (float)atol + (float)rtol * fmaxf(a0, a1);
      }
      const float ye = e / tol;
      acc = __fmaf_rn(ye, ye, acc);
    }
  }
  const float t = block_sum(acc, sh);
  if (threadIdx.x == 0) part[(size_t)b * nblk + blockIdx.x] = t;
}

// controller of every trajectory (dp45.cu:109-139); writes the completion flag
__global__ void k_t_decide(TrajG* traj, const TCoef* src7, const float* part, int nblk, int B, int n, int fixed,
                           const float* t_eval, int n_eval, int* done) {
  const int b = threadIdx.x;
  __shared__ int any;
  if (b == 0) any = 0;
  __syncthreads();
  if (b < B) {
    TrajG& T = traj[b];
    if (src7[b].active && T.status == 0) {
      const double h = T.h;
      bool accept = true;
      double factor = 1.0;
      if (!fixed) {
        float ss = 0.f;
        for (int q = 0; q < nblk; ++q) ss += part[(size_t)b * nblk + q];
        const double norm = sqrt((double)ss) / sqrt((double)n);
        if (isnan(norm)) {
          T.status = KURA_ERR_NONFINITE;
        } else {
          factor = (double)(0.9f * exp2f(-0.2f * log2f((float)norm)));
          accept = norm < 1.0;
        }
      }
      if (T.status == 0) {
        if (accept) {
          T.t_last = T.t;
          T.t = T.t + h;
          T.rot_y ^= 1;
          T.rot_g ^= 1;
          T.accepted++;
          if (!fixed) T.h = h * fmin(factor, 10.0);
          int e = T.eval_i;
          while (e < n_eval && T.t >= (double)t_eval[e]) e++;
          T.eval_end = e;
        } else {
          T.rejected++;
          if (factor < 1.0) T.h = h * fmax(factor, 0.2);
          if (!(T.h >= 1e-14 * fmax(1.0, fabs(T.t)))) T.status = KURA_ERR_STEP_UNDERFLOW;
        }
      }
    }
    if (T.status == 0 && !(T.t < T.t1) && T.eval_i >= T.eval_end) T.status = 1;
    if (T.status == 0 || T.eval_i < T.eval_end) atomicOr(&any, 1);
  }
  __syncthreads();
  if (b == 0) *done = any ? 0 : 1;
}

// order parameter at the pending output times of each trajectory: partial sums of
// (cos, sin) of the dense output (dp45.cu:70-76, kuramoto.cu:212-220)
__global__ void k_t_out_partial(TView v, const TrajG* traj, const float* t_eval, float* part, int nblk) {
  __shared__ float sh[32];
  const int b = blockIdx.y;
  const TrajG& T = traj[b];
  const int ncross = min(T.eval_end - T.eval_i, T_MAXC);
  const bool initial = T.need_init != 0;
  if (ncross <= 0 && !initial) return;
  const int nrec = initial ? 1 : ncross;
  const size_t bl = initial ? ((size_t)T.rot_y * v.bp + b) * v.np : ((size_t)(T.rot_y ^ 1) * v.bp + b) * v.np;
  // after the accept, k1 of the step sits in the k7 slot and vice versa
  const int k1s = slot_k7(T.rot_g), k7s = slot_k1(T.rot_g);
  __shared__ float sw[9];  // the record's weights: W[0..6], then the time offset hi and lo
  for (int c = 0; c < nrec; ++c) {
    // the weights in double, once per block (FP64 is a small fraction of this GPU's FP32 rate:
    // computed by every thread they cost more than the record's memory traffic)
    if (threadIdx.x == 0) {
      for (int j = 0; j < 9; ++j) sw[j] = 0.f;
      if (!initial) {
        const double hs = T.t - T.t_last, dl = (double)t_eval[T.eval_i + c] - T.t_last, x = dl / hs;
        for (int j = 0; j < 7; ++j) {
          const double cc = ((P_TAB[j][3] * x + P_TAB[j][2]) * x + P_TAB[j][1]) * x * x + P_TAB[j][0] * x;
          sw[j] = (float)(hs * cc);
        }
        const float mh0 = (float)dl;
        sw[7] = mh0;
        sw[8] = (float)(dl - (double)mh0);
      }
    }
    __syncthreads();
    float W[7];
#pragma unroll
    for (int j = 0; j < 7; ++j) W[j] = sw[j];
    const float mh = sw[7], ml = sw[8];
    float ax = 0.f, ay = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.n; i += gridDim.x * blockDim.x) {
      float gsum = 0.f;
      if (!initial) {
        gsum = __fmaf_rn(W[0], v.g[((size_t)k1s * v.bp + b) * v.np + i], gsum);
        for (int j = 1; j < 6; ++j) gsum = __fmaf_rn(W[j], v.g[((size_t)j * v.bp + b) * v.np + i], gsum);
        gsum = __fmaf_rn(W[6], v.g[((size_t)k7s * v.bp + b) * v.np + i], gsum);
      }
      const float om = v.omega[i];
      const f2 pr = two_prod(om, mh);
      const f2 s1 = two_sum(v.ph_hi[bl + i], pr.hi);
      const f2 s2 = two_sum(s1.hi, gsum);
      const float lo = v.ph_lo[bl + i] + ((s1.lo + s2.lo) + __fmaf_rn(om, ml, pr.lo));
      float sn, cs;
      sincos_pair(s2.hi, lo, &sn, &cs);
      ax += cs;
      ay += sn;
    }
    const float tx = block_sum(ax, sh);
    const float ty = block_sum(ay, sh);
    if (threadIdx.x == 0) {
      part[(((size_t)b * T_MAXC + c) * nblk + blockIdx.x) * 2] = tx;
      part[(((size_t)b * T_MAXC + c) * nblk + blockIdx.x) * 2 + 1] = ty;
    }
  }
}
__global__ void k_t_out_final(TrajG* traj, const float* part, int nblk, int B, int n, float* out_r, int* out_idx,
                              int ring) {
  const int b = threadIdx.x;
  if (b >= B) return;
  TrajG& T = traj[b];
  const bool initial = T.need_init != 0;
  int nrec = initial ? 1 : min(T.eval_end - T.eval_i, T_MAXC);
  if (nrec <= 0) return;
  if (!initial && T.eval_end - T.eval_i > T_MAXC) T.status = KURA_ERR_UNSUPPORTED;
  for (int c = 0; c < nrec && T.out_count < ring; ++c) {
    float X = 0.f, Y = 0.f;
    for (int q = 0; q < nblk; ++q) {
      X += part[(((size_t)b * T_MAXC + c) * nblk + q) * 2];
      Y += part[(((size_t)b * T_MAXC + c) * nblk + q) * 2 + 1];
    }
    const float xn = X / (float)n, yn = Y / (float)n;
    out_r[(size_t)b * ring + T.out_count] = sqrtf(xn * xn + yn * yn);
    out_idx[(size_t)b * ring + T.out_count] = initial ? -1 : T.eval_i;
    T.out_count++;
    if (!initial) T.eval_i++;
  }
  if (initial) T.need_init = 0;
}
__global__ void k_t_clear_k1(TrajG* traj, int B) {
  const int b = threadIdx.x;
  if (b < B) traj[b].need_k1 = 0;
}

// N*A for the volcano rule, exact in BF16 (integers in [-K, K])
__global__ void k_t_volcano_bf16(const uint32_t* __restrict__ bits, int n, int k, int words, int np,
                                 __nv_bfloat16* __restrict__ A, __nv_bfloat16* __restrict__ Alo) {
  for (int i = blockIdx.y; i < np; i += gridDim.y)
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < np; j += gridDim.x * blockDim.x) {
      int kk = 0;
      if (i < n && j < n) {
        for (int wd = 0; wd < words; ++wd) {
          const int m0 = 32 * wd, cnt = min(32, k - m0);
          const uint32_t valid = cnt >= 32 ? 0xffffffffu : ((1u << cnt) - 1u);
          const uint32_t even = 0x55555555u & valid, odd = 0xAAAAAAAAu & valid;
          const uint32_t dis = bits[(size_t)wd * n + i] ^ bits[(size_t)wd * n + j];
          kk += __popc(even) - __popc(odd) - 2 * __popc(dis & even) + 2 * __popc(dis & odd);
        }
      }
      const __nv_bfloat16 hi = __float2bfloat16_rn((float)kk);
      A[(size_t)i * np + j] = hi;
      if (Alo) Alo[(size_t)i * np + j] = __float2bfloat16_rn((float)kk - __bfloat162float(hi));
    }
}
// general adjacency: N*A = hi + lo in BF16
__global__ void k_t_split(const float* __restrict__ adj, int n, int np, float scale, __nv_bfloat16* hi,
                          __nv_bfloat16* lo) {
  for (int i = blockIdx.y; i < np; i += gridDim.y)
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < np; j += gridDim.x * blockDim.x) {
      const float a = (i < n && j < n) ? adj[(size_t)i * n + j] * scale : 0.f;
      const __nv_bfloat16 h = __float2bfloat16_rn(a);
      hi[(size_t)i * np + j] = h;
      lo[(size_t)i * np + j] = __float2bfloat16_rn(a - __bfloat162float(h));
    }
}
__global__ void k_t_adj_out(const __nv_bfloat16* hi, const __nv_bfloat16* lo, int n, int np, float invn, float* adj) {
  for (int i = blockIdx.y; i < n; i += gridDim.y)
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
      float a = __bfloat162float(hi[(size_t)i * np + j]);
      if (lo) a += __bfloat162float(lo[(size_t)i * np + j]);
      adj[(size_t)i * n + j] = __fmul_rn(a, invn);
    }
}

}  // namespace

// ====================================================================== host engine
struct TensorEngine::Impl {
  int n = 0, np = 0, bp = 0, B = 0, K = 0, seed = 1, fixed = 0, dense_level = 0, device = 0;
  double atol = 1e-6, rtol = 0.0;
  cudaStream_t st = nullptr;
  float* omega = nullptr;
  float* ph_hi = nullptr;
  float* ph_lo = nullptr;
  long long* ph_w = nullptr;
  float* g = nullptr;
  __nv_bfloat16* X = nullptr;
  float2* x32 = nullptr;
  __nv_bfloat16* Ahi = nullptr;
  __nv_bfloat16* Alo = nullptr;
  float* Flo = nullptr;
  float* fin_theta = nullptr;
  float* fin_coup = nullptr;
  TrajG* traj = nullptr;
  TCoef* src = nullptr;       // [8][bp]
  float* part = nullptr;      // reductions
  float* t_eval = nullptr;
  float* out_r = nullptr;
  int* out_idx = nullptr;
  int* done = nullptr;
  int* err = nullptr;
  int* any_active = nullptr;  // written by the coefficient kernels; the GEMMs skip when 0
  int* h_done = nullptr;      // pinned
  int ring = 0, n_eval = 0, nblk = 1;
  CUtensorMap tmA, tmAlo, tmX, tmXhi;
  bool has_lo = false, adj_set = false;
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // KURA_TIME_COUPLING=1: event nodes around the six coupling GEMMs of the attempt graph; the
  // durations of the last replay of each batch of replays are summed into the stats
  bool time_gemm = false;
  cudaEvent_t gev[12] = {};
};

static std::string g_terr;
#define TCU(x)                                                               \
  do {                                                                       \
    cudaError_t e_ = (x);                                                    \
    if (e_ != cudaSuccess) {                                                 \
      g_terr = std::string(#x) + ": " + cudaGetErrorString(e_);              \
      return e_ == cudaErrorMemoryAllocation ? KURA_ERR_NOMEM : KURA_ERR_CUDA; \
    }                                                                        \
  } while (0)

const char* TensorEngine::last_error() { return g_terr.c_str(); }

template <typename T> static cudaError_t zalloc(T** p, size_t count) {
  cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
  if (e == cudaSuccess) e = cudaMemset(*p, 0, std::max<size_t>(count, 1) * sizeof(T));
  // the memset runs on the legacy default stream, which does not order with the non-blocking
  // stream a handle may own: wait for it, so that no later copy on that stream lands first
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  return e;
}

TensorEngine::TensorEngine() : d(new Impl) {}
TensorEngine::~TensorEngine() {
  void* ptrs[] = {d->omega, d->ph_hi, d->ph_lo, d->ph_w, d->g, d->X, d->x32, d->Ahi, d->Alo, d->Flo, d->fin_theta,
                  d->fin_coup, d->traj, d->src, d->part, d->t_eval, d->out_r, d->out_idx, d->done, d->err,
                  d->any_active};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (d->h_done) cudaFreeHost(d->h_done);
  if (d->graph) cudaGraphExecDestroy(d->graph);
  if (d->ev0) cudaEventDestroy(d->ev0);
  if (d->ev1) cudaEventDestroy(d->ev1);
  for (cudaEvent_t e : d->gev)
    if (e) cudaEventDestroy(e);
  delete d;
}

int TensorEngine::init(int64_t n, int k, int batch, int seed, double atol, double rtol, int fixed, int dense_level,
                       int device, cudaStream_t st) {
  if (batch < 1 || batch > 128) { g_terr = "tensor engine: batch must be 1..128"; return KURA_ERR_UNSUPPORTED; }
  if (dense_level >= 1) { g_terr = "tensor engine keeps the order parameter only (dense level 0)"; return KURA_ERR_UNSUPPORTED; }
  if (n < 1 || n > (1LL << 20)) { g_terr = "tensor engine: n must be in [1, 2^20]"; return KURA_ERR_UNSUPPORTED; }
  Impl& I = *d;
  I.n = (int)n; I.K = k; I.B = batch; I.seed = seed; I.atol = atol; I.rtol = rtol; I.fixed = fixed;
  I.dense_level = dense_level; I.device = device; I.st = st;
  I.np = (I.n + 255) / 256 * 256;  // work units of two 128-row tiles
  I.bp = 16;
  while (I.bp < batch) I.bp *= 2;
  const size_t np = I.np, bp = I.bp;
  I.nblk = std::min(1024, (I.n + T_RBLK - 1) / T_RBLK);
  TCU(zalloc(&I.omega, np));
  TCU(zalloc(&I.ph_hi, 2 * bp * np));
  TCU(zalloc(&I.ph_lo, 2 * bp * np));
  TCU(zalloc(&I.ph_w, 2 * bp * np));
  TCU(zalloc(&I.g, 7 * bp * np));
  TCU(zalloc(&I.X, 4 * bp * np));
  TCU(zalloc(&I.x32, bp * np));
  TCU(zalloc(&I.Ahi, np * np));
  TCU(zalloc(&I.fin_theta, bp * np));
  TCU(zalloc(&I.fin_coup, 2 * bp * np));
  TCU(zalloc(&I.traj, bp));
  TCU(zalloc(&I.src, 8 * bp));
  TCU(zalloc(&I.part, (size_t)bp * T_MAXC * I.nblk * 2));
  TCU(zalloc(&I.done, 4));
  TCU(zalloc(&I.any_active, 16));
  TCU(zalloc(&I.err, 4));
  TCU(cudaHostAlloc((void**)&I.h_done, sizeof(int), cudaHostAllocDefault));
  TCU(cudaEventCreate(&I.ev0));
  TCU(cudaEventCreate(&I.ev1));
  const char* tg = getenv("KURA_TIME_COUPLING");
  I.time_gemm = tg && atoi(tg) != 0;
  if (I.time_gemm)
    for (cudaEvent_t& e : I.gev) TCU(cudaEventCreate(&e));
  // X is [4 bp][np]: a work unit's column block is 4 * x_bph(bp) rows (its hi + lo columns),
  // of which the A_lo pass reads the first half
  if (make_tmap_bf16(&I.tmA, I.Ahi, np, np, TG_BM, TE_BK) ||
      make_tmap_bf16(&I.tmX, I.X, np, 4 * bp, 4 * x_bph(I.bp), TE_BK) ||
      make_tmap_bf16(&I.tmXhi, I.X, np, 4 * bp, 2 * x_bph(I.bp), TE_BK)) {
    g_terr = "cuTensorMapEncodeTiled failed";
    return KURA_ERR_CUDA;
  }
  return KURA_OK;
}

size_t TensorEngine::memory_required(int64_t n, int batch) {
  size_t np = ((size_t)n + 255) / 256 * 256, bp = 16;
  while ((int)bp < batch) bp *= 2;
  return np * np * 2 + np * bp * (2 * 16 + 7 * 4 + 4 * 2 + 8 + 4 + 8) + np * 4;
}

int TensorEngine::set_frequencies(const float* omega) {
  TCU(cudaMemcpyAsync(d->omega, omega, sizeof(float) * d->n, cudaMemcpyHostToDevice, d->st));
  TCU(cudaStreamSynchronize(d->st));
  return KURA_OK;
}

int TensorEngine::generate_adjacency() {
  Impl& I = *d;
  const int words = (I.K + 31) / 32;
  uint32_t* bits = nullptr;
  if (words > 0) {
    TCU(cudaMalloc((void**)&bits, sizeof(uint32_t) * (size_t)words * I.n));
    TCU(launch_volcano_words(I.seed, I.n, I.K, words, bits, I.st));
  }
  // N*A_ij is an integer in [-K, K]: exact in BF16 for K <= 256, else exact as hi + lo
  const bool need_lo = I.K > 256;
  if (need_lo && !I.Alo) TCU(zalloc(&I.Alo, (size_t)I.np * I.np));
  if (need_lo && !I.Flo) TCU(zalloc(&I.Flo, (size_t)2 * I.bp * I.np));
  dim3 grid((unsigned)std::min((I.np + 255) / 256, 64), (unsigned)std::min(I.np, 65535));
  k_t_volcano_bf16<<<grid, 256, 0, I.st>>>(bits, I.n, I.K, words, I.np, I.Ahi, need_lo ? I.Alo : nullptr);
  TCU(cudaGetLastError());
  TCU(cudaStreamSynchronize(I.st));
  if (bits) cudaFree(bits);
  if (need_lo && make_tmap_bf16(&I.tmAlo, I.Alo, I.np, I.np, TG_BM, TE_BK)) {
    g_terr = "cuTensorMapEncodeTiled failed";
    return KURA_ERR_CUDA;
  }
  I.has_lo = need_lo;
  I.adj_set = true;
  return KURA_OK;
}

int TensorEngine::set_adjacency(const float* adj_host) {
  Impl& I = *d;
  float* dadj = nullptr;
  TCU(cudaMalloc((void**)&dadj, sizeof(float) * (size_t)I.n * I.n));
  TCU(cudaMemcpyAsync(dadj, adj_host, sizeof(float) * (size_t)I.n * I.n, cudaMemcpyHostToDevice, I.st));
  if (!I.Alo) TCU(zalloc(&I.Alo, (size_t)I.np * I.np));
  if (!I.Flo) TCU(zalloc(&I.Flo, (size_t)2 * I.bp * I.np));
  dim3 grid((unsigned)std::min((I.np + 255) / 256, 64), (unsigned)std::min(I.np, 65535));
  k_t_split<<<grid, 256, 0, I.st>>>(dadj, I.n, I.np, (float)I.n, I.Ahi, I.Alo);
  TCU(cudaGetLastError());
  TCU(cudaStreamSynchronize(I.st));
  cudaFree(dadj);
  if (make_tmap_bf16(&I.tmAlo, I.Alo, I.np, I.np, TG_BM, TE_BK)) {
    g_terr = "cuTensorMapEncodeTiled failed";
    return KURA_ERR_CUDA;
  }
  I.has_lo = true;
  I.adj_set = true;
  return KURA_OK;
}

int TensorEngine::get_adjacency(float* adj_host) {
  Impl& I = *d;
  float* dadj = nullptr;
  TCU(cudaMalloc((void**)&dadj, sizeof(float) * (size_t)I.n * I.n));
  dim3 grid((unsigned)std::min((I.n + 255) / 256, 64), (unsigned)std::min(I.n, 65535));
  k_t_adj_out<<<grid, 256, 0, I.st>>>(I.Ahi, I.has_lo ? I.Alo : nullptr, I.n, I.np, 1.0f / (float)I.n, dadj);
  TCU(cudaGetLastError());
  TCU(cudaMemcpyAsync(adj_host, dadj, sizeof(float) * (size_t)I.n * I.n, cudaMemcpyDeviceToHost, I.st));
  TCU(cudaStreamSynchronize(I.st));
  cudaFree(dadj);
  return KURA_OK;
}

int TensorEngine::set_state(int b, const float* theta_dev, const TrajG& T) {
  Impl& I = *d;
  const size_t off = (size_t)b * I.np;  // phase buffer 0
  TCU(launch_init_state(theta_dev, I.n, I.np, I.ph_hi + off, I.ph_lo + off, I.ph_w + off, I.st));
  TCU(cudaMemcpyAsync(I.traj + b, &T, sizeof(TrajG), cudaMemcpyHostToDevice, I.st));
  TCU(cudaStreamSynchronize(I.st));
  return KURA_OK;
}
float* TensorEngine::staging(int b) { return d->fin_theta + (size_t)b * d->np; }

int TensorEngine::set_horizon(const std::vector<float>& t_eval, int ring, std::vector<TrajG>& traj) {
  Impl& I = *d;
  I.n_eval = (int)t_eval.size();
  if (I.t_eval) cudaFree(I.t_eval);
  if (I.out_r) cudaFree(I.out_r);
  if (I.out_idx) cudaFree(I.out_idx);
  I.t_eval = nullptr; I.out_r = nullptr; I.out_idx = nullptr;
  TCU(zalloc(&I.t_eval, t_eval.size()));
  if (!t_eval.empty())
    TCU(cudaMemcpyAsync(I.t_eval, t_eval.data(), sizeof(float) * t_eval.size(), cudaMemcpyHostToDevice, I.st));
  I.ring = ring;
  TCU(zalloc(&I.out_r, (size_t)I.bp * ring));
  TCU(zalloc(&I.out_idx, (size_t)I.bp * ring));
  TCU(cudaMemcpyAsync(I.traj, traj.data(), sizeof(TrajG) * I.B, cudaMemcpyHostToDevice, I.st));
  TCU(cudaStreamSynchronize(I.st));
  if (I.graph) {
    cudaGraphExecDestroy(I.graph);
    I.graph = nullptr;
  }
  return KURA_OK;
}

template <int NCOL>
static cudaError_t launch_gemm(TensorEngine::Impl& I, const TCoef* src, int mode, const int* run_flag) {
  TView v{I.n, I.np, I.bp, I.B, mode, I.omega, I.ph_hi, I.ph_lo, I.ph_w, I.g, I.X, I.x32, I.fin_theta, I.fin_coup,
          I.Flo};
  constexpr int BP = NCOL / 4;  // trajectories per work unit
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, I.device);
  const int mtiles = I.np / (2 * TG_BM), ktiles = I.np / TE_BK;  // groups of two row tiles
  const int nsplit = I.bp / BP, xstride = 4 * BP;
  const int grid = std::min(mtiles * nsplit, sms);
  // Units of two row tiles fill whole waves of the grid; the rest run as one-tile units, when
  // that shortens the last wave (in unit times: a one-tile unit is half of a two-tile one)
  int big = mtiles;
  {
    const int full = (mtiles * nsplit) / grid;
    const int b = full * grid / nsplit;
    const int tail = (mtiles - b) * 2 * nsplit;
    const double t_split = full + 0.5 * ((tail + grid - 1) / grid);
    const double t_big = (mtiles * nsplit + grid - 1) / grid;
    if (b < mtiles && t_split < t_big) big = b;
  }
  const unsigned long long limit = 20000000000ull;
  if (I.has_lo) {
    auto kl = k_tensor_gemm<NCOL / 2, LoEpi<BP>, 2, TE_BK>;
    cudaFuncSetAttribute(kl, cudaFuncAttributeMaxDynamicSharedMemorySize, TGCfg<NCOL / 2, 2, TE_BK>::SMEM);
    LoEpi<BP> le{v, src};
    kl<<<grid, TG_THREADS, TGCfg<NCOL / 2, 2, TE_BK>::SMEM, I.st>>>(I.tmAlo, I.tmXhi, mtiles, big, ktiles, nsplit, xstride, le,
                                                             I.err, limit, run_flag);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  auto k = k_tensor_gemm<NCOL, KuraEpi<BP>, 2, TE_BK>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, TGCfg<NCOL, 2, TE_BK>::SMEM);
  KuraEpi<BP> ep{v, src, 1.0f / (float)I.n, I.has_lo ? 1 : 0};
  k<<<grid, TG_THREADS, TGCfg<NCOL, 2, TE_BK>::SMEM, I.st>>>(I.tmA, I.tmX, mtiles, big, ktiles, nsplit, xstride, ep, I.err, limit,
                                                   run_flag);
  return cudaGetLastError();
}

// one unit holds up to 64 trajectories (NCOL = 256: two accumulators fit in TMEM); a batch
// of 128 is two column blocks per row tile
static cudaError_t gemm(TensorEngine::Impl& I, const TCoef* src, int mode, const int* run_flag) {
  switch (I.bp) {
    case 16: return launch_gemm<64>(I, src, mode, run_flag);
    case 32: return launch_gemm<128>(I, src, mode, run_flag);
    default: return launch_gemm<256>(I, src, mode, run_flag);
  }
}

static cudaError_t coupling(TensorEngine::Impl& I, const TCoef* src, int mode, float* fin_theta, const int* run_flag,
                            int timed = -1) {
  TView v{I.n, I.np, I.bp, I.B, mode, I.omega, I.ph_hi, I.ph_lo, I.ph_w, I.g, I.X, I.x32, fin_theta, I.fin_coup,
          I.Flo};
  dim3 grid((unsigned)((I.n + 255) / 256), (unsigned)I.B);
  k_t_stage<<<grid, 256, 0, I.st>>>(v, src);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const bool tm = I.time_gemm && timed >= 0;
  if (tm && (e = cudaEventRecordWithFlags(I.gev[2 * timed], I.st, cudaEventRecordExternal)) != cudaSuccess) return e;
  if ((e = gemm(I, src, mode, run_flag)) != cudaSuccess) return e;
  if (tm) e = cudaEventRecordWithFlags(I.gev[2 * timed + 1], I.st, cudaEventRecordExternal);
  return e;
}

// one attempt of every trajectory, then its outputs
static cudaError_t attempt(TensorEngine::Impl& I) {
  TView v{I.n, I.np, I.bp, I.B, 0, I.omega, I.ph_hi, I.ph_lo, I.ph_w, I.g, I.X, I.x32, nullptr, I.fin_coup, I.Flo};
  k_t_coef<<<1, 512, 0, I.st>>>(I.traj, I.src, I.B, I.bp, I.fixed, I.any_active);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  for (int s = 2; s <= 7; ++s) {
    e = coupling(I, I.src + (size_t)(s - 1) * I.bp, 0, nullptr, I.any_active + 1, s - 2);
    if (e != cudaSuccess) return e;
  }
  if (!I.fixed) {
    k_t_error<<<dim3((unsigned)I.nblk, (unsigned)I.B), T_RBLK, 0, I.st>>>(v, I.src + 6 * (size_t)I.bp, I.atol, I.rtol,
                                                                        I.part, I.nblk);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  k_t_decide<<<1, 128, 0, I.st>>>(I.traj, I.src + 6 * (size_t)I.bp, I.part, I.nblk, I.B, I.n, I.fixed, I.t_eval,
                                  I.n_eval, I.done);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_t_out_partial<<<dim3((unsigned)I.nblk, (unsigned)I.B), T_RBLK, 0, I.st>>>(v, I.traj, I.t_eval, I.part, I.nblk);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_t_out_final<<<1, 128, 0, I.st>>>(I.traj, I.part, I.nblk, I.B, I.n, I.out_r, I.out_idx, I.ring);
  return cudaGetLastError();
}

int TensorEngine::run(std::vector<TrajG>& traj, kura_stats& stats, long long max_replays) {
  Impl& I = *d;
  if (!I.adj_set) { g_terr = "adjacency not set"; return KURA_ERR_INVALID; }
  TCU(cudaMemsetAsync(I.err, 0, sizeof(int), I.st));
  TCU(cudaEventRecord(I.ev0, I.st));
  // first slope of the run and the record at t0
  {
    TView v{I.n, I.np, I.bp, I.B, 0, I.omega, I.ph_hi, I.ph_lo, I.ph_w, I.g, I.X, I.x32, nullptr, I.fin_coup, I.Flo};
    k_t_coef<<<1, 512, 0, I.st>>>(I.traj, I.src, I.B, I.bp, I.fixed, I.any_active);
    TCU(cudaGetLastError());
    TCU(coupling(I, I.src, 0, nullptr, I.any_active));
    k_t_clear_k1<<<1, 128, 0, I.st>>>(I.traj, I.B);
    k_t_out_partial<<<dim3((unsigned)I.nblk, (unsigned)I.B), T_RBLK, 0, I.st>>>(v, I.traj, I.t_eval, I.part, I.nblk);
    k_t_out_final<<<1, 128, 0, I.st>>>(I.traj, I.part, I.nblk, I.B, I.n, I.out_r, I.out_idx, I.ring);
    TCU(cudaGetLastError());
  }
  if (!I.graph) {
    cudaGraph_t gr;
    TCU(cudaStreamBeginCapture(I.st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = attempt(I);
    cudaError_t e2 = cudaStreamEndCapture(I.st, &gr);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      g_terr = std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2);
      return KURA_ERR_CUDA;
    }
    TCU(cudaGraphInstantiate(&I.graph, gr, 0));
    cudaGraphDestroy(gr);
  }
  long long launches = 0;
  while (true) {
    for (int r = 0; r < 4; ++r) {
      TCU(cudaGraphLaunch(I.graph, I.st));
      launches++;
    }
    TCU(cudaMemcpyAsync(I.h_done, I.done, sizeof(int), cudaMemcpyDeviceToHost, I.st));
    TCU(cudaStreamSynchronize(I.st));
    int errv = 0;
    TCU(cudaMemcpy(&errv, I.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (errv) { g_terr = "tensor GEMM aborted (wait time limit)"; return KURA_ERR_BARRIER_TIMEOUT; }
    if (*I.h_done) break;
    if (I.time_gemm) {  // every replay of this batch stepped some trajectory: sample the last one
      for (int q = 0; q < 6; ++q) {
        float gm = 0.f;
        if (cudaEventElapsedTime(&gm, I.gev[2 * q], I.gev[2 * q + 1]) == cudaSuccess) {
          stats.coupling_ms += gm;
          stats.coupling_launches++;
        }
      }
    }
    if (max_replays > 0 && launches >= max_replays) break;
  }
  TCU(cudaEventRecord(I.ev1, I.st));
  TCU(cudaMemcpyAsync(traj.data(), I.traj, sizeof(TrajG) * I.B, cudaMemcpyDeviceToHost, I.st));
  TCU(cudaStreamSynchronize(I.st));
  float ms = 0;
  TCU(cudaEventElapsedTime(&ms, I.ev0, I.ev1));
  stats.kernel_ms += ms;
  stats.launches += launches;
  return KURA_OK;
}

int TensorEngine::read_order(int b, int count, float* r, int* idx) {
  TCU(cudaMemcpy(r, d->out_r + (size_t)b * d->ring, sizeof(float) * count, cudaMemcpyDeviceToHost));
  if (idx) TCU(cudaMemcpy(idx, d->out_idx + (size_t)b * d->ring, sizeof(int) * count, cudaMemcpyDeviceToHost));
  return KURA_OK;
}

int TensorEngine::get_state(int b, int rot_y, float* theta) {
  Impl& I = *d;
  const size_t off = ((size_t)rot_y * I.bp + b) * I.np;
  float* tmp = I.fin_theta + (size_t)b * I.np;
  TCU(launch_unwrap(I.ph_hi + off, I.ph_lo + off, I.ph_w + off, I.n, tmp, I.st));
  TCU(cudaMemcpyAsync(theta, tmp, sizeof(float) * I.n, cudaMemcpyDeviceToHost, I.st));
  TCU(cudaStreamSynchronize(I.st));
  return KURA_OK;
}

// mode 1: end-of-run record (theta at the last output time, couplings); mode 2: RHS
int TensorEngine::evaluate(int mode, int b, float* theta_out, float* coup_out) {
  Impl& I = *d;
  k_t_coef_final<<<1, 128, 0, I.st>>>(I.traj, I.src + 7 * (size_t)I.bp, I.B, I.t_eval, I.n_eval, mode == 1);
  TCU(cudaGetLastError());
  TCU(coupling(I, I.src + 7 * (size_t)I.bp, mode, I.fin_theta, nullptr));
  TCU(cudaStreamSynchronize(I.st));
  std::vector<float> tmp(2 * (size_t)I.n);
  if (theta_out)
    TCU(cudaMemcpy(theta_out, I.fin_theta + (size_t)b * I.np, sizeof(float) * I.n, cudaMemcpyDeviceToHost));
  if (coup_out)
    TCU(cudaMemcpy(coup_out, I.fin_coup + (size_t)b * I.np * 2, sizeof(float) * 2 * I.n, cudaMemcpyDeviceToHost));
  int errv = 0;
  TCU(cudaMemcpy(&errv, I.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (errv) { g_terr = "tensor GEMM aborted (wait time limit)"; return KURA_ERR_BARRIER_TIMEOUT; }
  return KURA_OK;
}

int TensorEngine::sync_traj(std::vector<TrajG>& traj, bool to_device) {
  Impl& I = *d;
  // on the engine's stream: the legacy-stream cudaMemcpy does not order with it
  if (to_device)
    TCU(cudaMemcpyAsync(I.traj, traj.data(), sizeof(TrajG) * I.B, cudaMemcpyHostToDevice, I.st));
  else
    TCU(cudaMemcpyAsync(traj.data(), I.traj, sizeof(TrajG) * I.B, cudaMemcpyDeviceToHost, I.st));
  TCU(cudaStreamSynchronize(I.st));
  return KURA_OK;
}

}  // namespace kura
