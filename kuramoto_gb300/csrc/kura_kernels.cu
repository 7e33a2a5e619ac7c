// kura_kernels.cu -- sm_103a kernels of the Kuramoto DP45 integrator.
//
// One persistent cooperative kernel runs the whole adaptive integration
// (dp45_run, dp45.cu:148-164): the six stage evaluations of each attempt, the
// error norm, the accept/reject controller, the dense output at every t_eval
// crossing and the order parameter, with the step size kept on the device.  The
// host launches it once per run (more often only when an output ring fills).
//
// Work split: CTA g owns rows [g*rows, (g+1)*rows) of the network for every
// trajectory of the batch.  One grid barrier per coupling evaluation exchanges
// what the other CTAs need:
//   * dense coupling (kuramoto.cu:110-115): every CTA publishes (cos, sin) of its
//     rows; after the barrier it streams its rows of A once, computing A*cos and
//     A*sin together (the reference reads A twice, with two GEMV calls);
//   * volcano coupling (-A, kuramoto.cu:62-101): every CTA publishes its partial
//     projections sum_n u_mn (cos, sin); after the barrier each CTA sums the
//     partials in a fixed order and back-projects for its rows.  The factor bits
//     come from Philox4x32-10 at stream element m*N+n and are kept in shared memory
//     for the CTA's rows, so neither A nor the factor is ever stored in HBM.
// Reductions use fixed orders, so every CTA reaches the same controller
// decisions and results do not depend on timing.
//
// Phases are held as wrapped float pairs (hi in [-pi, pi], lo, winding count),
// the frequency term omega*h of each stage is added with error-free products,
// and only the coupling part g = k - omega of each slope is stored.  This keeps
// the phase accumulation at about double-float accuracy without FP64 arithmetic
// in the per-oscillator loops (GB300's FP64 rate is a small fraction of FP32).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include "kura.h"
#include "kura_kernels.cuh"
#include "kura_device.cuh"

namespace kura {

// ------------------------------------------------------------------ memory helpers
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// streamed read of the adjacency: no L1 allocation, default L2 policy (a small A stays L2-resident)
__device__ __forceinline__ uint2 ld_stream_u2(const int8_t* p) {
  uint2 v;
  asm volatile("ld.global.nc.L1::no_allocate.v2.u32 {%0,%1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
  return v;
}
__device__ __forceinline__ uint4 ld_stream_u4(const int8_t* p) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}
// signed byte j of w as an exact float: byte ^ 0x80 placed under the exponent of 2^23
// (0x4B000000), minus 2^23 + 128
__device__ __forceinline__ float i8_to_f(uint32_t w_biased, int j) {
  return __int_as_float((int)__byte_perm(w_biased, 0x4B000000u, 0x7540u + (unsigned)j)) - 8388736.0f;
}
// Packed FP32 pairs (sm_100 and later): one instruction, each half rounded as the scalar
// operation.  (a.lo*b.lo + c.lo, a.hi*b.hi + c.hi):
__device__ __forceinline__ unsigned long long ffma2(unsigned long long a, unsigned long long b,
                                                    unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ float2 unpack_f2(unsigned long long v) {
  float2 r;
  asm("mov.b64 {%0,%1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
// byte j of w0 and of w1 (biased by 0x80, as for i8_to_f) as the exact float pair
// (lo: w0, hi: w1): both placed under the exponent of 2^23, then 2^23 + 128 subtracted from
// the pair in one packed add
__device__ __forceinline__ unsigned long long i8_pair_to_f2(uint32_t w0, uint32_t w1, int j) {
  const uint32_t lo = __byte_perm(w0, 0x4B000000u, 0x7540u + (unsigned)j);
  const uint32_t hi = __byte_perm(w1, 0x4B000000u, 0x7540u + (unsigned)j);
  const unsigned long long bias = 0xCB000080CB000080ull;  // (-8388736.0f, -8388736.0f)
  unsigned long long d;
  asm("{\n\t.reg .b64 t;\n\tmov.b64 t, {%1,%2};\n\tadd.rn.f32x2 %0, t, %3;\n\t}"
      : "=l"(d) : "r"(lo), "r"(hi), "l"(bias));
  return d;
}
// 16 bytes global -> shared without a register round trip (L2 only); src_bytes 0 zero-fills
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc, int src_bytes) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(gsrc), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ float4 ld_stream4(const float* p) {
  float4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p));
  return v;
}

// ------------------------------------------------------------------ per-evaluation source
// What one coupling evaluation integrates for one trajectory:
//   theta = phase[base] + omega*(m_hi + m_lo) + sum_j W[j] * g[slot[j]]
struct __align__(16) SrcB {
  float W[7];  // 16-byte aligned: read as two float4 (the second ends with E[0])
  float E[7];      // error weights h*e_j (error phase)
  float m_hi, m_lo;
  int slot[7];     // physical g slot of logical k_1..k_7
  int base;        // physical phase buffer
  int gout;        // g slot receiving c*(sin*Fc - cos*Fs), -1: none
  int active;
  int store_y7;    // keep the stage value (the candidate y) in buffer base^1
  int rec;         // output record (r always; theta / couplings by dense level)
  int oslot, oidx;
  int nW;
};

__device__ __forceinline__ int slot_k1(int rot_g) { return rot_g ? 6 : 0; }
__device__ __forceinline__ int slot_k7(int rot_g) { return rot_g ? 0 : 6; }

__host__ __device__ constexpr int pw_of(int coup, int kmax) { return coup == KURA_COUPLING_VOLCANO ? 2 * kmax + 2 : 2; }
__host__ __device__ constexpr int align16(int b) { return (b + 15) & ~15; }

// shared-memory layout (bytes), also used by the host to size the launch
__host__ __device__ inline void smem_layout(int coup, int bmax, int kmax, int rows, int xs_smem, int* off,
                                            int* total) {
  int pw = pw_of(coup, kmax);
  int o = 0;
  off[0] = o; o += align16(bmax * (int)sizeof(TrajG));
  off[1] = o; o += align16(7 * bmax * (int)sizeof(SrcB));  // [0]: current source; [1..6]: stages 2..7
  off[2] = o; o += align16(KW * bmax * pw * 4);          // red
  off[3] = o; o += align16(bmax * pw * 4);               // rsum
  int sl = 2 * KT > bmax * pw ? 2 * KT : bmax * pw;
  off[4] = o; o += align16(sl * 4);                      // slice
  off[5] = o; o += align16(16 * 4);                      // flags
  off[6] = o; o += align16(coup == KURA_COUPLING_VOLCANO ? rows * 4 : 0);   // factor bits
  // x tile; the int8 product's holds (cos, cos, sin, sin) per column and one such float4 of
  // padding per 16 columns for one trajectory, (cos, sin) and two pairs of padding for a batch
  off[7] = o; o += align16(coup == KURA_COUPLING_VOLCANO ? 0
                           : coup == COUP_DENSE_I8 ? (bmax == 1 ? (CT_I8 / 16) * I8_CHUNK4 * 16
                                                                : bmax * (CT / 16) * I8_CHUNK * 8)
                                                   : bmax * ((bmax == 1 ? CT_F1 : CT) / 4) * F_CHUNK * 8);
  // f3 (volcano); for K <= 8 it also holds the table of sum_m +-f3_m over all sign patterns
  off[8] = o; o += align16(coup == KURA_COUPLING_VOLCANO ? (bmax * 2 * kmax * 4 + bmax * 256 * 8) : bmax * 2 * kmax * 4);
  // own (cos, sin) (volcano); the ring of A chunks in flight (dense float, int8 of one trajectory)
  off[9] = o; o += align16(coup == KURA_COUPLING_VOLCANO && xs_smem ? bmax * rows * 8
                           : coup == KURA_COUPLING_DENSE ? KW * A_STAGES * A_ROWS * 32 * 16
                           : coup == COUP_DENSE_I8 && bmax == 1 ? KW * I8_SLOTS * 32 * 16 : 0);
  *total = o;
}

// Warp reduce-scatter of 16 values per lane: four butterfly levels each halve the
// values a lane keeps (8 + 4 + 2 + 1 shuffles), a fifth adds the pair.  Afterwards
// lane l holds, in v[0], the warp total of value index
// 8*bit4(l) + 4*bit3(l) + 2*bit2(l) + bit1(l) (lanes l and l^1 hold the same total).
__device__ __forceinline__ void warp_reduce_scatter16(float (&v)[16], int lane) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const bool up = lane & 16;
    float send = up ? v[j] : v[j + 8];
    float keep = up ? v[j + 8] : v[j];
    v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const bool up = lane & 8;
    float send = up ? v[j] : v[j + 4];
    float keep = up ? v[j + 4] : v[j];
    v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const bool up = lane & 4;
    float send = up ? v[j] : v[j + 2];
    float keep = up ? v[j + 2] : v[j];
    v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  {
    const bool up = lane & 2;
    float send = up ? v[0] : v[1];
    float keep = up ? v[1] : v[0];
    v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
  }
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
}
__device__ __forceinline__ int scatter16_index(int lane) {
  return ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
}

template <int COUP, int BMAX, int KMAX>
struct Engine {
  static constexpr int PW = pw_of(COUP, KMAX);
  // rows per warp and pass of the dense coupling: each staged x value is reused RG times
  static constexpr int RG = A_ROWS;

  const KParams& p;
  TrajG* tr;
  SrcB* sb;       // the source the next coupling evaluation integrates
  SrcB* sb_base;  // [0]: general source; [1..6]: the six stages of the current attempt
  float* red;
  float* rsum;
  float* slice;
  int* flag;
  uint32_t* ubits;
  float2* xt;
  float* f3;
  float2* xs;   // (cos, sin) of the CTA's rows, [b][rows]: shared memory, or the CTA's part of xbuf
  float4* ring;  // [warp][A_STAGES][A_ROWS][lane] (dense float coupling)
  int G, gi, tid, lane, warp, r0, r1, B;
  unsigned target;
  int nbar, xpar;

  __device__ Engine(const KParams& pp, unsigned char* smem) : p(pp) {
    int off[10], total;
    smem_layout(COUP, BMAX, KMAX, pp.rows, pp.xs_smem, off, &total);
    tr = (TrajG*)(smem + off[0]);
    sb_base = (SrcB*)(smem + off[1]);
    sb = sb_base;
    red = (float*)(smem + off[2]);
    rsum = (float*)(smem + off[3]);
    slice = (float*)(smem + off[4]);
    flag = (int*)(smem + off[5]);
    ubits = (uint32_t*)(smem + off[6]);
    xt = (float2*)(smem + off[7]);
    f3 = (float*)(smem + off[8]);
    G = gridDim.x;
    gi = blockIdx.x;
    tid = threadIdx.x;
    lane = tid & 31;
    warp = tid >> 5;
    r0 = min(p.n, gi * p.rows);
    r1 = min(p.n, r0 + p.rows);
    B = p.batch;
    target = 0;
    nbar = 0;
    xpar = 0;
    xs = pp.xs_smem ? (float2*)(smem + off[9]) : nullptr;
    ring = (float4*)(smem + off[9]);  // the dense products' chunks of A in flight
  }

  // (cos, sin) of row i of trajectory b for the volcano coupling (own rows only)
  __device__ __forceinline__ float2* xrow(int b) {
    return xs ? xs + (size_t)b * p.rows - r0 : p.xbuf + (size_t)b * p.ld;
  }

  // Thread-to-work mapping of the elementwise phases.  With few rows per CTA (latency
  // bound) each trajectory of the batch gets its own group of KW/B warps, so the
  // trajectories proceed side by side; with many rows (throughput bound) all warps
  // sweep one trajectory after the other.  Returns the trajectory range [b0, b1) of
  // this thread and its row offset / stride.
  __device__ __forceinline__ bool all_warps_mode() const { return r1 - r0 >= 1024; }
  __device__ __forceinline__ void work_map(int& b0, int& b1, int& lt, int& gt) const {
    if (all_warps_mode()) {
      b0 = 0; b1 = B; lt = tid; gt = KT;
    } else {
      const int nwb = KW / B;
      b0 = warp / nwb;
      b1 = b0 < B ? b0 + 1 : b0;
      lt = (warp - b0 * nwb) * 32 + lane;
      gt = nwb * 32;
    }
  }

  // Grid barrier with a time limit.  Returns false (on every thread) when the
  // launch is being abandoned: this CTA timed out or another CTA flagged an error.
  __device__ bool grid_sync() {
    __syncthreads();
    target += (unsigned)G;
    if (tid == 0) {
      __threadfence();
      red_release_add(p.bar, 1u);
      unsigned long long t0 = global_ns();
      int abort = 0;
      unsigned spins = 0;
      while (true) {
        unsigned v = ld_acquire_u32(p.bar);
        if ((int)(v - (target + p.bar_extra)) >= 0) break;
        if (*(volatile int*)p.err != 0) { abort = 1; break; }
        if ((++spins & 63u) == 0 && global_ns() - t0 > p.timeout_ns) {
          atomicCAS(p.err, 0, KURA_ERR_BARRIER_TIMEOUT);
          abort = 1;
          break;
        }
      }
      __threadfence();
      flag[0] = abort;
    }
    __syncthreads();
    nbar++;
    return flag[0] == 0;
  }

  __device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
  }

  // red[warp][b][0..npw) summed over warps -> part[par][gi][b][0..npw)
  __device__ void publish_partials(int npw) {
    __syncthreads();
    int par = nbar & 1;
    const int nwb = KW / B;
    const bool allw = all_warps_mode();
    for (int v = tid; v < B * npw; v += KT) {
      int b = v / npw, w = v - b * npw;
      float s = 0.f;
      const int q0 = allw ? 0 : b * nwb, q1 = allw ? KW : (b + 1) * nwb;
      for (int q = q0; q < q1; ++q) s += red[(q * BMAX + b) * PW + w];
      p.part[((size_t)(par * G + gi) * B + b) * PW_MAX + w] = s;
    }
  }
  // part[par][*][b][w] summed over CTAs in a fixed order -> rsum[b*PW + w].  The
  // CTAs are split into slices that threads sum in parallel; each thread issues its
  // loads 16 at a time so their latencies overlap.
  __device__ void gather_partials(int npw) {
    const int par = (nbar - 1) & 1;  // the parity published before the barrier just passed
    const int NV = B * npw;
    // slices of at most 16 CTAs where the slice buffer (2 KT values for up to 8
    // trajectories) allows, so that every thread needs one round of loads; the slicing does
    // not depend on the batch size, so a trajectory's sums (and so its whole integration)
    // are the same bits whether it runs alone or inside a batch
    int S = 2 * KT / (8 * npw);
    if (S < 1) S = 1;
    if (S > (G + 15) / 16) S = (G + 15) / 16;
    const size_t stride = (size_t)B * PW_MAX;
    for (int t = tid; t < S * NV; t += KT) {
      int v = t % NV, sl = t / NV;
      int b = v / npw, w = v - b * npw;
      int g0 = (int)((long long)sl * G / S), g1 = (int)((long long)(sl + 1) * G / S);
      const float* src = p.part + ((size_t)par * G * B + b) * PW_MAX + w;
      float s = 0.f;
      for (int g = g0; g < g1; g += 16) {
        float v16[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) v16[u] = (g + u < g1) ? __ldcg(src + (size_t)(g + u) * stride) : 0.f;
#pragma unroll
        for (int u = 0; u < 16; ++u) s += v16[u];
      }
      slice[sl * NV + v] = s;
    }
    __syncthreads();
    for (int v = tid; v < NV; v += KT) {
      float s = 0.f;
      for (int sl = 0; sl < S; ++sl) s += slice[sl * NV + v];
      rsum[(v / npw) * PW + (v % npw)] = s;
    }
    __syncthreads();
  }

  // ---- epilogue of one row: slope, couplings, RHS output
  __device__ __forceinline__ void epilogue(int b, int i, float Fc, float Fs, float cs, float sn) {
    const SrcB& s = sb[b];
    float gval = tr[b].c1 * (sn * Fc - cs * Fs);
    if (s.gout >= 0) p.g[((size_t)s.gout * B + b) * p.ld + i] = gval;
    if (s.rec) {
      if (p.mode == MODE_INTEGRATE) {
        if (p.dense_level >= 2) {
          float* dst = p.out_coup + ((size_t)b * p.ring + s.oslot) * 2 * p.ld;
          dst[2 * i] = Fc;
          dst[2 * i + 1] = Fs;
        }
      } else {
        float* dst = p.fin_coup + (size_t)b * 2 * p.ld;
        dst[2 * i] = Fc;
        dst[2 * i + 1] = Fs;
        if (p.mode == MODE_RHS) p.fin_theta[(size_t)b * p.ld + i] = p.omega[i] + gval;
      }
    }
  }

  // ---- one coupling evaluation for every active trajectory (one grid barrier)
  // Phase A of the regenerated coupling when every warp serves every trajectory and the
  // (cos, sin) of the CTA's rows live in shared memory.  Pass 1 takes the thread's
  // (row, trajectory) pairs four at a time, all loads of a batch before its arithmetic, so the
  // L2 latencies of different trajectories overlap (a thread has only 2-3 rows per
  // trajectory); it writes (cos, sin) to shared memory.  Pass 2 forms each trajectory's
  // projections and r sums from shared memory (the thread reads back its own rows).
  __device__ void phase_a_pairs(bool want_r, int npw) {
    const int ld = p.ld, k = p.k;
    const bool emit_mode = (p.dense_level >= 1 && p.mode == MODE_INTEGRATE) || p.mode == MODE_FINAL;
    // the (row, active trajectory) pairs of the CTA are dealt to its threads evenly (pair P =
    // row + nrows * trajectory goes to thread P % KT), so no thread takes a third row of
    // every trajectory while others take two; the slopes and phases a pair reads were written
    // by other threads of the CTA
    __syncthreads();
    uint32_t actb = 0;
    int nact = 0;
    for (int b = 0; b < B; ++b)
      if (sb[b].active) actb |= (uint32_t)b << (4 * nact++);
    const int nrows = r1 - r0;
    const int npairs = nrows * nact;
    constexpr int U = 4;
    int P = tid, bi = tid / nrows, rr = tid % nrows;
    for (int p0 = tid; p0 < npairs; p0 += U * KT) {
      float om[U], yh[U], yl[U], gs[U], mh[U], ml[U];
      int bq[U], iq[U];
      bool act[U];
      // the pair's sources are read here, before any store of the batch, so that no shared
      // memory store can stand between the arithmetic chains of the batch
#pragma unroll
      for (int q = 0; q < U; ++q) {
        const bool in = P < npairs;
        const int b = in ? (int)((actb >> (4 * bi)) & 15u) : 0;
        const int i = r0 + (in ? rr : 0);
        P += KT;
        rr += KT;
        while (rr >= nrows) {
          rr -= nrows;
          ++bi;
        }
        const SrcB& s = sb[b];
        act[q] = in;
        bq[q] = b;
        iq[q] = i;
        mh[q] = s.m_hi;
        ml[q] = s.m_lo;
        om[q] = yh[q] = yl[q] = gs[q] = 0.f;
        if (in) {
          const size_t boff = ((size_t)s.base * B + b) * ld;
          om[q] = p.omega[i];
          yh[q] = p.ph_hi[boff + i];
          yl[q] = p.ph_lo[boff + i];
          const int nW = s.nW;
          // weights in two vector reads (W[7] is followed by E[0]); slopes 2..6 sit in their
          // own slots, only k1 and k7 move (FSAL)
          const float4 wa = *reinterpret_cast<const float4*>(&s.W[0]);
          const float4 wb = *reinterpret_cast<const float4*>(&s.W[4]);
          const float Wr[7] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z};
          const int s0 = s.slot[0], s6 = s.slot[6];
#pragma unroll
          for (int j = 0; j < 7; ++j) {
            const int sj = j == 0 ? s0 : (j == 6 ? s6 : j);
            if (j < nW) gs[q] = __fmaf_rn(Wr[j], p.g[((size_t)sj * B + b) * ld + i], gs[q]);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < U; ++q) {
        if (!act[q]) continue;
        const int b = bq[q], i = iq[q];
        const f2 pr = two_prod(om[q], mh[q]);
        const f2 s1 = two_sum(yh[q], pr.hi);
        const f2 s2 = two_sum(s1.hi, gs[q]);
        const float lo = yl[q] + ((s1.lo + s2.lo) + __fmaf_rn(om[q], ml[q], pr.lo));
        float sn, cs;
        sincos_pair(s2.hi, lo, &sn, &cs);
        xrow(b)[i] = make_float2(cs, sn);
        const SrcB& s = sb[b];
        const bool emit = s.rec && emit_mode;
        if (s.store_y7 || emit) {
          const size_t boff = ((size_t)s.base * B + b) * ld;
          f2 y = two_sum(s2.hi, lo);
          long long w = p.ph_w[boff + i];
          if (s.store_y7) {
            float hi7 = y.hi, lo7 = y.lo;
            long long w7 = w;
            wrap_phase(hi7, lo7, w7);
            size_t o = ((size_t)(s.base ^ 1) * B + b) * ld + i;
            p.ph_hi[o] = hi7;
            p.ph_lo[o] = lo7;
            p.ph_w[o] = w7;
          } else {
            double th = (double)w * TWO_PI_D + (double)y.hi + (double)y.lo;
            if (p.mode == MODE_INTEGRATE)
              p.out_theta[((size_t)b * p.ring + s.oslot) * ld + i] = (float)th;
            else
              p.fin_theta[(size_t)b * ld + i] = (float)th;
          }
        }
      }
    }
    __syncthreads();  // pass 2 reads rows written by other threads
    for (int b = 0; b < B; ++b) {
      float acc[PW];
#pragma unroll
      for (int v = 0; v < PW; ++v) acc[v] = 0.f;
      if (sb[b].active) {
        const float2* xb = xrow(b);
        // sum_n u_mn x_n = 2 (sum over the n with u_mn = +1) - sum_n x_n: one predicated add
        // per mode and row (the factor bits above k are zero)
        float sx = 0.f, sy = 0.f;
        for (int i = r0 + tid; i < r1; i += KT) {
          const float2 x = xb[i];
          const uint32_t u = ubits[i - r0];
          sx += x.x;
          sy += x.y;
#pragma unroll
          for (int m = 0; m < KMAX; ++m) {
            if (u & (1u << m)) {
              acc[2 * m] += x.x;
              acc[2 * m + 1] += x.y;
            }
          }
        }
#pragma unroll
        for (int m = 0; m < KMAX; ++m) {
          acc[2 * m] = 2.f * acc[2 * m] - sx;
          acc[2 * m + 1] = 2.f * acc[2 * m + 1] - sy;
        }
        if (want_r) {
          acc[PW - 2] = sx;
          acc[PW - 1] = sy;
        }
      }
      // compact layout: [2k projections][sum cos, sum sin]
      float* dst = red + (warp * BMAX + b) * PW;
#pragma unroll
      for (int c0 = 0; c0 < 2 * KMAX; c0 += 16) {
        float v16[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) v16[j] = acc[c0 + j];
        warp_reduce_scatter16(v16, lane);
        const int v = c0 + scatter16_index(lane);
        if (!(lane & 1) && v < 2 * k) dst[v] = v16[0];
      }
      if (want_r) {
        float t0 = warp_sum(acc[PW - 2]);
        float t1 = warp_sum(acc[PW - 1]);
        if (lane == 0) {
          dst[npw - 2] = t0;
          dst[npw - 1] = t1;
        }
      }
    }
  }

  __device__ bool coupling_eval(bool want_r) {
    const int n = p.n, ld = p.ld, k = p.k;
    const bool need_part = (COUP == KURA_COUPLING_VOLCANO) || want_r;
    const int npw = (COUP == KURA_COUPLING_VOLCANO ? 2 * k : 0) + (want_r ? 2 : 0);
    // phase A: stage value, sincos, exchange data and partial sums.  Each trajectory has its
    // own group of KW/B warps, so the trajectories of a batch proceed side by side.
    int b0, b1, lt, gt;
    work_map(b0, b1, lt, gt);
    bool paired = false;
    if constexpr (COUP == KURA_COUPLING_VOLCANO) {
      if (xs != nullptr && all_warps_mode()) {
        phase_a_pairs(want_r, npw);
        paired = true;
      }
    }
    if (!paired)
    for (int b = b0; b < b1; ++b) {
      const SrcB& s = sb[b];
      float acc[PW];
#pragma unroll
      for (int v = 0; v < PW; ++v) acc[v] = 0.f;
      if (s.active) {
        const size_t boff = ((size_t)s.base * B + b) * ld;
        const float* hiB = p.ph_hi + boff;
        const float* loB = p.ph_lo + boff;
        float2* xo = (COUP == KURA_COUPLING_VOLCANO) ? xrow(b) : p.xbuf + ((size_t)xpar * B + b) * ld;
        const float* gp[7];
        float Wr[7];
#pragma unroll
        for (int j = 0; j < 7; ++j) {
          gp[j] = p.g + ((size_t)s.slot[j] * B + b) * ld;
          Wr[j] = s.W[j];
        }
        const int nW = s.nW;
        const float mh = s.m_hi, ml = s.m_lo;
        const bool keep_y7 = s.store_y7;
        const bool emit = s.rec && ((p.dense_level >= 1 && p.mode == MODE_INTEGRATE) || p.mode == MODE_FINAL);
        // U rows per thread and pass: all loads of the U rows are issued before any of
        // their arithmetic, so their L2 latencies overlap (stores below could alias the
        // next rows' loads otherwise, which keeps the compiler from hoisting them)
        constexpr int U = 4;
        for (int i0 = r0 + lt; i0 < r1; i0 += U * gt) {
          float om[U], yh[U], yl[U], gsum[U];
          uint32_t ub[U];
#pragma unroll
          for (int q = 0; q < U; ++q) {
            const int i = i0 + q * gt;
            const bool ok = i < r1;
            om[q] = ok ? p.omega[i] : 0.f;
            yh[q] = ok ? hiB[i] : 0.f;
            yl[q] = ok ? loB[i] : 0.f;
            ub[q] = (COUP == KURA_COUPLING_VOLCANO && ok) ? ubits[i - r0] : 0u;
            gsum[q] = 0.f;
#pragma unroll
            for (int j = 0; j < 7; ++j)
              if (j < nW) gsum[q] = __fmaf_rn(Wr[j], ok ? gp[j][i] : 0.f, gsum[q]);
          }
#pragma unroll
          for (int q = 0; q < U; ++q) {
          const int i = i0 + q * gt;
          if (i >= r1) break;
          const f2 pr = two_prod(om[q], mh);
          const f2 s1 = two_sum(yh[q], pr.hi);
          const f2 s2 = two_sum(s1.hi, gsum[q]);
          const float lo = yl[q] + ((s1.lo + s2.lo) + __fmaf_rn(om[q], ml, pr.lo));
          float sn, cs;
          sincos_pair(s2.hi, lo, &sn, &cs);
          xo[i] = make_float2(cs, sn);
          if (keep_y7 || emit) {
            f2 y = two_sum(s2.hi, lo);
            long long w = p.ph_w[boff + i];
            if (keep_y7) {
              float hi7 = y.hi, lo7 = y.lo;
              long long w7 = w;
              wrap_phase(hi7, lo7, w7);
              size_t o = ((size_t)(s.base ^ 1) * B + b) * ld + i;
              p.ph_hi[o] = hi7;
              p.ph_lo[o] = lo7;
              p.ph_w[o] = w7;
            } else {
              double th = (double)w * TWO_PI_D + (double)y.hi + (double)y.lo;
              if (p.mode == MODE_INTEGRATE)
                p.out_theta[((size_t)b * p.ring + s.oslot) * ld + i] = (float)th;
              else
                p.fin_theta[(size_t)b * ld + i] = (float)th;
            }
          }
          if (COUP == KURA_COUPLING_VOLCANO) {
            // sums over the rows with u_mn = +1 (the factor bits above k are zero)
#pragma unroll
            for (int m = 0; m < KMAX; ++m) {
              if (ub[q] & (1u << m)) {
                acc[2 * m] += cs;
                acc[2 * m + 1] += sn;
              }
            }
          }
          if (COUP == KURA_COUPLING_VOLCANO || want_r) {
            acc[PW - 2] += cs;
            acc[PW - 1] += sn;
          }
          }
        }
      }
      if (COUP == KURA_COUPLING_VOLCANO) {
        // sum_n u_mn x_n = 2 (sum over u_mn = +1) - sum_n x_n
#pragma unroll
        for (int m = 0; m < KMAX; ++m) {
          acc[2 * m] = 2.f * acc[2 * m] - acc[PW - 2];
          acc[2 * m + 1] = 2.f * acc[2 * m + 1] - acc[PW - 1];
        }
      }
      if (need_part) {
        // compact layout: [2k projections][sum cos, sum sin]
        float* dst = red + (warp * BMAX + b) * PW;
        if (COUP == KURA_COUPLING_VOLCANO) {
          // the 2*KMAX projections, 16 at a time, reduce-scattered across the warp
#pragma unroll
          for (int c0 = 0; c0 < 2 * KMAX; c0 += 16) {
            float v16[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) v16[j] = acc[c0 + j];
            warp_reduce_scatter16(v16, lane);
            const int v = c0 + scatter16_index(lane);
            if (!(lane & 1) && v < 2 * k) dst[v] = v16[0];
          }
        }
        if (want_r) {
          float t0 = warp_sum(acc[PW - 2]);
          float t1 = warp_sum(acc[PW - 1]);
          if (lane == 0) {
            dst[npw - 2] = t0;
            dst[npw - 1] = t1;
          }
        }
      }
    }
    // phase C is needed when a slope or coupling output is written; an output pass that
    // records only r skips it
    bool need_F = false;
    for (int bb = 0; bb < B; ++bb) {
      const SrcB& sbb = sb[bb];
      need_F |= sbb.active && (sbb.gout >= 0 || (sbb.rec && (p.dense_level >= 2 || p.mode != MODE_INTEGRATE)));
    }
    if (need_part) publish_partials(npw);
    if (!grid_sync()) return false;
    if (need_part) gather_partials(npw);

    // phase C: couplings for the CTA's rows
    if (!need_F) {
      // r only
    } else if (COUP == KURA_COUPLING_VOLCANO) {
      // f3[b][2m] = (-1)^m / N * sum_n u_mn cos_n (m1, kuramoto.cu:62-81)
      for (int v = tid; v < B * 2 * KMAX; v += KT) {
        int b = v / (2 * KMAX), w = v % (2 * KMAX);
        int m = w >> 1;
        float sgn = (m & 1) ? -1.f : 1.f;
        f3[v] = (m < k) ? (sgn * rsum[b * PW + w]) / (float)n : 0.f;
      }
      __syncthreads();
      // m2 (kuramoto.cu:83-101): F_n = sum_m u_mn f3_m, summed in order of m.  For k <= 8
      // the 2^k sums, one per sign pattern, are tabulated once and looked up per row.
      float2* tab = reinterpret_cast<float2*>(f3 + BMAX * 2 * KMAX);
      const bool use_tab = (k <= 8);
      if (use_tab) {
        for (int v = tid; v < (B << k); v += KT) {
          const int b = v >> k, pat = v & ((1 << k) - 1);
          const float* fb = f3 + b * 2 * KMAX;
          float Fc = 0.f, Fs = 0.f;
          for (int m = 0; m < k; ++m) {
            const bool pos = (pat >> m) & 1;
            Fc += pos ? fb[2 * m] : -fb[2 * m];
            Fs += pos ? fb[2 * m + 1] : -fb[2 * m + 1];
          }
          tab[b * 256 + pat] = make_float2(Fc, Fs);
        }
        __syncthreads();
      }
      for (int b = b0; b < b1; ++b) {
        const SrcB& s = sb[b];
        if (!s.active) continue;
        const float2* xb = xrow(b);
        const float* fb = f3 + b * 2 * KMAX;
        const float2* tb = tab + b * 256;
        const float c1 = tr[b].c1;
        float* gdst = s.gout >= 0 ? p.g + ((size_t)s.gout * B + b) * ld : nullptr;
        const bool rec = s.rec;
        if (use_tab && !rec && gdst) {
          // the common case, 4 rows at a time: every shared-memory read of the batch before
          // its stores, which the compiler cannot reorder across
          constexpr int U = 4;
          for (int i0 = r0 + lt; i0 < r1; i0 += U * gt) {
            float2 F[U], x[U];
#pragma unroll
            for (int q = 0; q < U; ++q) {
              const int i = i0 + q * gt;
              const bool ok = i < r1;
              F[q] = ok ? tb[ubits[i - r0]] : make_float2(0.f, 0.f);
              x[q] = ok ? xb[i] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int q = 0; q < U; ++q) {
              const int i = i0 + q * gt;
              if (i < r1) gdst[i] = c1 * (x[q].y * F[q].x - x[q].x * F[q].y);
            }
          }
          continue;
        }
        for (int i = r0 + lt; i < r1; i += gt) {
          const uint32_t u = ubits[i - r0];
          float Fc = 0.f, Fs = 0.f;
          if (use_tab) {
            const float2 F = tb[u];
            Fc = F.x;
            Fs = F.y;
          } else {
#pragma unroll
            for (int m = 0; m < KMAX; ++m) {
              if (m < k) {
                bool pos = (u >> m) & 1u;
                Fc += pos ? fb[2 * m] : -fb[2 * m];
                Fs += pos ? fb[2 * m + 1] : -fb[2 * m + 1];
              }
            }
          }
          const float2 x = xb[i];
          if (!rec && gdst) {
            gdst[i] = c1 * (x.y * Fc - x.x * Fs);
          } else {
            epilogue(b, i, Fc, Fs, x.x, x.y);
          }
        }
      }
    } else if constexpr (COUP == COUP_DENSE_I8) {
      dense_matvec_i8();
    } else {
      dense_matvec();
    }
    if (want_r && gi == 0 && tid < B) {
      const int b = tid;
      const SrcB& s = sb[b];
      if (s.active && s.rec && p.mode == MODE_INTEGRATE) {
        float X = rsum[b * PW + npw - 2], Y = rsum[b * PW + npw - 1];
        float xn = X / (float)n, yn = Y / (float)n;
        p.out_r[(size_t)b * p.ring + s.oslot] = sqrtf(xn * xn + yn * yn);
        p.out_idx[(size_t)b * p.ring + s.oslot] = s.oidx;
      }
    }
    xpar ^= 1;
    __syncthreads();
    return true;
  }

  // A (rows r0..r1 of this CTA) times the (cos, sin) of every trajectory.  x is
  // staged in shared memory one column tile at a time; each warp works on up to RG rows,
  // each lane on 16-byte chunks of them.
  static constexpr int CTF = BMAX == 1 ? CT_F1 : CT;  // columns per x tile of the float product
  // A lane's 4 columns of x are 32 bytes from the next lane's, so back to back they would
  // fall on four of the eight 16-byte bank groups; a stride of F_CHUNK = 6 (cos, sin) pairs
  // (48 bytes) per 4 columns uses all eight.
  static constexpr int CTFP = CTF / 4 * F_CHUNK;
  // One x tile for the NR rows this warp holds.  A streams through the warp's ring of
  // A_STAGES * RG chunk slots with cp.async: every lane copies its own 16 bytes of each
  // row, ST = A_STAGES * RG / NR column steps ahead, and reads back only what it copied,
  // so the ring needs no barrier and holds no registers per byte in flight.  A warp with
  // fewer rows (small N, the last pass) keeps as many bytes in flight with more steps.
  // The prologue's copies start before the x tile has landed; neither part holds a barrier,
  // so warps with different NR run side by side between the caller's barriers.
  template <int NR>
  __device__ __forceinline__ void mv_f32_prologue(float4* my, const float* const (&src)[RG], int c0, int nit) {
    constexpr int ST = A_STAGES * RG / NR;
    static_assert(ST * NR <= A_STAGES * RG, "ring slots");
#pragma unroll
    for (int s = 0; s < ST - 1; ++s) {
      if (s < nit)
#pragma unroll
        for (int q = 0; q < NR; ++q) cp_async16(my + (s * NR + q) * 32, src[q] + c0 + 128 * s, 16);
      cp_async_commit();
    }
    cp_async_wait<ST - 1>();  // this thread's copies of the x tile, committed before, have landed
  }
  template <int NR>
  __device__ __forceinline__ void mv_f32_steps(float4* my, const float* const (&src)[RG], int c0, int nit,
                                               float (&acc)[RG][BMAX][2]) {
    constexpr int ST = A_STAGES * RG / NR;
    for (int it = 0; it < nit; ++it) {
      const int ahead = it + ST - 1;
      if (ahead < nit) {
        const int sl = ahead % ST;
#pragma unroll
        for (int q = 0; q < NR; ++q) cp_async16(my + (sl * NR + q) * 32, src[q] + c0 + 128 * ahead, 16);
      }
      cp_async_commit();
      cp_async_wait<ST - 1>();  // the chunks of step it have landed
      const int sl = it % ST;
      float4 a[NR];
#pragma unroll
      for (int q = 0; q < NR; ++q) a[q] = my[(sl * NR + q) * 32];
      const int cc = lane * 4 + 128 * it;
#pragma unroll
      for (int b = 0; b < BMAX; ++b) {
        if (b < B) {
          const float4* xp = reinterpret_cast<const float4*>(xt + b * CTFP + (cc >> 2) * F_CHUNK);
          float4 x01 = xp[0], x23 = xp[1];  // (c0,s0,c1,s1), (c2,s2,c3,s3)
#pragma unroll
          for (int q = 0; q < NR; ++q) {
            acc[q][b][0] += a[q].x * x01.x + a[q].y * x01.z + a[q].z * x23.x + a[q].w * x23.z;
            acc[q][b][1] += a[q].x * x01.y + a[q].y * x01.w + a[q].z * x23.y + a[q].w * x23.w;
          }
        }
      }
    }
    cp_async_wait<0>();
  }

  __device__ void dense_matvec() {
    const int ld = p.ld;
    const int rows_per_pass = KW * RG;
    float4* my = ring + (size_t)warp * (A_STAGES * RG * 32) + lane;
    for (int pr0 = r0; pr0 < r1; pr0 += rows_per_pass) {
      float acc[RG][BMAX][2];
#pragma unroll
      for (int q = 0; q < RG; ++q)
#pragma unroll
        for (int b = 0; b < BMAX; ++b) acc[q][b][0] = acc[q][b][1] = 0.f;
      // warp w takes rows pr0 + w + KW*q of the pass, so small row blocks keep every warp
      // busy; its nr rows in the CTA's block are q < nr
      const int row0 = pr0 + warp;
      const int nr = r1 > row0 ? min(RG, (r1 - row0 + KW - 1) / KW) : 0;
      const float* src[RG];
#pragma unroll
      for (int q = 0; q < RG; ++q) {
        const int row = row0 + KW * q;
        src[q] = p.adj + (size_t)(row < r1 ? row : r0) * ld + lane * 4;
      }
      int c0 = 0;
      for (; c0 < ld; c0 += CTF) {
        __syncthreads();  // the previous tile's readers are done
        const int cw = min(CTF, ld - c0);  // a multiple of 32
        // the x tile, 16 bytes (two columns) per copy, in one commit group ahead of the ring's
        for (int b = 0; b < B; ++b)
          for (int c = 2 * tid; c < cw; c += 2 * KT)
            cp_async16(xt + b * CTFP + (c >> 2) * F_CHUNK + (c & 3), p.xbuf + ((size_t)xpar * B + b) * ld + c0 + c,
                       16);
        cp_async_commit();
        // column steps of this lane: cc = lane*4 + 128*it < cw
        const int nit = (cw - lane * 4 + 127) >> 7;
        if (nr == 4) mv_f32_prologue<4>(my, src, c0, nit);
        else if (nr == 3) mv_f32_prologue<3>(my, src, c0, nit);
        else if (nr == 2) mv_f32_prologue<2>(my, src, c0, nit);
        else if (nr == 1) mv_f32_prologue<1>(my, src, c0, nit);
        else cp_async_wait<0>();
        __syncthreads();  // every thread's part of the x tile has landed
        if (nr == 4) mv_f32_steps<4>(my, src, c0, nit, acc);
        else if (nr == 3) mv_f32_steps<3>(my, src, c0, nit, acc);
        else if (nr == 2) mv_f32_steps<2>(my, src, c0, nit, acc);
        else if (nr == 1) mv_f32_steps<1>(my, src, c0, nit, acc);
      }
      const int xt_c0 = c0 - CTF;  // first column of the tile still staged
#pragma unroll
      for (int q = 0; q < RG; ++q)
        if (q < nr)
#pragma unroll
          for (int b = 0; b < BMAX; ++b) {
            acc[q][b][0] = warp_sum(acc[q][b][0]);
            acc[q][b][1] = warp_sum(acc[q][b][1]);
          }
      // lane q*BMAX+b finishes row row0+q of trajectory b; its own (cos, sin) come from the
      // staged tile when the last tile holds the row
#pragma unroll
      for (int q = 0; q < RG; ++q)
#pragma unroll
        for (int b = 0; b < BMAX; ++b) {
          int row = row0 + KW * q;
          if (lane == q * BMAX + b && b < B && row < r1 && sb[b].active) {
            const int c = row - xt_c0;
            const float2 x = c >= 0 ? xt[b * CTFP + (c >> 2) * F_CHUNK + (c & 3)]
                                    : __ldcg(&p.xbuf[((size_t)xpar * B + b) * ld + row]);
            epilogue(b, row, acc[q][b][0], acc[q][b][1], x.x, x.y);
          }
        }
    }
  }

  static constexpr int CTX = BMAX == 1 ? CT_I8 : CT;  // columns per x tile of the int8 product
  // The int8 product's x tile holds per column the float4 (cos, cos, sin, sin), so that one
  // packed FP32 FMA multiplies the converted bytes of two rows by the same column.  A lane's
  // 16 columns start I8_CHUNK4 = 17 float4 (272 bytes) after the previous lane's, which puts
  // the 8 lanes of each phase of a 16-byte shared-memory read on distinct banks.
  static constexpr int CTXP = CTX / 16 * I8_CHUNK4;  // float4 per trajectory
  // The columns [c0, c0 + cw) of the staged tile for the first RGT of the pass's RG_I8 rows of
  // this warp (rows pr0 + warp + KW*q), 16 int8 columns per lane and step; rows 2qp and 2qp+1
  // share the packed accumulators acc[qp].  A streams through the warp's ring of I8_SLOTS
  // chunk slots (16 bytes per lane) with cp.async, I8_SLOTS / RGT steps deep, so the loads of
  // the next step are in flight during this step's conversion and FMAs.  No barrier inside:
  // warps with different RGT run side by side between the tile barriers of the caller.
  static constexpr int RG_I8 = 8;
  template <int RGT>
  __device__ __forceinline__ void mv_i8_tile(unsigned long long (&acc)[RG_I8 / 2][2], int row0, int c0, int cw) {
    static_assert(RGT % 2 == 0 && RGT <= RG_I8 && I8_SLOTS % RGT == 0, "rows are taken in pairs");
    constexpr int ST = I8_SLOTS / RGT;
    const int ld8 = p.ld8;
    const float4* xt4 = reinterpret_cast<const float4*>(xt);
    uint4* my = reinterpret_cast<uint4*>(ring) + (size_t)warp * (I8_SLOTS * 32) + lane;
    const int8_t* src[RGT];
    int nb[RGT];
#pragma unroll
    for (int q = 0; q < RGT; ++q) {
      const int row = row0 + KW * q;
      nb[q] = row < r1 ? 16 : 0;  // rows past the CTA's block are zero-filled
      src[q] = p.adj8 + (size_t)(row < r1 ? row : r0) * ld8 + c0 + lane * 16;
    }
    // steps of this lane: columns cc = lane*16 + 512*it < cw (cw is a multiple of 16)
    const int nit = cw > lane * 16 ? (cw - lane * 16 + 511) >> 9 : 0;
#pragma unroll
    for (int s = 0; s < ST - 1; ++s) {
      if (s < nit)
#pragma unroll
        for (int q = 0; q < RGT; ++q) cp_async16(my + (s * RGT + q) * 32, src[q] + 512 * s, nb[q]);
      cp_async_commit();
    }
    for (int it = 0; it < nit; ++it) {
      const int ahead = it + ST - 1;
      if (ahead < nit) {
        const int sl = ahead % ST;
#pragma unroll
        for (int q = 0; q < RGT; ++q) cp_async16(my + (sl * RGT + q) * 32, src[q] + 512 * ahead, nb[q]);
      }
      cp_async_commit();
      cp_async_wait<ST - 1>();  // the chunks of step it have landed
      const int sl = it % ST;
      uint32_t a[RGT][4];
#pragma unroll
      for (int q = 0; q < RGT; ++q) {
        const uint4 v = my[(sl * RGT + q) * 32];
        a[q][0] = v.x ^ 0x80808080u;
        a[q][1] = v.y ^ 0x80808080u;
        a[q][2] = v.z ^ 0x80808080u;
        a[q][3] = v.w ^ 0x80808080u;
      }
      const int cc = lane * 16 + 512 * it;
#pragma unroll
      for (int wd = 0; wd < 4; ++wd) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          // ((cos, cos), (sin, sin)) of column cc + 4*wd + j
          const ulonglong2 xj = *reinterpret_cast<const ulonglong2*>(xt4 + (cc >> 4) * I8_CHUNK4 + 4 * wd + j);
#pragma unroll
          for (int qp = 0; qp < RGT / 2; ++qp) {
            const unsigned long long kp = i8_pair_to_f2(a[2 * qp][wd], a[2 * qp + 1][wd], j);
            acc[qp][0] = ffma2(kp, xj.x, acc[qp][0]);
            acc[qp][1] = ffma2(kp, xj.y, acc[qp][1]);
          }
        }
      }
    }
    cp_async_wait<0>();
  }
  // one pass over the RG_I8 rows per warp of one trajectory
  __device__ void mv_i8_pass(int pr0) {
    const int ld = p.ld, ld8 = p.ld8;
    float4* xt4 = reinterpret_cast<float4*>(xt);
    // [qp][0]: (sum k cos) of rows (2qp, 2qp+1); [qp][1]: the same for sin
    unsigned long long acc[RG_I8 / 2][2];
#pragma unroll
    for (int q = 0; q < RG_I8 / 2; ++q) acc[q][0] = acc[q][1] = 0ull;
    const int row0 = pr0 + warp;
    const int nr = r1 > row0 ? min(RG_I8, (r1 - row0 + KW - 1) / KW) : 0;
    int c0 = 0;
    for (; c0 < ld8; c0 += CTX) {
      __syncthreads();
      const int cw = min(CTX, ld8 - c0);  // a multiple of 16
      for (int c = tid; c < cw; c += KT) {
        const float2 x = __ldcg(&p.xbuf[(size_t)xpar * ld + c0 + c]);
        xt4[(c >> 4) * I8_CHUNK4 + (c & 15)] = make_float4(x.x, x.x, x.y, x.y);
      }
      __syncthreads();
      // a warp with at most 4 rows in the pass (small N, the last pass) converts no bytes of
      // the absent ones
      if (nr <= 4) mv_i8_tile<4>(acc, row0, c0, cw);
      else mv_i8_tile<RG_I8>(acc, row0, c0, cw);
    }
    float accf[RG_I8][2];
#pragma unroll
    for (int qp = 0; qp < RG_I8 / 2; ++qp)
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const float2 u = unpack_f2(acc[qp][v]);
        accf[2 * qp][v] = warp_sum(u.x);
        accf[2 * qp + 1][v] = warp_sum(u.y);
      }
    // the row's own (cos, sin) from the staged tile when the last tile holds it
    const int xt_c0 = c0 - CTX;
#pragma unroll
    for (int q = 0; q < RG_I8; ++q) {
      const int row = row0 + KW * q;
      if (lane == q && row < r1 && sb[0].active) {
        const int c = row - xt_c0;
        float2 x;
        if (c >= 0) {
          const float4 v = xt4[(c >> 4) * I8_CHUNK4 + (c & 15)];
          x = make_float2(v.x, v.z);
        } else {
          x = __ldcg(&p.xbuf[(size_t)xpar * ld + row]);
        }
        epilogue(0, row, accf[q][0] * p.invn, accf[q][1] * p.invn, x.x, x.y);
      }
    }
  }
  // The batch form: x tile of (cos, sin) pairs, I8_CHUNK = 18 pairs (144 bytes) per 16
  // columns, and one scalar FMA per byte, trajectory and sum; the register budget of eight
  // trajectories leaves no room for the packed form's operands.
  static constexpr int CTXB = CTX / 16 * I8_CHUNK;  // float2 per trajectory
  template <int RG, int CPL>
  __device__ void mv_i8_pass_batch(int pr0) {
    constexpr int NWD = CPL / 4;
    const int ld = p.ld, ld8 = p.ld8;
    float acc[RG][BMAX][2];
#pragma unroll
    for (int q = 0; q < RG; ++q)
#pragma unroll
      for (int b = 0; b < BMAX; ++b) acc[q][b][0] = acc[q][b][1] = 0.f;
    const int row0 = pr0 + warp;
    for (int c0 = 0; c0 < ld8; c0 += CTX) {
      __syncthreads();
      const int cw = min(CTX, ld8 - c0);  // a multiple of 16
      for (int t = tid; t < B * CTX; t += KT) {
        int b = t / CTX, c = t - b * CTX;
        xt[b * CTXB + (c >> 4) * I8_CHUNK + (c & 15)] =
            (c < cw) ? __ldcg(&p.xbuf[((size_t)xpar * B + b) * ld + c0 + c]) : make_float2(0.f, 0.f);
      }
      __syncthreads();
      for (int cc = lane * CPL; cc < cw; cc += 32 * CPL) {
        uint32_t a[RG][NWD];
#pragma unroll
        for (int q = 0; q < RG; ++q) {
          const int row = row0 + KW * q;
          const int8_t* src = p.adj8 + (size_t)row * ld8 + c0 + cc;
          if (CPL == 16) {
            const uint4 v = (row < r1) ? ld_stream_u4(src) : make_uint4(0u, 0u, 0u, 0u);
            a[q][0] = v.x;
            a[q][1 % NWD] = v.y;
            a[q][2 % NWD] = v.z;
            a[q][3 % NWD] = v.w;
          } else {
            const uint2 v = (row < r1) ? ld_stream_u2(src) : make_uint2(0u, 0u);
            a[q][0] = v.x;
            a[q][1 % NWD] = v.y;
          }
#pragma unroll
          for (int wd = 0; wd < NWD; ++wd) a[q][wd] ^= 0x80808080u;
        }
#pragma unroll
        for (int wd = 0; wd < NWD; ++wd) {
#pragma unroll
          for (int b = 0; b < BMAX; ++b) {
            if (b < B) {
              const float4* xp = reinterpret_cast<const float4*>(xt + b * CTXB + (cc >> 4) * I8_CHUNK + 4 * wd);
              const float4 x01 = xp[0], x23 = xp[1];  // (c0,s0,c1,s1), (c2,s2,c3,s3)
#pragma unroll
              for (int q = 0; q < RG; ++q) {
                const uint32_t w = a[q][wd];
                const float k0 = i8_to_f(w, 0), k1 = i8_to_f(w, 1), k2 = i8_to_f(w, 2), k3 = i8_to_f(w, 3);
                acc[q][b][0] += k0 * x01.x + k1 * x01.z + k2 * x23.x + k3 * x23.z;
                acc[q][b][1] += k0 * x01.y + k1 * x01.w + k2 * x23.y + k3 * x23.w;
              }
            }
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < RG; ++q)
#pragma unroll
      for (int b = 0; b < BMAX; ++b) {
        acc[q][b][0] = warp_sum(acc[q][b][0]);
        acc[q][b][1] = warp_sum(acc[q][b][1]);
      }
#pragma unroll
    for (int q = 0; q < RG; ++q)
#pragma unroll
      for (int b = 0; b < BMAX; ++b) {
        const int row = row0 + KW * q;
        if (lane == (q * BMAX + b) % 32 && b < B && row < r1 && sb[b].active) {
          float2 x = __ldcg(&p.xbuf[((size_t)xpar * B + b) * ld + row]);
          epilogue(b, row, acc[q][b][0] * p.invn, acc[q][b][1] * p.invn, x.x, x.y);
        }
      }
  }
  // The same product with A stored as the integers N*A (int8, exact for the reference's
  // volcano rule, K <= 127): a quarter of the HBM bytes.  Each lane streams 16 columns of
  // 8 rows (one trajectory) or 2 rows (a batch) per load; the sums are scaled by 1/N
  // before the epilogue.  One trajectory converts the bytes of two rows at a time into a
  // packed float pair and multiplies it by a column's (cos, cos) and (sin, sin) with packed
  // FMAs: 2.5 instructions per byte and trajectory instead of 4.  (16 rows of 8 columns
  // halves the shared-memory reads of x but measured 2x slower at N=65536: half the bytes in
  // flight per load.)
  __device__ void dense_matvec_i8() {
    constexpr int RG = BMAX == 1 ? 8 : 2;
    for (int pr0 = r0; pr0 < r1; pr0 += KW * RG) {
      if constexpr (BMAX > 1) mv_i8_pass_batch<RG, 16>(pr0);
      else mv_i8_pass(pr0);
    }
  }

  // ---- error norm of the attempt (dp45.cu:79-84, 116-119); sum of squares -> rsum[b*PW]
  __device__ bool error_phase() {
    const int ld = p.ld;
    int b0, b1, lt, gt;
    work_map(b0, b1, lt, gt);
    for (int b = b0; b < b1; ++b) {
      const SrcB& s = sb[b];
      float acc = 0.f;
      if (s.active) {
        const size_t yb = ((size_t)s.base * B + b) * ld, y7b = ((size_t)(s.base ^ 1) * B + b) * ld;
        const float* gp[7];
        float Er[7];
#pragma unroll
        for (int j = 0; j < 7; ++j) {
          gp[j] = p.g + ((size_t)s.slot[j] * B + b) * ld;
          Er[j] = s.E[j];
        }
        constexpr int U = 4;
        for (int i0 = r0 + lt; i0 < r1; i0 += U * gt) {
          float ev[U];
#pragma unroll
          for (int q = 0; q < U; ++q) {
            const int i = i0 + q * gt;
            ev[q] = 0.f;
            if (i < r1) {
#pragma unroll
              for (int j = 0; j < 7; ++j) ev[q] = __fmaf_rn(Er[j], gp[j][i], ev[q]);
            }
          }
#pragma unroll
          for (int q = 0; q < U; ++q) {
          const int i = i0 + q * gt;
          if (i >= r1) break;
          float e = ev[q];
          float tol = (float)p.atol;
          if (p.rtol != 0.0) {
            float a0 = fabsf(__fmaf_rn((float)p.ph_w[yb + i], P2_1, p.ph_hi[yb + i]));
            float a1 = fabsf(__fmaf_rn((float)p.ph_w[y7b + i], P2_1, p.ph_hi[y7b + i]));
            tol = (float)p.atol + (float)p.rtol * fmaxf(a0, a1);
          }
          float ye = e / tol;
          acc = __fmaf_rn(ye, ye, acc);
          }
        }
      }
      float t = warp_sum(acc);
      if (lane == 0) red[(warp * BMAX + b) * PW] = t;
    }
    publish_partials(1);
    if (!grid_sync()) return false;
    gather_partials(1);
    return true;
  }

  // ---- per-trajectory sources
  // the six stages of one attempt (the stage loop of dp45_step, dp45.cu:90-106), filled at
  // once by 16 threads per (stage, trajectory); the active flags are copied from sb_base
  __device__ void setup_attempt() {
    __syncthreads();  // the active flags were just written by threads tid < B
    for (int t = tid; t < 6 * B * 16; t += KT) {
      const int j = t & 15, b = (t >> 4) % B, s = 2 + (t >> 4) / B;
      SrcB& S = sb_base[(s - 1) * BMAX + b];
      const TrajG& T = tr[b];
      const double h = T.h;
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
        S.oslot = -1;
        S.oidx = 0;
        S.active = sb_base[b].active;
      }
    }
    __syncthreads();
  }
  // dense output at te from the last accepted step (interpolate, dp45.cu:70-76).
  // k1s / k7s choose the physical slopes; the end-of-run record passes the slot of
  // k7 for both, as the reference's FSAL copy leaves them (dp45.cu:160).
  __device__ void fill_eval(int b, int j, double te, int k1s, int k7s) {
    SrcB& S = sb[b];
    const TrajG& T = tr[b];
    const double hs = T.t - T.t_last, dl = te - T.t_last;
    if (j < 7) {
      const double x = dl / hs;
      const double c = ((P_TAB[j][3] * x + P_TAB[j][2]) * x + P_TAB[j][1]) * x * x + P_TAB[j][0] * x;
      S.W[j] = (float)(hs * c);
    } else if (j == 14) {
      float hi = (float)dl;
      S.m_hi = hi;
      S.m_lo = (float)(dl - (double)hi);
    } else if (j == 15) {
      S.nW = 7;
      S.slot[0] = k1s;
      for (int q = 1; q < 6; ++q) S.slot[q] = q;
      S.slot[6] = k7s;
      S.base = T.rot_y ^ 1;
      S.gout = -1;
      S.store_y7 = 0;
      S.rec = 1;
    }
  }
  __device__ void fill_y(int b, int j) {
    SrcB& S = sb[b];
    const TrajG& T = tr[b];
    if (j < 7) {
      S.W[j] = 0.f;
    } else if (j == 14) {
      S.m_hi = S.m_lo = 0.f;
    } else if (j == 15) {
      S.nW = 0;
      for (int q = 0; q < 7; ++q) S.slot[q] = q;
      S.base = T.rot_y;
      S.gout = -1;
      S.store_y7 = 0;
      S.rec = 0;
      S.oslot = -1;
      S.oidx = -1;
    }
  }

  // controller of one trajectory after the error norm (dp45.cu:109-139)
  __device__ void decide(int b) {
    TrajG& T = tr[b];
    const double h = T.h;
    bool accept = true;
    double factor = 1.0;
    if (!p.fixed) {
      double norm = sqrt((double)rsum[b * PW]) / sqrt((double)p.n);
      if (isnan(norm)) {
        T.status = KURA_ERR_NONFINITE;
        return;
      }
      // 0.9 norm^(-1/5) (dp45.cu:120); norm = +inf gives 0: the attempt is rejected with the 0.2 floor
      factor = (double)(0.9f * exp2f(-0.2f * log2f((float)norm)));
      accept = norm < 1.0;
    }
    if (accept) {
      T.t_last = T.t;
      T.t = T.t + h;
      T.rot_y ^= 1;
      T.rot_g ^= 1;
      T.accepted++;
      if (!p.fixed) T.h = h * fmin(factor, 10.0);
      int e = T.eval_i;
      while (e < p.n_eval && T.t >= (double)p.t_eval[e]) e++;
      T.eval_end = e;
      if (p.log_cap > 0) {
        p.log_t[(size_t)b * p.log_cap + T.log_count] = T.t;
        p.log_h[(size_t)b * p.log_cap + T.log_count] = T.h;
      }
      T.log_count++;
    } else {
      T.rejected++;
      if (factor < 1.0) T.h = h * fmax(factor, 0.2);
      if (!(T.h >= 1e-14 * fmax(1.0, fabs(T.t)))) T.status = KURA_ERR_STEP_UNDERFLOW;
    }
  }

  __device__ void write_back() {
    if (gi == 0 && tid < B) p.traj[tid] = tr[tid];
    if (gi == 0 && tid == 0) atomicAdd((unsigned long long*)p.counters, (unsigned long long)nbar);
  }

  // ---- the whole launch
  __device__ void run() {
    if (tid < B) tr[tid] = p.traj[tid];
    if (COUP == KURA_COUPLING_VOLCANO) {
      for (int lr = tid; lr < r1 - r0; lr += KT) {
        int i = r0 + lr;
        uint32_t w = 0;
        for (int m = 0; m < p.k; ++m)
          w |= (stream_word(p.seed, (unsigned long long)m * (unsigned long long)p.n + (unsigned long long)i) & 1u) << m;
        ubits[lr] = w;
      }
    }
    __syncthreads();

    if (p.mode == MODE_FINAL || p.mode == MODE_RHS) {
      if (tid < B * 16) {
        const int b = tid >> 4, j = tid & 15;
        const TrajG& T = tr[b];
        if (p.mode == MODE_FINAL && p.n_eval > 0 && T.accepted > 0) {
          int ks = slot_k1(T.rot_g);  // after the last FSAL swap this slot holds k7
          fill_eval(b, j, (double)p.t_eval[p.n_eval - 1], ks, ks);
        } else {
          fill_y(b, j);
        }
        if (j == 15) {
          sb[b].active = 1;
          sb[b].rec = 1;
          sb[b].oslot = -1;
        }
      }
      __syncthreads();
      if (!coupling_eval(false)) return;
      write_back();
      return;
    }

    // first slope of the run (dp45.cu:151) and the record at t0 (kuramoto.cu:587-626)
    if (tid < B * 16) {
      const int b = tid >> 4, j = tid & 15;
      const TrajG& T = tr[b];
      fill_y(b, j);
      if (j == 15) {
        SrcB& S = sb[b];
        S.active = (T.status == 0 && T.need_k1);
        S.gout = slot_k1(T.rot_g);
        if (S.active && T.need_init && T.out_count < p.ring) {
          S.rec = 1;
          S.oslot = T.out_count;
          S.oidx = -1;
        }
      }
    }
    __syncthreads();
    {
      bool any = false, want_r = false;
      for (int b = 0; b < B; ++b) {
        any |= (bool)sb[b].active;
        want_r |= (sb[b].active && sb[b].rec);
      }
      if (any) {
        if (!coupling_eval(want_r)) return;
        if (tid < B) {
          if (sb[tid].active) {
            tr[tid].need_k1 = 0;
            if (sb[tid].rec) { tr[tid].need_init = 0; tr[tid].out_count++; }
          }
        }
        __syncthreads();
      }
    }

    long long attempts = 0;
    while (true) {
      if (tid == 0) {
        int todo_out = 0, todo_step = 0, stop = 0;
        for (int b = 0; b < B; ++b) {
          TrajG& T = tr[b];
          if (T.status != 0) continue;
          if (T.eval_i < T.eval_end) {
            if (T.out_count < p.ring) todo_out = 1; else stop = 1;
            continue;
          }
          if (!(T.t < T.t1)) { T.status = 1; continue; }
          if (p.log_cap > 0 && T.log_count >= p.log_cap) { stop = 1; continue; }
          todo_step = 1;
        }
        if (p.max_attempts >= 0 && attempts >= p.max_attempts) stop = 1;
        flag[1] = todo_out;
        flag[2] = todo_step;
        flag[3] = stop;
      }
      __syncthreads();
      if (flag[1]) {
        // one pending output of every trajectory that owes one
        if (tid < B * 16) {
          const int b = tid >> 4, j = tid & 15;
          const TrajG& T = tr[b];
          const bool act = (T.status == 0 && T.eval_i < T.eval_end && T.out_count < p.ring);
          if (act) {
            // after the accept, k1 of the step sits in the k7 slot and vice versa
            fill_eval(b, j, (double)p.t_eval[T.eval_i], slot_k7(T.rot_g), slot_k1(T.rot_g));
            if (j == 15) {
              sb[b].oslot = T.out_count;
              sb[b].oidx = T.eval_i;
            }
          }
          if (j == 15) sb[b].active = act;
        }
        __syncthreads();
        if (!coupling_eval(true)) return;
        if (tid < B && sb[tid].active) {
          tr[tid].eval_i++;
          tr[tid].out_count++;
        }
        __syncthreads();
        continue;
      }
      if (flag[3] || !flag[2]) break;

      // ---- one attempt of every stepping trajectory (dp45_step, dp45.cu:87-141)
      if (tid < B) {
        const TrajG& T = tr[tid];
        sb[tid].active = (T.status == 0 && T.eval_i >= T.eval_end && T.t < T.t1 &&
                          !(p.log_cap > 0 && T.log_count >= p.log_cap));
      }
      setup_attempt();  // ends with __syncthreads
      for (int s = 2; s <= 7; ++s) {
        sb = sb_base + (s - 1) * BMAX;
        if (!coupling_eval(false)) return;
      }
      // sb stays on stage 7: the error phase uses its E weights, slots and phase buffers
      if (!p.fixed) {
        if (!error_phase()) return;
      }
      if (tid < B && sb[tid].active) decide(tid);
      __syncthreads();
      sb = sb_base;
      attempts++;
    }
    write_back();
  }
};

template <int COUP, int BMAX, int KMAX>
__global__ void __launch_bounds__(KT, 1) k_persistent(const KParams p) {
  extern __shared__ __align__(16) unsigned char smem[];
  Engine<COUP, BMAX, KMAX> e(p, smem);
  e.run();
}

template <int COUP, int BMAX, int KMAX>
static const void* kernel_ptr() {
  return (const void*)&k_persistent<COUP, BMAX, KMAX>;
}

static const void* pick_kernel(int coupling, int bmax, int kmax) {
  if (coupling == KURA_COUPLING_DENSE) {
    if (bmax == 1) return kernel_ptr<KURA_COUPLING_DENSE, 1, 1>();
    if (bmax == 8) return kernel_ptr<KURA_COUPLING_DENSE, 8, 1>();
  } else if (coupling == COUP_DENSE_I8) {
    if (bmax == 1) return kernel_ptr<COUP_DENSE_I8, 1, 1>();
    if (bmax == 8) return kernel_ptr<COUP_DENSE_I8, 8, 1>();
  } else {
    if (bmax == 1 && kmax == 8) return kernel_ptr<KURA_COUPLING_VOLCANO, 1, 8>();
    if (bmax == 8 && kmax == 8) return kernel_ptr<KURA_COUPLING_VOLCANO, 8, 8>();
    if (bmax == 1 && kmax == 32) return kernel_ptr<KURA_COUPLING_VOLCANO, 1, 32>();
    if (bmax == 8 && kmax == 32) return kernel_ptr<KURA_COUPLING_VOLCANO, 8, 32>();
  }
  return nullptr;
}

cudaError_t persistent_config(int coupling, int bmax, int kmax, size_t* smem_bytes, int* blocks_per_sm,
                              int rows_per_cta, int* xs_smem) {
  const void* f = pick_kernel(coupling, bmax, kmax);
  if (!f) return cudaErrorInvalidValue;
  int off[10], total;
  const int kk = coupling != KURA_COUPLING_VOLCANO ? 1 : kmax;
  // keep the CTA's (cos, sin) in shared memory when it fits comfortably
  *xs_smem = 1;
  smem_layout(coupling, bmax, kk, rows_per_cta, 1, off, &total);
  if (coupling != KURA_COUPLING_VOLCANO || total > 200 * 1024) {
    *xs_smem = 0;
    smem_layout(coupling, bmax, kk, rows_per_cta, 0, off, &total);
  }
  *smem_bytes = (size_t)total;
  cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, total);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, KT, (size_t)total);
}

cudaError_t launch_persistent(const KParams& p, int grid, int bmax, int kmax, size_t smem, cudaStream_t st) {
  const void* f = pick_kernel(p.coupling, bmax, kmax);
  if (!f) return cudaErrorInvalidValue;
  KParams copy = p;
  void* args[] = {&copy};
  return cudaLaunchCooperativeKernel(f, dim3(grid), dim3(KT), args, smem, st);
}

// ------------------------------------------------------------------ small kernels
// theta (unwrapped float) -> wrapped (hi, lo, winding)
__global__ void k_init_state(const float* __restrict__ theta, int n, float* hi, float* lo, long long* w) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    double t = (double)theta[i];
    double k = rint(t / TWO_PI_D);
    double r = t - k * TWO_PI_D;
    float h = (float)r;
    hi[i] = h;
    lo[i] = (float)(r - (double)h);
    w[i] = (long long)k;
  }
}
__global__ void k_unwrap(const float* hi, const float* lo, const long long* w, int n, float* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)((double)w[i] * TWO_PI_D + (double)hi[i] + (double)lo[i]);
}
cudaError_t launch_init_state(const float* theta, int n, int ld, float* hi, float* lo, long long* w,
                              cudaStream_t st) {
  (void)ld;
  if (n <= 0) return cudaSuccess;
  k_init_state<<<(n + 255) / 256, 256, 0, st>>>(theta, n, hi, lo, w);
  return cudaGetLastError();
}
cudaError_t launch_unwrap(const float* hi, const float* lo, const long long* w, int n, float* out,
                          cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_unwrap<<<(n + 255) / 256, 256, 0, st>>>(hi, lo, w, n, out);
  return cudaGetLastError();
}

// factor bits packed per oscillator: bits[wd*n + i] bit (m - 32*wd) = low bit of element m*n+i
__global__ void k_volcano_words(int seed, int n, int k, int words, uint32_t* bits) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * words) return;
  int i = (int)(t % n), wd = (int)(t / n);
  uint32_t w = 0;
  int m0 = 32 * wd, m1 = min(k, m0 + 32);
  for (int m = m0; m < m1; ++m)
    w |= (stream_word(seed, (unsigned long long)m * (unsigned long long)n + (unsigned long long)i) & 1u) << (m - m0);
  bits[(size_t)wd * n + i] = w;
}
cudaError_t launch_volcano_words(int seed, int n, int k, int words, uint32_t* bits, cudaStream_t st) {
  long long tot = (long long)n * words;
  if (tot <= 0) return cudaSuccess;
  k_volcano_words<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(seed, n, k, words, bits);
  return cudaGetLastError();
}

// N*A_ij = sum_m (-1)^m u_mi u_mj = (#even m) - (#odd m) - 2*popc(even disagreements) + 2*popc(odd ones);
// the entry is that integer times fl(1/N), rounded once (kuramoto.cu:137-157 forms it by a GEMM).
__global__ void k_volcano_adjacency(const uint32_t* __restrict__ bits, int n, int k, int words, int ld,
                                    float* __restrict__ adj) {
  const float invn = 1.0f / (float)n;
  for (int i = blockIdx.y; i < n; i += gridDim.y)
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < ld; j += gridDim.x * blockDim.x) {
    float v = 0.f;
    if (j < n) {
      int kk = 0;
      for (int wd = 0; wd < words; ++wd) {
        int m0 = 32 * wd, cnt = min(32, k - m0);
        uint32_t valid = cnt >= 32 ? 0xffffffffu : ((1u << cnt) - 1u);
        uint32_t even = 0x55555555u & valid, odd = 0xAAAAAAAAu & valid;  // m0 is even
        uint32_t dis = bits[(size_t)wd * n + i] ^ bits[(size_t)wd * n + j];
        kk += __popc(even) - __popc(odd) - 2 * __popc(dis & even) + 2 * __popc(dis & odd);
      }
      v = __fmul_rn((float)kk, invn);
    }
    adj[(size_t)i * ld + j] = v;
  }
}
// N*A as int8: kk of the row above, exact for k <= 127
__global__ void k_volcano_adjacency_i8(const uint32_t* __restrict__ bits, int n, int k, int words, int ld8,
                                       int8_t* __restrict__ adj8) {
  for (int i = blockIdx.y; i < n; i += gridDim.y)
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < ld8; j += gridDim.x * blockDim.x) {
      int kk = 0;
      if (j < n) {
        for (int wd = 0; wd < words; ++wd) {
          int m0 = 32 * wd, cnt = min(32, k - m0);
          uint32_t valid = cnt >= 32 ? 0xffffffffu : ((1u << cnt) - 1u);
          uint32_t even = 0x55555555u & valid, odd = 0xAAAAAAAAu & valid;
          uint32_t dis = bits[(size_t)wd * n + i] ^ bits[(size_t)wd * n + j];
          kk += __popc(even) - __popc(odd) - 2 * __popc(dis & even) + 2 * __popc(dis & odd);
        }
      }
      adj8[(size_t)i * ld8 + j] = (int8_t)kk;
    }
}
cudaError_t launch_volcano_adjacency_i8(const uint32_t* bits, int n, int k, int words, int ld8, int8_t* adj8,
                                        cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  dim3 grid((unsigned)min((ld8 + 255) / 256, 64), (unsigned)min(n, 65535));
  k_volcano_adjacency_i8<<<grid, 256, 0, st>>>(bits, n, k, words, ld8, adj8);
  return cudaGetLastError();
}
cudaError_t launch_volcano_adjacency(const uint32_t* bits, int n, int k, int words, int ld, float* adj,
                                     cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  dim3 grid((unsigned)min((ld + 255) / 256, 64), (unsigned)min(n, 65535));
  k_volcano_adjacency<<<grid, 256, 0, st>>>(bits, n, k, words, ld, adj);
  return cudaGetLastError();
}

}  // namespace kura
