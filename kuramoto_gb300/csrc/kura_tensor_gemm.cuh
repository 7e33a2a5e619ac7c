// kura_tensor_gemm.cuh -- tcgen05 GEMM with a fused epilogue:
//   C[m][c] = sum_k A[m][k] * X[c][k]      (A: M x K BF16, X: NCOL x K BF16, both K-major)
// accumulated in FP32 in tensor memory.  A work unit is a 128-row tile times one block of
// NCOL columns (NCOL <= 512); CTAs loop over units (persistent).
//
// Roles (192 threads): warp 0 lane 0 streams A and X tiles with TMA (64-byte swizzle, 32
// BF16 of K per stage, so that even NCOL = 512 keeps 5 stages in flight) into a ring of
// STAGES shared-memory stages; warp 1 lane 0 issues the MMAs (M = 128, N = min(NCOL,
// 256), K = 16 per instruction) and commits each stage back to the producer; warps 2-5
// read the accumulator (warp w owns TMEM lanes 32*(w%4)..+31, one tile row per thread)
// and call the epilogue.  With NCOL <= 256 two accumulators alternate in TMEM, so the MMAs
// of one unit run while the epilogue reads the previous one.  Every wait is bounded: on a timeout the CTA records an error,
// stops issuing work, waits (bounded) for its own TMA copies, frees TMEM and returns.
#pragma once
#include "kura_umma.cuh"

namespace kura {

constexpr int TG_BM = 128;  // rows per tile (M of one MMA)
constexpr int TG_BK = 32;   // K per stage (one 64-byte swizzle row of BF16)
constexpr int TG_ROWB = TG_BK * 2;  // bytes per tile row
constexpr int TG_THREADS = 192;  // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue

// NCOL columns per work unit, MT row tiles of 128 per work unit (sharing every X stage: MT = 2
// halves the operand bytes per flop that X costs), BK of K per stage: 32 (rows of 64 bytes, the
// 64-byte swizzle) or 64 (rows of 128 bytes, the 128-byte swizzle)
template <int NCOL, int MT = 1, int BK = TG_BK> struct TGCfg {
  static constexpr int NMMA = NCOL > 256 ? 256 : NCOL;  // N of one MMA instruction
  static constexpr int NH = NCOL / NMMA;                // MMAs per K step and row tile
  static constexpr int ROWB = BK * 2;                  // bytes per operand row of a stage
  static constexpr int A1_BYTES = TG_BM * BK * 2;       // one row tile of a stage
  static constexpr int A_BYTES = MT * A1_BYTES;
  static constexpr int X_BYTES = NCOL * BK * 2;
  static constexpr int STAGE_BYTES = A_BYTES + X_BYTES;
  // as many stages as 225 KB of the 227 KB per CTA hold (at most 8): the bytes in flight hide
  // the latency of the operand loads
  static constexpr int STAGES = (225 * 1024) / STAGE_BYTES > 8 ? 8 : (225 * 1024) / STAGE_BYTES;
  static constexpr int ACC_COLS = MT * NCOL < 32 ? 32 : MT * NCOL;  // one accumulator (all row tiles)
  static constexpr int NACC = 2 * ACC_COLS <= 512 ? 2 : 1;           // double-buffered when TMEM allows
  static constexpr int TMEM_COLS = ACC_COLS * NACC;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 /* align */ + 256 /* barriers */;
  static_assert(NCOL % 16 == 0 && NCOL <= 512 && MT * NCOL <= 512, "NCOL");
  static_assert(STAGES >= 2, "stages");
  static_assert(BK == 32 || BK == 64, "BK");
};

// Work units: (MT row tiles of 128, column block); column block sp covers X rows
// sp * xstride .. + NCOL; mtiles counts groups of MT * 128 rows.  The first big_tiles groups
// run as units of MT row tiles; the rest run one row tile per unit, so that the last wave of
// a persistent grid holds units of half the work (a tail of one-tile units instead of a
// partly filled wave of MT-tile units).  Epilogue interface:
// Epi::row(taddr, row, m0, sp) is called by
// every thread of warps 1-4 with taddr = TMEM address of this thread's accumulator row
// (lane field set, column 0).  With NCOL <= 256 the accumulator is double-buffered in TMEM,
// so one unit's epilogue overlaps the next unit's MMAs.
template <int NCOL, class Epi, int MT = 1, int BK = TG_BK>
__global__ void __launch_bounds__(TG_THREADS, 1)
    k_tensor_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmX, int mtiles,
                  int big_tiles, int ktiles, int nsplit, int xstride, Epi epi, int* err, unsigned long long limit_ns,
                  const int* run_flag) {
  using C = TGCfg<NCOL, MT, BK>;
  if (run_flag && *run_flag == 0) return;  // nothing to compute (every column inactive)
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(smem + C::STAGES * C::STAGE_BYTES);
  uint64_t* full = bars;                     // [STAGES]
  uint64_t* empty = bars + C::STAGES;        // [STAGES]
  uint64_t* accfull = bars + 2 * C::STAGES;  // [2] MMAs of a unit done
  uint64_t* accempty = accfull + 2;          // [2] epilogue of a unit done (4 warp arrivals)
  uint32_t* tmem_slot = (uint32_t*)(accempty + 2);
  volatile int* sabort = (volatile int*)(tmem_slot + 1);
  const int nbig = big_tiles * nsplit;
  const int units = nbig + (mtiles - big_tiles) * MT * nsplit;
  // unit u -> first row tile, row tiles in the unit, column block
  auto decode = [&](int u, int& rt0, int& mtu, int& sp) {
    if (u < nbig) {
      rt0 = (u / nsplit) * MT;
      mtu = MT;
      sp = u % nsplit;
    } else {
      const int v = u - nbig;
      rt0 = big_tiles * MT + v / nsplit;
      mtu = 1;
      sp = v % nsplit;
    }
  };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < C::STAGES; ++s) {
      umma::mbar_init(&full[s], 1);
      umma::mbar_init(&empty[s], 1);
    }
    for (int q = 0; q < 2; ++q) {
      umma::mbar_init(&accfull[q], 1);
      umma::mbar_init(&accempty[q], 4);
    }
    *sabort = 0;
    umma::fence_barrier_init();
    umma::prefetch_tmap(&tmA);
    umma::prefetch_tmap(&tmX);
  }
  if (warp == 2) umma::tmem_alloc(tmem_slot, C::TMEM_COLS);  // warp 2 also frees it
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = umma::idesc_bf16_f32(TG_BM, C::NMMA);

  if (warp == 0) {
    // ---------------- TMA producer
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0;
      long long issued = 0;
      for (int u = blockIdx.x; u < units && !*sabort; u += gridDim.x) {
        int rt0, mtu, sp;
        decode(u, rt0, mtu, sp);
        const int xr0 = sp * xstride;
        for (int kt = 0; kt < ktiles; ++kt) {
          if (!umma::mbar_wait(&empty[s], ph ^ 1, limit_ns, sabort)) {
            *sabort = 1;
            break;
          }
          unsigned char* st = smem + s * C::STAGE_BYTES;
          umma::mbar_arrive_expect_tx(&full[s], mtu * C::A1_BYTES + C::X_BYTES);
#pragma unroll
          for (int mt = 0; mt < MT; ++mt)
            if (mt < mtu) umma::tma_load_2d(st + mt * C::A1_BYTES, &tmA, &full[s], kt * BK, (rt0 + mt) * TG_BM);
#pragma unroll
          for (int h = 0; h < (NCOL + 255) / 256; ++h)
            umma::tma_load_2d(st + C::A_BYTES + h * 256 * C::ROWB, &tmX, &full[s], kt * BK, xr0 + h * 256);
          ++issued;
          if (++s == C::STAGES) { s = 0; ph ^= 1; }
        }
      }
      // drain: wait (bounded) until every issued stage has landed, so no copy is in
      // flight when the CTA exits
      int ds = s;
      uint32_t dph = ph;
      for (int q = 0; q < C::STAGES; ++q) {
        if (--ds < 0) { ds = C::STAGES - 1; dph ^= 1; }
        if (issued - q <= 0) break;
        umma::mbar_wait(&full[ds], dph, limit_ns, nullptr);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issue (lane 0): runs ahead of the epilogue by one accumulator
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0;
      uint32_t it = 0;
      for (int u = blockIdx.x; u < units && !*sabort; u += gridDim.x, ++it) {
        int rt0, mtu, sp;
        decode(u, rt0, mtu, sp);
        const uint32_t buf = it % C::NACC, use = it / C::NACC;  // accumulator and its use count
        const uint32_t tacc = tmem + buf * C::ACC_COLS;
        // the accumulator must have been read out by the epilogue of its previous use
        if (!umma::mbar_wait(&accempty[buf], (use & 1) ^ 1, limit_ns, sabort)) {
          *sabort = 1;
          break;
        }
        umma::tc_fence_after();
        for (int kt = 0; kt < ktiles && !*sabort; ++kt) {
          if (!umma::mbar_wait(&full[s], ph, limit_ns, sabort)) {
            *sabort = 1;
            break;
          }
          umma::tc_fence_after();
          const uint32_t a0 = umma::smem_u32(smem + s * C::STAGE_BYTES);
          const uint32_t x0 = a0 + C::A_BYTES;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk) {
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
              if (mt >= mtu) break;
              const uint32_t aa = a0 + mt * C::A1_BYTES + kk * 32;
              const uint64_t ad = BK == 64 ? umma::sw128_desc(aa) : umma::sw64_desc(aa);
#pragma unroll
              for (int h = 0; h < C::NH; ++h) {
                const uint32_t xa = x0 + h * C::NMMA * C::ROWB + kk * 32;
                const uint64_t xd = BK == 64 ? umma::sw128_desc(xa) : umma::sw64_desc(xa);
                umma::mma_bf16(tacc + mt * NCOL + h * C::NMMA, ad, xd, idesc, (kt > 0 || kk > 0) ? 1u : 0u);
              }
            }
          }
          umma::mma_commit(&empty[s]);  // frees the stage once these MMAs have read it
          if (++s == C::STAGES) { s = 0; ph ^= 1; }
        }
        umma::mma_commit(&accfull[buf]);
      }
    }
  } else {
    // ---------------- epilogue (warps 2-5; warp w reads TMEM lanes 32*(w%4)..+31)
    const int q = warp & 3;
    uint32_t it = 0;
    for (int u = blockIdx.x; u < units; u += gridDim.x, ++it) {
      const uint32_t buf = it % C::NACC, use = it / C::NACC;
      bool ok = umma::mbar_wait(&accfull[buf], use & 1, limit_ns, sabort);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) {
        if (lane == 0) *sabort = 1;
        break;
      }
      umma::tc_fence_after();
      const int row = q * 32 + lane;
      int rt0, mtu, sp;
      decode(u, rt0, mtu, sp);
#pragma unroll 1
      for (int mt = 0; mt < mtu; ++mt)
        epi.row(tmem + buf * C::ACC_COLS + mt * NCOL + ((uint32_t)(q * 32) << 16), row, (rt0 + mt) * TG_BM, sp);
      umma::tc_fence_before();
      __syncwarp();
      if (lane == 0) umma::mbar_arrive(&accempty[buf]);
    }
  }
  __syncthreads();
  if (*sabort && threadIdx.x == 0 && err) atomicCAS(err, 0, -4);
  if (warp == 2) {
    umma::tc_fence_after();
    umma::tmem_dealloc(tmem, C::TMEM_COLS);
  }
}

// host: 2-D tensor map of a K-major BF16 matrix [rows][k] (row stride k elements) with a
// (TG_BK x box_rows) box and the 64-byte swizzle.  cuTensorMapEncodeTiled is fetched from
// the driver at run time, so the library does not link libcuda.
typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
inline int make_tmap_bf16(CUtensorMap* map, const void* base, uint64_t k, uint64_t rows, uint32_t box_rows,
                          int bk = TG_BK) {
  static PFN_encodeTiled fn = nullptr;
  if (!fn) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &f, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !f)
      return -1;
    fn = (PFN_encodeTiled)f;
  }
  cuuint64_t dims[2] = {k, rows};
  cuuint64_t strides[1] = {k * 2};
  cuuint32_t box[2] = {(cuuint32_t)bk, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -2;
}

}  // namespace kura
