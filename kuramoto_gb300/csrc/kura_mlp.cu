// kura_mlp.cu -- the order-parameter surrogate: a 4-layer MLP (SiLU, BF16 weights, FP32
// accumulation) trained and evaluated on the GPU by this library's own kernels.
//
// The reference has no learned component.  This network maps features of a Kuramoto run
// (coupling, rank, frequency scale and family, the first samples of r(t)) to the steady
// mean and spread of r, and places coupling-sweep points near the volcano transition.
//
// Every GEMM of the forward and the backward pass runs on tcgen05 through k_tensor_gemm
// (TMA-fed shared memory, FP32 accumulation in TMEM) with its own fused epilogue:
//   forward  Z_l = H_l W_l^T + b_l       A = H_l [B][in], X = W_l [out][in]
//            H_{l+1} = silu(Z_l) (BF16, plus its transpose) and silu'(Z_l) kept for backward
//   weights  dW_l = dZ_l^T H_l            A = dZ_l^T [out][B], X = H_l^T [in][B]
//   inputs   dZ_{l-1} = (dZ_l W_l) * silu'(Z_{l-1})   A = dZ_l [B][out], X = W_l^T [in][out]
// Widths are padded to multiples of 64 (the K tile) with zero weights, which stay zero:
// their gradients vanish.  Adam updates FP32 master weights and rewrites the BF16 copies;
// one whole training step (gather, forward, loss, backward, Adam) is a CUDA graph replayed
// once per step, with the step counter on the device.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "kura.h"
#include "kura_kernels.cuh"
#include "kura_tensor_gemm.cuh"

namespace kura {
namespace {

constexpr int NL = 4;    // linear layers
constexpr int PADW = 64;  // widths padded to the K tile
typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// ---------------------------------------------------------------- GEMM epilogues
// forward: z = acc + b; hidden layers store silu(z) (row-major and transposed, BF16) and
// silu'(z); the last layer stores z
template <int NCOL> struct FwdEpi {
  const float* bias;
  int last, Bt;
  bf16* H;   // [Bt][NCOL]
  bf16* HT;  // [NCOL][Bt]
  float* S;  // [Bt][NCOL]
  float* Y;  // [Bt][NCOL]
  __device__ void row(uint32_t taddr, int row, int m0, int) {
    const int r = m0 + row;
#pragma unroll 1
    for (int c0 = 0; c0 < NCOL; c0 += 16) {
      float a[16];
      umma::tmem_ld16(taddr + c0, a);
      umma::tmem_ld_wait();
      float z[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) z[j] = a[j] + bias[c0 + j];
      if (last) {
        float4* y = reinterpret_cast<float4*>(Y + (size_t)r * NCOL + c0);
#pragma unroll
        for (int q = 0; q < 4; ++q) y[q] = make_float4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
        continue;
      }
      float h[16], d[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const float s = 1.f / (1.f + expf(-z[j]));
        h[j] = z[j] * s;
        d[j] = s * (1.f + z[j] * (1.f - s));
      }
      uint4* hp = reinterpret_cast<uint4*>(H + (size_t)r * NCOL + c0);
      hp[0] = make_uint4(pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]), pack_bf16(h[4], h[5]), pack_bf16(h[6], h[7]));
      hp[1] = make_uint4(pack_bf16(h[8], h[9]), pack_bf16(h[10], h[11]), pack_bf16(h[12], h[13]),
                         pack_bf16(h[14], h[15]));
#pragma unroll
      for (int j = 0; j < 16; ++j) HT[(size_t)(c0 + j) * Bt + r] = __float2bfloat16_rn(h[j]);
      float4* sp = reinterpret_cast<float4*>(S + (size_t)r * NCOL + c0);
#pragma unroll
      for (int q = 0; q < 4; ++q) sp[q] = make_float4(d[4 * q], d[4 * q + 1], d[4 * q + 2], d[4 * q + 3]);
    }
  }
};

// weight gradient: rows are output units; rows beyond the padded width are not stored
template <int NCOL> struct DwEpi {
  float* G;  // [out_p][NCOL]
  int out_p;
  __device__ void row(uint32_t taddr, int row, int m0, int) {
    const int r = m0 + row;
#pragma unroll 1
    for (int c0 = 0; c0 < NCOL; c0 += 16) {
      float a[16];
      umma::tmem_ld16(taddr + c0, a);
      umma::tmem_ld_wait();
      if (r >= out_p) continue;
      float4* g = reinterpret_cast<float4*>(G + (size_t)r * NCOL + c0);
#pragma unroll
      for (int q = 0; q < 4; ++q) g[q] = make_float4(a[4 * q], a[4 * q + 1], a[4 * q + 2], a[4 * q + 3]);
    }
  }
};

// input gradient of a hidden layer: dZ_{l-1} = (dZ_l W_l) * silu'(Z_{l-1}), BF16, both layouts
template <int NCOL> struct DhEpi {
  const float* S;  // [Bt][NCOL]
  bf16* dZ;        // [Bt][NCOL]
  bf16* dZT;       // [NCOL][Bt]
  int Bt;
  __device__ void row(uint32_t taddr, int row, int m0, int) {
    const int r = m0 + row;
#pragma unroll 1
    for (int c0 = 0; c0 < NCOL; c0 += 16) {
      float a[16];
      umma::tmem_ld16(taddr + c0, a);
      umma::tmem_ld_wait();
      const float4* sp = reinterpret_cast<const float4*>(S + (size_t)r * NCOL + c0);
      float d[16];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 s = sp[q];
        d[4 * q] = a[4 * q] * s.x;
        d[4 * q + 1] = a[4 * q + 1] * s.y;
        d[4 * q + 2] = a[4 * q + 2] * s.z;
        d[4 * q + 3] = a[4 * q + 3] * s.w;
      }
      uint4* dp = reinterpret_cast<uint4*>(dZ + (size_t)r * NCOL + c0);
      dp[0] = make_uint4(pack_bf16(d[0], d[1]), pack_bf16(d[2], d[3]), pack_bf16(d[4], d[5]), pack_bf16(d[6], d[7]));
      dp[1] = make_uint4(pack_bf16(d[8], d[9]), pack_bf16(d[10], d[11]), pack_bf16(d[12], d[13]),
                         pack_bf16(d[14], d[15]));
#pragma unroll
      for (int j = 0; j < 16; ++j) dZT[(size_t)(c0 + j) * Bt + r] = __float2bfloat16_rn(d[j]);
    }
  }
};

// ---------------------------------------------------------------- small kernels
// minibatch rows of the dataset (training) or of a caller's chunk (idx == null): BF16 input
// rows and their transpose, FP32 targets; rows >= nvalid are zero
__global__ void k_mlp_gather(const float* __restrict__ X, const float* __restrict__ T, const int* __restrict__ idx,
                             const int* counter, int in_dim, int out_dim, int out_p, int Bt, int nvalid, bf16* H0,
                             bf16* HT0, float* Tb) {
  const int step = counter ? *counter : 0;
  const int total = Bt * PADW;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int c = t / Bt, r = t % Bt;  // c-major: the transposed store is coalesced
    float v = 0.f;
    long long src = -1;
    if (r < nvalid) src = idx ? (long long)idx[(long long)step * Bt + r] : (long long)r;
    if (src >= 0 && c < in_dim) v = X[src * in_dim + c];
    const bf16 b = __float2bfloat16_rn(v);
    HT0[(size_t)c * Bt + r] = b;
    H0[(size_t)r * PADW + c] = b;
    if (c < out_p) Tb[(size_t)r * out_p + c] = (src >= 0 && c < out_dim && T) ? T[src * out_dim + c] : 0.f;
  }
}

// mean squared error over the valid rows and the first out_dim outputs; its gradient
// 2 (y - t) / (n out_dim) in both layouts (BF16)
__global__ void k_mlp_loss(const float* __restrict__ Y, const float* __restrict__ Tb, int nvalid, int out_dim,
                           int out_p, int Bt, bf16* dZ, bf16* dZT, float* loss, const int* counter) {
  __shared__ float red[32];
  const float scale = 2.f / ((float)nvalid * (float)out_dim);
  float acc = 0.f;
  for (int t = threadIdx.x; t < Bt * out_p; t += blockDim.x) {
    const int j = t / Bt, r = t % Bt;
    float g = 0.f;
    if (r < nvalid && j < out_dim) {
      const float e = Y[(size_t)r * out_p + j] - Tb[(size_t)r * out_p + j];
      acc = fmaf(e, e, acc);
      g = scale * e;
    }
    const bf16 b = __float2bfloat16_rn(g);
    dZ[(size_t)r * out_p + j] = b;
    dZT[(size_t)j * Bt + r] = b;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    loss[counter ? *counter : 0] = s / ((float)nvalid * (float)out_dim);
  }
}

// bias gradient: column sums of dZ in row order (deterministic)
__global__ void k_mlp_bias_grad(const bf16* __restrict__ dZ, int Bt, int out_p, float* gb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= out_p) return;
  float s = 0.f;
  for (int r = 0; r < Bt; ++r) s += __bfloat162float(dZ[(size_t)r * out_p + c]);
  gb[c] = s;
}

// Adam on the flat FP32 parameters (Kingma & Ba), learning rate interpolated linearly from
// lr0 to lr1 over the run; the step number comes from the device counter
__global__ void k_mlp_adam(float* P, const float* __restrict__ G, float* M, float* V, long long n, const int* counter,
                           float lr0, float lr1, long long total_steps, float b1, float b2, float eps) {
  const int step = *counter;
  const float frac = total_steps > 1 ? (float)step / (float)(total_steps - 1) : 0.f;
  const float lr = lr0 + (lr1 - lr0) * frac;
  const float c1 = 1.f - powf(b1, (float)(step + 1)), c2 = 1.f - powf(b2, (float)(step + 1));
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float g = G[i];
    const float m = b1 * M[i] + (1.f - b1) * g;
    const float v = b2 * V[i] + (1.f - b2) * g * g;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
  }
}

struct PackLayer {
  long long w_off;
  int in_p, out_p;
  bf16* W;
  bf16* WT;
};
struct PackArgs {
  PackLayer l[NL];
};
// BF16 copies of the weights, [out][in] and [in][out]; optionally advances the step counter
__global__ void k_mlp_pack(const float* __restrict__ P, PackArgs a, int* counter) {
  const PackLayer& L = a.l[blockIdx.y];
  const int total = L.in_p * L.out_p;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int o = t / L.in_p, i = t % L.in_p;
    const bf16 b = __float2bfloat16_rn(P[L.w_off + t]);
    L.W[t] = b;
    L.WT[(size_t)i * L.out_p + o] = b;
  }
  if (counter && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) atomicAdd(counter, 1);
}

struct Layer {
  int in, out, in_p, out_p, out_m;  // out_m: rows of dZ^T (at least one 128-row M tile)
  long long w_off, b_off;
};

int round_up(int x, int m) { return (x + m - 1) / m * m; }

uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform01(uint64_t& s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace
}  // namespace kura

using kura::bf16;
using kura::Layer;
using kura::NL;
using kura::PADW;

struct kura_mlp {
  int device = 0, in_dim = 0, hidden = 0, out_dim = 0, Bt = 0, sms = 0;
  Layer L[NL];
  long long nparam = 0;  // padded flat size
  float *P = nullptr, *G = nullptr, *Mo = nullptr, *Vo = nullptr;
  bf16 *W[NL] = {}, *WT[NL] = {};
  bf16 *H[NL] = {}, *HT[NL] = {};  // input of layer l
  float* S[NL] = {};               // silu'(Z_{l-1}), the derivative at the input of layer l (l >= 1)
  float* Y = nullptr;
  bf16 *dZ[NL] = {}, *dZT[NL] = {};  // gradient at the output of layer l
  float *Tb = nullptr, *loss = nullptr, *Xin = nullptr, *Tin = nullptr;
  int *counter = nullptr, *err = nullptr;
  CUtensorMap fA[NL], fX[NL], wA[NL], wX[NL], hA[NL], hX[NL];
  cudaStream_t st = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  std::vector<void*> allocs;
};

namespace {

int mlp_fail(int code, const std::string& msg) {
  kura::set_last_error(msg.c_str());
  return code;
}
#define MLPCU(x)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (x);                                                                         \
    if (e_ != cudaSuccess)                                                                        \
      return mlp_fail(e_ == cudaErrorMemoryAllocation ? KURA_ERR_NOMEM : KURA_ERR_CUDA,           \
                      std::string(#x) + ": " + cudaGetErrorString(e_));                          \
  } while (0)

template <class T>
cudaError_t dalloc(kura_mlp* m, T** p, size_t count) {
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(count, 1));
  if (e == cudaSuccess) {
    m->allocs.push_back(*p);
    e = cudaMemset(*p, 0, sizeof(T) * std::max<size_t>(count, 1));
    // the zero-fill runs on the legacy default stream, unordered with a non-blocking stream
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  }
  return e;
}

constexpr unsigned long long GEMM_LIMIT_NS = 20000000000ull;

template <int NCOL, class Epi>
cudaError_t gemm(kura_mlp* m, const CUtensorMap& a, const CUtensorMap& x, int mtiles, int ktiles, const Epi& e) {
  kura::k_tensor_gemm<NCOL, Epi><<<std::min(mtiles, m->sms), kura::TG_THREADS, kura::TGCfg<NCOL>::SMEM, m->st>>>(
      a, x, mtiles, mtiles, ktiles, 1, 0, e, m->err, GEMM_LIMIT_NS, nullptr);
  return cudaGetLastError();
}

template <int NCOL>
cudaError_t set_attrs_n() {
  cudaError_t e = cudaFuncSetAttribute(kura::k_tensor_gemm<NCOL, kura::FwdEpi<NCOL>>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, kura::TGCfg<NCOL>::SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kura::k_tensor_gemm<NCOL, kura::DwEpi<NCOL>>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kura::TGCfg<NCOL>::SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kura::k_tensor_gemm<NCOL, kura::DhEpi<NCOL>>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kura::TGCfg<NCOL>::SMEM);
  return e;
}

// dispatch on a padded width (64, 128, 256)
template <class F>
cudaError_t by_width(int w, F&& f) {
  switch (w) {
    case 64: return f(std::integral_constant<int, 64>());
    case 128: return f(std::integral_constant<int, 128>());
    case 256: return f(std::integral_constant<int, 256>());
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t forward(kura_mlp* m) {
  for (int l = 0; l < NL; ++l) {
    const Layer& L = m->L[l];
    const bool last = (l == NL - 1);
    cudaError_t e = by_width(L.out_p, [&](auto w) {
      constexpr int W = decltype(w)::value;
      kura::FwdEpi<W> ep{m->P + L.b_off, last ? 1 : 0, m->Bt, last ? nullptr : m->H[l + 1],
                         last ? nullptr : m->HT[l + 1], last ? nullptr : m->S[l + 1], last ? m->Y : nullptr};
      return gemm<W>(m, m->fA[l], m->fX[l], m->Bt / kura::TG_BM, L.in_p / kura::TG_BK, ep);
    });
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t backward(kura_mlp* m) {
  for (int l = NL - 1; l >= 0; --l) {
    const Layer& L = m->L[l];
    cudaError_t e = by_width(L.in_p, [&](auto w) {
      constexpr int W = decltype(w)::value;
      kura::DwEpi<W> ep{m->G + L.w_off, L.out_p};
      return gemm<W>(m, m->wA[l], m->wX[l], L.out_m / kura::TG_BM, m->Bt / kura::TG_BK, ep);
    });
    if (e != cudaSuccess) return e;
    kura::k_mlp_bias_grad<<<(L.out_p + 127) / 128, 128, 0, m->st>>>(m->dZ[l], m->Bt, L.out_p, m->G + L.b_off);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (l == 0) break;
    e = by_width(L.in_p, [&](auto w) {
      constexpr int W = decltype(w)::value;
      kura::DhEpi<W> ep{m->S[l], m->dZ[l - 1], m->dZT[l - 1], m->Bt};
      return gemm<W>(m, m->hA[l], m->hX[l], m->Bt / kura::TG_BM, L.out_p / kura::TG_BK, ep);
    });
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

kura::PackArgs pack_args(kura_mlp* m) {
  kura::PackArgs a;
  for (int l = 0; l < NL; ++l) a.l[l] = {m->L[l].w_off, m->L[l].in_p, m->L[l].out_p, m->W[l], m->WT[l]};
  return a;
}

cudaError_t pack(kura_mlp* m, int* counter) {
  kura::k_mlp_pack<<<dim3(64, NL), 256, 0, m->st>>>(m->P, pack_args(m), counter);
  return cudaGetLastError();
}

int check_err(kura_mlp* m) {
  int e = 0;
  MLPCU(cudaMemcpy(&e, m->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e != 0) {
    cudaMemset(m->err, 0, sizeof(int));
    cudaStreamSynchronize(0);
    return mlp_fail(KURA_ERR_BARRIER_TIMEOUT, "a tensor-core GEMM of the MLP timed out waiting for its operands");
  }
  return KURA_OK;
}

// unpadded parameter order: per layer W [out][in] row-major, then b [out]
long long public_count(const kura_mlp* m) {
  long long c = 0;
  for (const Layer& L : m->L) c += (long long)L.out * L.in + L.out;
  return c;
}
void to_public(const kura_mlp* m, const std::vector<float>& pad, float* out) {
  long long k = 0;
  for (const Layer& L : m->L) {
    for (int o = 0; o < L.out; ++o)
      for (int i = 0; i < L.in; ++i) out[k++] = pad[L.w_off + (long long)o * L.in_p + i];
    for (int o = 0; o < L.out; ++o) out[k++] = pad[L.b_off + o];
  }
}

}  // namespace

extern "C" int kura_mlp_create(int32_t in_dim, int32_t hidden, int32_t out_dim, int32_t batch, uint64_t seed,
                               int32_t device, kura_mlp** out) {
  if (!out) return mlp_fail(KURA_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (in_dim < 1 || in_dim > PADW) return mlp_fail(KURA_ERR_UNSUPPORTED, "in_dim must be 1..64");
  if (out_dim < 1 || out_dim > PADW) return mlp_fail(KURA_ERR_UNSUPPORTED, "out_dim must be 1..64");
  if (hidden != 64 && hidden != 128 && hidden != 256) return mlp_fail(KURA_ERR_UNSUPPORTED, "hidden must be 64, 128 or 256");
  if (batch < 128 || batch > 4096 || batch % 128) return mlp_fail(KURA_ERR_UNSUPPORTED, "batch must be a multiple of 128 in 128..4096");
  kura_mlp* m = new kura_mlp();
  m->device = device;
  m->in_dim = in_dim;
  m->hidden = hidden;
  m->out_dim = out_dim;
  m->Bt = batch;
  const int dims[NL + 1] = {in_dim, hidden, hidden, hidden, out_dim};
  long long off = 0;
  for (int l = 0; l < NL; ++l) {
    Layer& L = m->L[l];
    L.in = dims[l];
    L.out = dims[l + 1];
    L.in_p = kura::round_up(L.in, PADW);
    L.out_p = kura::round_up(L.out, PADW);
    L.out_m = std::max(L.out_p, kura::TG_BM);
    L.w_off = off;
    off += (long long)L.out_p * L.in_p;
    L.b_off = off;
    off += L.out_p;
  }
  m->nparam = off;
  auto bail = [&](int rc) {
    kura_mlp_destroy(m);
    return rc;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, device);
  const int Bt = batch;
  if (e == cudaSuccess) e = dalloc(m, &m->P, off);
  if (e == cudaSuccess) e = dalloc(m, &m->G, off);
  if (e == cudaSuccess) e = dalloc(m, &m->Mo, off);
  if (e == cudaSuccess) e = dalloc(m, &m->Vo, off);
  for (int l = 0; l < NL && e == cudaSuccess; ++l) {
    const Layer& L = m->L[l];
    e = dalloc(m, &m->W[l], (size_t)L.out_p * L.in_p);
    if (e == cudaSuccess) e = dalloc(m, &m->WT[l], (size_t)L.out_p * L.in_p);
    if (e == cudaSuccess) e = dalloc(m, &m->H[l], (size_t)Bt * L.in_p);
    if (e == cudaSuccess) e = dalloc(m, &m->HT[l], (size_t)Bt * L.in_p);
    if (e == cudaSuccess && l > 0) e = dalloc(m, &m->S[l], (size_t)Bt * L.in_p);
    if (e == cudaSuccess) e = dalloc(m, &m->dZ[l], (size_t)Bt * L.out_p);
    if (e == cudaSuccess) e = dalloc(m, &m->dZT[l], (size_t)Bt * L.out_m);
  }
  if (e == cudaSuccess) e = dalloc(m, &m->Y, (size_t)Bt * m->L[NL - 1].out_p);
  if (e == cudaSuccess) e = dalloc(m, &m->Tb, (size_t)Bt * m->L[NL - 1].out_p);
  if (e == cudaSuccess) e = dalloc(m, &m->Xin, (size_t)Bt * in_dim);
  if (e == cudaSuccess) e = dalloc(m, &m->Tin, (size_t)Bt * out_dim);
  if (e == cudaSuccess) e = dalloc(m, &m->loss, 1);
  if (e == cudaSuccess) e = dalloc(m, &m->counter, 1);
  if (e == cudaSuccess) e = dalloc(m, &m->err, 1);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&m->ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&m->ev[1]);
  if (e == cudaSuccess) e = set_attrs_n<64>();
  if (e == cudaSuccess) e = set_attrs_n<128>();
  if (e == cudaSuccess) e = set_attrs_n<256>();
  if (e != cudaSuccess)
    return bail(mlp_fail(e == cudaErrorMemoryAllocation ? KURA_ERR_NOMEM : KURA_ERR_CUDA, cudaGetErrorString(e)));
  // tensor maps of every GEMM operand (the buffers never move)
  for (int l = 0; l < NL; ++l) {
    const Layer& L = m->L[l];
    int bad = kura::make_tmap_bf16(&m->fA[l], m->H[l], L.in_p, Bt, kura::TG_BM);
    bad |= kura::make_tmap_bf16(&m->fX[l], m->W[l], L.in_p, L.out_p, std::min(256, L.out_p));
    bad |= kura::make_tmap_bf16(&m->wA[l], m->dZT[l], Bt, L.out_m, kura::TG_BM);
    bad |= kura::make_tmap_bf16(&m->wX[l], m->HT[l], Bt, L.in_p, std::min(256, L.in_p));
    if (l > 0) {
      bad |= kura::make_tmap_bf16(&m->hA[l], m->dZ[l], L.out_p, Bt, kura::TG_BM);
      bad |= kura::make_tmap_bf16(&m->hX[l], m->WT[l], L.out_p, L.in_p, std::min(256, L.in_p));
    }
    if (bad) return bail(mlp_fail(KURA_ERR_CUDA, "cuTensorMapEncodeTiled failed for an MLP operand"));
  }
  // Glorot-uniform weights from a seeded splitmix64 stream, zero biases and padding
  std::vector<float> p(off, 0.f);
  uint64_t s = seed;
  for (const Layer& L : m->L) {
    const double a = std::sqrt(6.0 / (double)(L.in + L.out));
    for (int o = 0; o < L.out; ++o)
      for (int i = 0; i < L.in; ++i) p[L.w_off + (long long)o * L.in_p + i] = (float)((2 * kura::uniform01(s) - 1) * a);
  }
  e = cudaMemcpy(m->P, p.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = pack(m, nullptr);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
  if (e != cudaSuccess) return bail(mlp_fail(KURA_ERR_CUDA, cudaGetErrorString(e)));
  *out = m;
  return KURA_OK;
}

extern "C" void kura_mlp_destroy(kura_mlp* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  if (m->st) cudaStreamSynchronize(m->st);
  for (void* p : m->allocs) cudaFree(p);
  for (cudaEvent_t v : m->ev)
    if (v) cudaEventDestroy(v);
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
}

extern "C" int kura_mlp_param_count(const kura_mlp* m, int64_t* count) {
  if (!m || !count) return mlp_fail(KURA_ERR_INVALID, "NULL argument");
  *count = public_count(m);
  return KURA_OK;
}

extern "C" int kura_mlp_get_params(kura_mlp* m, float* params, int64_t count) {
  if (!m || !params) return mlp_fail(KURA_ERR_INVALID, "NULL argument");
  if (count != public_count(m)) return mlp_fail(KURA_ERR_INVALID, "count must equal kura_mlp_param_count");
  MLPCU(cudaSetDevice(m->device));
  std::vector<float> pad(m->nparam);
  MLPCU(cudaStreamSynchronize(m->st));
  MLPCU(cudaMemcpy(pad.data(), m->P, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost));
  to_public(m, pad, params);
  return KURA_OK;
}

extern "C" int kura_mlp_set_params(kura_mlp* m, const float* params, int64_t count) {
  if (!m || !params) return mlp_fail(KURA_ERR_INVALID, "NULL argument");
  if (count != public_count(m)) return mlp_fail(KURA_ERR_INVALID, "count must equal kura_mlp_param_count");
  MLPCU(cudaSetDevice(m->device));
  std::vector<float> pad(m->nparam, 0.f);
  long long k = 0;
  for (const Layer& L : m->L) {
    for (int o = 0; o < L.out; ++o)
      for (int i = 0; i < L.in; ++i) pad[L.w_off + (long long)o * L.in_p + i] = params[k++];
    for (int o = 0; o < L.out; ++o) pad[L.b_off + o] = params[k++];
  }
  MLPCU(cudaStreamSynchronize(m->st));
  MLPCU(cudaMemcpy(m->P, pad.data(), sizeof(float) * m->nparam, cudaMemcpyHostToDevice));
  MLPCU(pack(m, nullptr));
  MLPCU(cudaStreamSynchronize(m->st));
  return KURA_OK;
}

extern "C" int kura_mlp_forward(kura_mlp* m, const float* x, int64_t n, float* y) {
  if (!m || !x || !y || n < 0) return mlp_fail(KURA_ERR_INVALID, "bad argument");
  MLPCU(cudaSetDevice(m->device));
  const Layer& Lo = m->L[NL - 1];
  for (int64_t r0 = 0; r0 < n; r0 += m->Bt) {
    const int rows = (int)std::min<int64_t>(m->Bt, n - r0);
    MLPCU(cudaMemcpyAsync(m->Xin, x + r0 * m->in_dim, sizeof(float) * rows * m->in_dim, cudaMemcpyHostToDevice, m->st));
    kura::k_mlp_gather<<<64, 256, 0, m->st>>>(m->Xin, nullptr, nullptr, nullptr, m->in_dim, m->out_dim, Lo.out_p,
                                              m->Bt, rows, m->H[0], m->HT[0], m->Tb);
    MLPCU(cudaGetLastError());
    MLPCU(forward(m));
    MLPCU(cudaMemcpy2DAsync(y + r0 * m->out_dim, sizeof(float) * m->out_dim, m->Y, sizeof(float) * Lo.out_p,
                            sizeof(float) * m->out_dim, rows, cudaMemcpyDeviceToHost, m->st));
    MLPCU(cudaStreamSynchronize(m->st));
    int rc = check_err(m);
    if (rc != KURA_OK) return rc;
  }
  return KURA_OK;
}

extern "C" int kura_mlp_gradients(kura_mlp* m, const float* x, const float* target, int64_t n, float* grads,
                                  float* loss) {
  if (!m || !x || !target || !grads) return mlp_fail(KURA_ERR_INVALID, "NULL argument");
  if (n < 1 || n > m->Bt) return mlp_fail(KURA_ERR_INVALID, "n must be 1..batch");
  MLPCU(cudaSetDevice(m->device));
  const Layer& Lo = m->L[NL - 1];
  MLPCU(cudaMemcpyAsync(m->Xin, x, sizeof(float) * n * m->in_dim, cudaMemcpyHostToDevice, m->st));
  MLPCU(cudaMemcpyAsync(m->Tin, target, sizeof(float) * n * m->out_dim, cudaMemcpyHostToDevice, m->st));
  kura::k_mlp_gather<<<64, 256, 0, m->st>>>(m->Xin, m->Tin, nullptr, nullptr, m->in_dim, m->out_dim, Lo.out_p, m->Bt,
                                            (int)n, m->H[0], m->HT[0], m->Tb);
  MLPCU(cudaGetLastError());
  MLPCU(forward(m));
  kura::k_mlp_loss<<<1, 1024, 0, m->st>>>(m->Y, m->Tb, (int)n, m->out_dim, Lo.out_p, m->Bt, m->dZ[NL - 1],
                                          m->dZT[NL - 1], m->loss, nullptr);
  MLPCU(cudaGetLastError());
  MLPCU(backward(m));
  std::vector<float> pad(m->nparam);
  float l = 0.f;
  MLPCU(cudaStreamSynchronize(m->st));
  int rc = check_err(m);
  if (rc != KURA_OK) return rc;
  MLPCU(cudaMemcpy(pad.data(), m->G, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost));
  MLPCU(cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
  to_public(m, pad, grads);
  if (loss) *loss = l;
  return KURA_OK;
}

extern "C" int kura_mlp_train(kura_mlp* m, const float* x, const float* target, int64_t n_samples, int32_t epochs,
                              float lr, float lr_final, uint64_t shuffle_seed, float* epoch_loss, double* device_ms) {
  if (!m || !x || !target) return mlp_fail(KURA_ERR_INVALID, "NULL argument");
  if (n_samples < m->Bt) return mlp_fail(KURA_ERR_INVALID, "need at least one full batch of samples");
  if (epochs < 1) return mlp_fail(KURA_ERR_INVALID, "epochs must be >= 1");
  MLPCU(cudaSetDevice(m->device));
  const Layer& Lo = m->L[NL - 1];
  const long long per_epoch = n_samples / m->Bt;
  const long long total = per_epoch * epochs;
  // the minibatch rows of every step: one shuffle per epoch (Fisher-Yates on splitmix64)
  std::vector<int> idx((size_t)total * m->Bt);
  std::vector<int> perm(n_samples);
  uint64_t s = shuffle_seed;
  for (int ep = 0; ep < epochs; ++ep) {
    for (long long i = 0; i < n_samples; ++i) perm[i] = (int)i;
    for (long long i = n_samples - 1; i > 0; --i) {
      const long long j = (long long)(kura::splitmix64(s) % (uint64_t)(i + 1));
      std::swap(perm[i], perm[j]);
    }
    std::memcpy(&idx[(size_t)ep * per_epoch * m->Bt], perm.data(), sizeof(int) * per_epoch * m->Bt);
  }
  float *dX = nullptr, *dT = nullptr, *dL = nullptr;
  int* dI = nullptr;
  int rc = KURA_OK;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  auto run = [&]() -> int {
    MLPCU(cudaMalloc((void**)&dX, sizeof(float) * n_samples * m->in_dim));
    MLPCU(cudaMalloc((void**)&dT, sizeof(float) * n_samples * m->out_dim));
    MLPCU(cudaMalloc((void**)&dI, sizeof(int) * idx.size()));
    MLPCU(cudaMalloc((void**)&dL, sizeof(float) * total));
    MLPCU(cudaMemcpyAsync(dX, x, sizeof(float) * n_samples * m->in_dim, cudaMemcpyHostToDevice, m->st));
    MLPCU(cudaMemcpyAsync(dT, target, sizeof(float) * n_samples * m->out_dim, cudaMemcpyHostToDevice, m->st));
    MLPCU(cudaMemcpyAsync(dI, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, m->st));
    // fresh Adam state
    MLPCU(cudaMemsetAsync(m->Mo, 0, sizeof(float) * m->nparam, m->st));
    MLPCU(cudaMemsetAsync(m->Vo, 0, sizeof(float) * m->nparam, m->st));
    MLPCU(cudaMemsetAsync(m->counter, 0, sizeof(int), m->st));
    MLPCU(cudaStreamSynchronize(m->st));
    // one training step, captured
    MLPCU(cudaStreamBeginCapture(m->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    kura::k_mlp_gather<<<64, 256, 0, m->st>>>(dX, dT, dI, m->counter, m->in_dim, m->out_dim, Lo.out_p, m->Bt, m->Bt,
                                              m->H[0], m->HT[0], m->Tb);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = forward(m);
    if (e == cudaSuccess) {
      kura::k_mlp_loss<<<1, 1024, 0, m->st>>>(m->Y, m->Tb, m->Bt, m->out_dim, Lo.out_p, m->Bt, m->dZ[NL - 1],
                                              m->dZT[NL - 1], dL, m->counter);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = backward(m);
    if (e == cudaSuccess) {
      kura::k_mlp_adam<<<160, 256, 0, m->st>>>(m->P, m->G, m->Mo, m->Vo, m->nparam, m->counter, lr, lr_final, total,
                                               0.9f, 0.999f, 1e-8f);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = pack(m, m->counter);
    cudaError_t ce = cudaStreamEndCapture(m->st, &g);
    MLPCU(e);
    MLPCU(ce);
    MLPCU(cudaGraphInstantiate(&ge, g, 0));
    MLPCU(cudaEventRecord(m->ev[0], m->st));
    for (long long i = 0; i < total; ++i) MLPCU(cudaGraphLaunch(ge, m->st));
    MLPCU(cudaEventRecord(m->ev[1], m->st));
    MLPCU(cudaStreamSynchronize(m->st));
    int r = check_err(m);
    if (r != KURA_OK) return r;
    float ms = 0.f;
    MLPCU(cudaEventElapsedTime(&ms, m->ev[0], m->ev[1]));
    if (device_ms) *device_ms = ms;
    if (epoch_loss) {
      std::vector<float> lh(total);
      MLPCU(cudaMemcpy(lh.data(), dL, sizeof(float) * total, cudaMemcpyDeviceToHost));
      for (int ep = 0; ep < epochs; ++ep) {
        double a = 0;
        for (long long i = 0; i < per_epoch; ++i) a += lh[(size_t)ep * per_epoch + i];
        epoch_loss[ep] = (float)(a / per_epoch);
      }
    }
    return KURA_OK;
  };
  rc = run();
  if (rc != KURA_OK) cudaGetLastError();
  if (ge) cudaGraphExecDestroy(ge);
  if (g) cudaGraphDestroy(g);
  cudaStreamSynchronize(m->st);
  for (void* p : {(void*)dX, (void*)dT, (void*)dI, (void*)dL})
    if (p) cudaFree(p);
  return rc;
}
