// kura_device.cuh -- device arithmetic shared by the integrator engines: the
// Dormand-Prince tableau, float-pair (error-free) arithmetic, phase reduction and
// wrapping, sin/cos of a float pair, and the Philox4x32-10 counter generator.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace kura {

// ------------------------------------------------------------------ tableau
// Dormand-Prince 5(4) weights, nodes, error weights and the 4th-order continuous
// extension (the same rationals as dp45.cu:6-21).  Row s-1 of A_TAB holds the
// weights of k_1..k_{s-1} for stage s; row 6 is the 5th-order solution b.
static __constant__ double A_TAB[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {1.0 / 5, 0, 0, 0, 0, 0},
    {3.0 / 40, 9.0 / 40, 0, 0, 0, 0},
    {44.0 / 45, -56.0 / 15, 32.0 / 9, 0, 0, 0},
    {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729, 0, 0},
    {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656, 0},
    {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84}};
static __constant__ double C_TAB[7] = {0.0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1.0, 1.0};
static __constant__ double E_TAB[7] = {-71.0 / 57600, 0, 71.0 / 16695, -71.0 / 1920, 17253.0 / 339200, -22.0 / 525,
                                1.0 / 40};
static __constant__ double P_TAB[7][4] = {
    {1.0, -8048581381.0 / 2820520608, 8663915743.0 / 2820520608, -12715105075.0 / 11282082432},
    {0, 0, 0, 0},
    {0, 131558114200.0 / 32700410799, -68118460800.0 / 10900136933, 87487479700.0 / 32700410799},
    {0, -1754552775.0 / 470086768, 14199869525.0 / 1410260304, -10690763975.0 / 1880347072},
    {0, 127303824393.0 / 49829197408, -318862633887.0 / 49829197408, 701980252875.0 / 199316789632},
    {0, -282668133.0 / 205662961, 2019193451.0 / 616988883, -1453857185.0 / 822651844},
    {0, 40617522.0 / 29380423, -110615467.0 / 29380423, 69997945.0 / 29380423}};

// ------------------------------------------------------------------ float-pair arithmetic
struct f2 { float hi, lo; };
__device__ __forceinline__ f2 two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ f2 two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

// 2*pi = P2_1 + P2_2 + P2_3 (Cody-Waite split).  With an FMA, hi - k*P2_1 is exact
// for |k| < 2^24, because both operands are multiples of ulp(P2_1) near the result.
constexpr double TWO_PI_D = 6.283185307179586476925286766559;
constexpr float P2_1 = (float)TWO_PI_D;
constexpr float P2_2 = (float)(TWO_PI_D - (double)P2_1);
constexpr float P2_3 = (float)(TWO_PI_D - (double)P2_1 - (double)P2_2);
constexpr float INV_2PI = (float)(1.0 / TWO_PI_D);

__device__ __forceinline__ float reduce_arg(float hi, float lo) {
  float k = rintf(hi * INV_2PI);
  float r = __fmaf_rn(-k, P2_1, hi);
  r = __fmaf_rn(-k, P2_2, r);
  return __fadd_rn(r, __fmaf_rn(-k, P2_3, lo));
}
__device__ __forceinline__ void wrap_phase(float& hi, float& lo, long long& w) {
  float k = rintf(hi * INV_2PI);
  if (k != 0.f) {
    float h2 = __fmaf_rn(-k, P2_1, hi);
    float l2 = __fadd_rn(lo, __fmaf_rn(-k, P2_2, __fmul_rn(-k, P2_3)));
    f2 s = two_sum(h2, l2);
    hi = s.hi;
    lo = s.lo;
    w += (long long)k;
  }
}

// sin and cos of hi + lo.  Cody-Waite reduction by pi/2 (three-part constant; the
// first FMA is exact for |q| < 2^24) to r in about [-pi/4, pi/4], then the Taylor
// series of sin (to r^9) and cos (to r^10) in Horner form: truncation error below
// 2e-9 at |r| = pi/4, total error about 1e-7 absolute.
constexpr double PIO2_D = 1.5707963267948966192313216916398;
constexpr float PO2_1 = (float)PIO2_D;
constexpr float PO2_2 = (float)(PIO2_D - (double)PO2_1);
constexpr float PO2_3 = (float)(PIO2_D - (double)PO2_1 - (double)PO2_2);
constexpr float TWO_OVER_PI = (float)(1.0 / PIO2_D);
__device__ __forceinline__ void sincos_pair(float hi, float lo, float* sn, float* cs) {
  float q = rintf(hi * TWO_OVER_PI);
  float r = __fmaf_rn(-q, PO2_1, hi);
  r = __fmaf_rn(-q, PO2_2, r);
  r = __fadd_rn(r, __fmaf_rn(-q, PO2_3, lo));
  const int quad = ((int)q) & 3;
  const float r2 = r * r;
  float ps = __fmaf_rn(r2, (float)(1.0 / 362880), (float)(-1.0 / 5040));
  ps = __fmaf_rn(r2, ps, (float)(1.0 / 120));
  ps = __fmaf_rn(r2, ps, (float)(-1.0 / 6));
  ps = __fmaf_rn(r * r2, ps, r);
  float pc = __fmaf_rn(r2, (float)(-1.0 / 3628800), (float)(1.0 / 40320));
  pc = __fmaf_rn(r2, pc, (float)(-1.0 / 720));
  pc = __fmaf_rn(r2, pc, (float)(1.0 / 24));
  pc = __fmaf_rn(r2, pc, -0.5f);
  pc = __fmaf_rn(r2, pc, 1.0f);
  const float a = (quad & 1) ? pc : ps;
  const float b = (quad & 1) ? ps : pc;
  *sn = (quad & 2) ? -a : a;
  *cs = ((quad + 1) & 2) ? -b : b;
}

// ------------------------------------------------------------------ Philox4x32-10
// Salmon et al. (SC'11).  Stream element q: block q/4 (128-bit counter), word q%4,
// key = the seed widened like an int passed to curand_init (kuramoto.cu:57-60).
__device__ __forceinline__ uint4 philox10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
  }
  return c;
}
__device__ __forceinline__ uint32_t stream_word(int seed, unsigned long long q) {
  unsigned long long s = (unsigned long long)(long long)seed;
  uint4 o = philox10(make_uint4((uint32_t)(q >> 2), (uint32_t)(q >> 34), 0u, 0u), (uint32_t)s, (uint32_t)(s >> 32));
  uint32_t sel = (uint32_t)(q & 3);
  return sel == 0 ? o.x : sel == 1 ? o.y : sel == 2 ? o.z : o.w;
}


}  // namespace kura
