// kora_core.hpp -- CPU restatement of the reference Kuramoto DP45 integrator.
//
// TEST INFRASTRUCTURE ONLY.  This is the oracle: it is linked, called or executed
// only by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
// arm, and only as the checker or the timed CPU baseline.  No product code path
// uses it.
//
// Every piece restates the reference algorithm (znicolaou/kuramoto) in plain C++,
// templated on the real type R (float mirrors `kuramoto`, double mirrors
// `kuramoto_64`):
//   * Philox4x32-10 counter RNG: published algorithm of Salmon et al., "Parallel
//     random numbers: as easy as 1, 2, 3" (SC'11); the stream mapping (key = seed,
//     element q = word q%4 of block q/4) is the one the reference's cuRAND calls
//     use (kuramoto.cu:57-60, 69, 90-94, 131-133).
//   * volcano factor bits u_mn = +/-1 from the low bit of element m*N+n
//     (kuramoto.cu:74, 93, 133) and the dense rule
//     A = (1/N) sum_m (-1)^m u_m u_m^T (kuramoto.cu:137-157).
//   * glibc rand() initial phases and frequencies (kuramoto.cu:416, 495-541).
//   * the right-hand side (kuramoto.cu:42-55, 62-126).
//   * the Dormand-Prince 4/5 stepper, controller and dense output
//     (dp45.cu:6-21, 34-164).
//   * the observer step_eval and the end-of-run record (kuramoto.cu:164-265,
//     587-647).
// Parallel loops use a fixed partition of the index space (independent of the
// thread count), so results do not depend on OMP_NUM_THREADS.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace kora {

// ---------------------------------------------------------------- Philox4x32-10
struct u32x4 { uint32_t v[4]; };

// Salmon et al. (SC'11), Philox4x32 with 10 rounds: multipliers 0xD2511F53 and
// 0xCD9E8D57, Weyl key increments 0x9E3779B9 and 0xBB67AE85.
inline u32x4 philox4x32_10(u32x4 ctr, uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint64_t p0 = (uint64_t)0xD2511F53u * ctr.v[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * ctr.v[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    u32x4 n;
    n.v[0] = hi1 ^ ctr.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ ctr.v[3] ^ k1;
    n.v[3] = lo0;
    ctr = n;
  }
  return ctr;
}

// Element q of the stream that curand_init(seed, 0, 0) starts: block q/4 (a
// 128-bit counter), word q%4.  The seed is widened like an `int` passed as
// `unsigned long long` (kuramoto.cu:57-59).
inline uint32_t philox_stream_word(int32_t seed, uint64_t q) {
  uint64_t s = (uint64_t)(int64_t)seed;
  u32x4 c; c.v[0] = (uint32_t)(q >> 2); c.v[1] = (uint32_t)(q >> 34); c.v[2] = 0; c.v[3] = 0;
  u32x4 o = philox4x32_10(c, (uint32_t)s, (uint32_t)(s >> 32));
  return o.v[q & 3];
}

// u_{m,n} in {-1,+1} for m < K, n < N, stored as int8 at m*N+n (kuramoto.cu:74).
inline void volcano_factor(int32_t seed, int64_t N, int32_t K, int8_t* u) {
  int64_t total = (int64_t)K * N;
  // blocks of 4 consecutive stream elements share one Philox call
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < (total + 3) / 4; ++b) {
    uint64_t s = (uint64_t)(int64_t)seed;
    u32x4 c; c.v[0] = (uint32_t)b; c.v[1] = (uint32_t)((uint64_t)b >> 32); c.v[2] = 0; c.v[3] = 0;
    u32x4 o = philox4x32_10(c, (uint32_t)s, (uint32_t)(s >> 32));
    for (int w = 0; w < 4; ++w) {
      int64_t q = 4 * b + w;
      if (q < total) u[q] = (o.v[w] & 1u) ? 1 : -1;
    }
  }
}

// Dense volcano adjacency, row-major (row i at A + i*N).  N*A_ij is the integer
// k_ij = sum_m (-1)^m u_mi u_mj; the entry is k_ij * fl(1/N) rounded once to R
// (kuramoto.cu:137-157 computes the same sum with u2 = (-1)^m u1 / N in a GEMM).
template <typename R>
void volcano_adjacency(int32_t seed, int64_t N, int32_t K, R* A) {
  std::vector<int8_t> u((size_t)K * N);
  volcano_factor(seed, N, K, u.data());
  const R invN = (R)1 / (R)N;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    for (int64_t j = 0; j < N; ++j) {
      int k = 0;
      for (int m = 0; m < K; ++m) {
        int t = u[(size_t)m * N + i] * u[(size_t)m * N + j];
        k += (m & 1) ? -t : t;
      }
      A[(size_t)i * N + j] = (R)k * invN;
    }
  }
}

// ------------------------------------------------------------- host generator
// srand(seed) is called once; theta0 consumes N draws first when it is generated
// (kuramoto.cu:416, 498-500), then the frequencies (kuramoto.cu:526-537).  The
// expressions keep the C++ overload semantics of the reference (float log, double
// pow/cos/tan), which makes the output byte-identical.
inline void host_random_inputs(int32_t seed, int64_t N, float I, float freq, int normal,
                               int gen_theta, int gen_omega, float* theta0, float* omega) {
  srand(seed);
  if (gen_theta)
    for (int64_t j = 0; j < N; ++j) theta0[j] = I / 2 * (2.0 / RAND_MAX * rand() - 1);
  if (gen_omega) {
    for (int64_t j = 0; j < N; ++j) {
      if (normal) {
        float u = rand() / (float)RAND_MAX;
        float v = rand() / (float)RAND_MAX;
        // float log, then double pow and cos, as the C++ overloads resolve there
        omega[j] = freq * std::pow(-2 * std::log(u), 0.5) * std::cos(2 * M_PI * v);
      } else {
        float u = rand() / (float)RAND_MAX;
        omega[j] = freq * std::tan(M_PI * (u - 0.5));
      }
    }
  }
}

// ---------------------------------------------------------------- tableau
// Dormand-Prince 5(4) coefficients and the 4th-order continuous extension,
// as the reference stores them (dp45.cu:6-21): each rational is evaluated in
// double and rounded to R.
template <typename R> struct Tableau {
  R a[7][6];  // a[s][j], s = 1..5 stage rows; a[6] = 5th-order weights b
  R c[7];
  R e[7];
  R p[7][4];
  Tableau() {
    std::memset(this, 0, sizeof(*this));
    a[1][0] = 1.0 / 5;
    a[2][0] = 3.0 / 40; a[2][1] = 9.0 / 40;
    a[3][0] = 44.0 / 45; a[3][1] = -56.0 / 15; a[3][2] = 32.0 / 9;
    a[4][0] = 19372.0 / 6561; a[4][1] = -25360.0 / 2187; a[4][2] = 64448.0 / 6561; a[4][3] = -212.0 / 729;
    a[5][0] = 9017.0 / 3168; a[5][1] = -355.0 / 33; a[5][2] = 46732.0 / 5247; a[5][3] = 49.0 / 176;
    a[5][4] = -5103.0 / 18656;
    a[6][0] = 35.0 / 384; a[6][1] = 0; a[6][2] = 500.0 / 1113; a[6][3] = 125.0 / 192;
    a[6][4] = -2187.0 / 6784; a[6][5] = 11.0 / 84;
    const double cc[7] = {0.0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1.0, 1.0};
    for (int i = 0; i < 7; ++i) c[i] = (R)cc[i];
    const double ee[7] = {-71.0 / 57600, 0, 71.0 / 16695, -71.0 / 1920, 17253.0 / 339200, -22.0 / 525, 1.0 / 40};
    for (int i = 0; i < 7; ++i) e[i] = (R)ee[i];
    const double pp[7][4] = {
        {1.0, -8048581381.0 / 2820520608, 8663915743.0 / 2820520608, -12715105075.0 / 11282082432},
        {0, 0, 0, 0},
        {0, 131558114200.0 / 32700410799, -68118460800.0 / 10900136933, 87487479700.0 / 32700410799},
        {0, -1754552775.0 / 470086768, 14199869525.0 / 1410260304, -10690763975.0 / 1880347072},
        {0, 127303824393.0 / 49829197408, -318862633887.0 / 49829197408, 701980252875.0 / 199316789632},
        {0, -282668133.0 / 205662961, 2019193451.0 / 616988883, -1453857185.0 / 822651844},
        {0, 40617522.0 / 29380423, -110615467.0 / 29380423, 69997945.0 / 29380423}};
    for (int j = 0; j < 7; ++j)
      for (int q = 0; q < 4; ++q) p[j][q] = (R)pp[j][q];
  }
};

// ---------------------------------------------------------------- reductions
// Fixed-partition sum (chunks of 4096, partials added in chunk order): the
// result does not depend on the number of threads.
template <typename R, typename F>
double chunked_sum(int64_t n, F f) {
  const int64_t C = 4096;
  int64_t nc = (n + C - 1) / C;
  std::vector<double> part((size_t)std::max<int64_t>(nc, 1), 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nc; ++c) {
    double s = 0;
    int64_t e = std::min(n, (c + 1) * C);
    for (int64_t i = c * C; i < e; ++i) s += (double)f(i);
    part[(size_t)c] = s;
  }
  double s = 0;
  for (int64_t c = 0; c < nc; ++c) s += part[(size_t)c];
  return s;
}

// ---------------------------------------------------------------- model
template <typename R> struct Model {
  using value_type = R;
  int64_t N = 0;
  int32_t K = 0;
  int onthefly = 0;            // -A
  const R* A = nullptr;        // dense, row-major
  std::vector<int8_t> U;       // -A factor, K*N
  std::vector<R> omega;
  R c1 = 0;
  std::vector<R> y2, f2, f3;

  void init() {
    y2.assign((size_t)2 * N, 0);
    f2.assign((size_t)2 * N, 0);
    f3.assign((size_t)2 * std::max(K, 1), 0);
  }
  // makey2 (kuramoto.cu:49-55)
  void makey2(const R* y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
      y2[2 * i] = std::cos(y[i]);
      y2[2 * i + 1] = std::sin(y[i]);
    }
  }
  // makecoupling (kuramoto.cu:104-116): f[2i] = (A cos)_i, f[2i+1] = (A sin)_i
  void makecoupling(R* f) {
    if (onthefly) {
      // m1 (kuramoto.cu:62-81): f3[2m] = (sum_n (-1)^m u_mn y2[2n]) / N
      for (int m = 0; m < K; ++m) {
        const int8_t* um = U.data() + (size_t)m * N;
        R s = (m & 1) ? (R)-1 : (R)1;
        // sequential sum over n within fixed chunks; chunks added in order
        const int64_t C = 4096;
        int64_t nc = (N + C - 1) / C;
        std::vector<R> pc((size_t)nc), ps((size_t)nc);
#pragma omp parallel for schedule(static)
        for (int64_t c = 0; c < nc; ++c) {
          R a = 0, b = 0;
          int64_t e = std::min(N, (c + 1) * C);
          for (int64_t n = c * C; n < e; ++n) {
            a += y2[2 * n] * s * um[n];
            b += y2[2 * n + 1] * s * um[n];
          }
          pc[(size_t)c] = a; ps[(size_t)c] = b;
        }
        R a = 0, b = 0;
        for (int64_t c = 0; c < nc; ++c) { a += pc[(size_t)c]; b += ps[(size_t)c]; }
        f3[2 * m] = a / (R)N;
        f3[2 * m + 1] = b / (R)N;
      }
      // m2 (kuramoto.cu:83-101): f[2n] = sum_m u_mn f3[2m]
#pragma omp parallel for schedule(static)
      for (int64_t n = 0; n < N; ++n) {
        R a = 0, b = 0;
        for (int m = 0; m < K; ++m) {
          R u = (R)U[(size_t)m * N + n];
          a += f3[2 * m] * u;
          b += f3[2 * m + 1] * u;
        }
        f[2 * n] = a;
        f[2 * n + 1] = b;
      }
    } else {
      // two GEMVs over the same matrix (kuramoto.cu:113-114)
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < N; ++i) {
        const R* row = A + (size_t)i * N;
        R a = 0, b = 0;
        for (int64_t j = 0; j < N; ++j) {
          a += row[j] * y2[2 * j];
          b += row[j] * y2[2 * j + 1];
        }
        f[2 * i] = a;
        f[2 * i + 1] = b;
      }
    }
  }
  // dydt (kuramoto.cu:118-126) with tot_kuramoto (kuramoto.cu:42-47)
  void dydt(const R* y, R* f) {
    makey2(y);
    makecoupling(f2.data());
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i)
      f[i] = omega[i] + c1 * (y2[2 * i + 1] * f2[2 * i] - y2[2 * i] * f2[2 * i + 1]);
  }
  // order parameter at the current y2 (kuramoto.cu:212-220)
  R order_from_y2() {
    R X = (R)chunked_sum<R>(N, [&](int64_t i) { return y2[2 * i]; });
    R Y = (R)chunked_sum<R>(N, [&](int64_t i) { return y2[2 * i + 1]; });
    return (R)std::pow((X / N * X / N + Y / N * Y / N), 0.5);
  }
};

// ---------------------------------------------------------------- outputs
struct Outputs {
  std::vector<double> order;      // r at t0 (fresh start) and at each t_eval
  std::vector<double> thetas;     // dense >= 1: rows of N
  std::vector<double> couplings;  // dense >= 2: rows of 2N
  std::vector<double> times;      // dense >= 1: t after each accepted step
  std::vector<double> steph;      // h after each accepted step
  std::vector<double> final_theta, final_coupling;
  double final_t = 0, final_h = 0;
  int64_t steps = 0, attempts = 0;
  int status = 0;                 // 0 ok, 1 attempt cap reached
};

// ---------------------------------------------------------------- DP45 driver
template <typename R> struct Integrator {
  Model<R>& M;
  Tableau<R> T;
  int64_t N;
  std::vector<R> y, ylast, ytemp, yerr, yeval;
  std::vector<R> k[7];
  R atl, rtl, t_last = 0;
  int fixed;

  Integrator(Model<R>& m, R atol, R rtol, int fixedstep) : M(m), N(m.N), atl(atol), rtl(rtol), fixed(fixedstep) {
    y.assign(N, 0); ylast.assign(N, 0); ytemp.assign(N, 0); yerr.assign(N, 0); yeval.assign(N, 0);
    for (int j = 0; j < 7; ++j) k[j].assign(N, 0);
  }

  // stage combination ytemp = y + h * sum_j a[s][j] k_j (dp45.cu:34-69)
  void stage(int s, R h) {
    const R* a = T.a[s];
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
      R acc = a[0] * k[0][i];
      for (int j = 1; j < s; ++j) acc = acc + a[j] * k[j][i];
      ytemp[i] = y[i] + h * acc;
    }
  }

  // dp45_step (dp45.cu:87-141); returns 1 on accept
  int step(R* t, R* h) {
    for (int s = 1; s <= 6; ++s) {
      stage(s, *h);
      M.dydt(ytemp.data(), k[s].data());
    }
    if (fixed) {
      t_last = *t;
      ylast = y; y = ytemp;
      *t = *t + *h;
      return 1;
    }
    const R* e = T.e;
    R hh = *h;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
      R s = e[0] * k[0][i] + e[1] * k[1][i] + e[2] * k[2][i] + e[3] * k[3][i] + e[4] * k[4][i] + e[5] * k[5][i] +
            e[6] * k[6][i];
      yerr[i] = hh * s / (atl + rtl * std::max(std::fabs(y[i]), std::fabs(ytemp[i])));
    }
    double ss = chunked_sum<R>(N, [&](int64_t i) { return (double)yerr[i] * (double)yerr[i]; });
    R norm = (R)std::sqrt(ss);
    norm /= std::pow((double)N, 0.5);
    R factor = 0.9 * std::pow(norm, -0.2);
    if (norm < 1) {
      t_last = *t;
      ylast = y; y = ytemp;
      *t = *t + *h;
      if (factor > 10) factor = 10;
      *h *= factor;
      return 1;
    } else if (factor < 1) {
      if (factor < 0.2) factor = 0.2;
      *h *= factor;
    }
    return 0;
  }

  // interpolate (dp45.cu:70-76) at t_eval within the last accepted step;
  // k1_is_k7 reproduces the end-of-run call made after the FSAL copy
  // (dp45.cu:160 then kuramoto.cu:632).
  void eval(R t, R t_eval, bool k1_is_k7) {
    R hs = t - t_last, h2 = t_eval - t_last;
    const std::vector<R>& K1 = k1_is_k7 ? k[6] : k[0];
    const auto& P = T.p;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
      R x = h2 / hs;
      R q[4];
      for (int c = 0; c < 4; ++c)
        q[c] = P[0][c] * K1[i] + P[1][c] * k[1][i] + P[2][c] * k[2][i] + P[3][c] * k[3][i] + P[4][c] * k[4][i] +
               P[5][c] * k[5][i] + P[6][c] * k[6][i];
      yeval[i] = ylast[i] + hs * (x * q[0] + x * x * q[1] + x * x * x * q[2] + x * x * x * x * q[3]);
    }
  }
};

struct RunSpec {
  double t0 = 0, t1 = 100, dt = 1, h0 = 0.01, atol = 1e-6, rtol = 0;
  int fixed = 0;
  int dense = 0;           // -D level
  int initial_record = 1;  // fresh start writes r(theta0) (kuramoto.cu:587-626)
  int64_t max_attempts = -1;
};

// output grid t_eval = dt*n for n = int(t0/dt)+1 .. int(t1/dt) (kuramoto.cu:543-550)
template <typename R> std::vector<R> eval_grid(R t0, R t1, R dt) {
  int n0 = int(t0 / dt) + 1;
  int n1 = int(t1 / dt) + 1;
  std::vector<R> g;
  for (int n = n0; n < n1; ++n) g.push_back(dt * n);
  return g;
}

// The whole run: initial record, dp45_run loop with step_eval, end record.
template <typename R>
void run(Model<R>& M, const R* theta0, const RunSpec& S, Outputs& O) {
  M.init();
  Integrator<R> I(M, (R)S.atol, (R)S.rtol, S.fixed);
  int64_t N = M.N;
  for (int64_t i = 0; i < N; ++i) I.y[i] = theta0[i];
  R t = (R)S.t0, h = (R)S.h0, t1 = (R)S.t1;
  std::vector<R> t_eval = eval_grid<R>(t, t1, (R)S.dt);
  int n_eval = (int)t_eval.size();
  std::vector<R> floc((size_t)2 * N, 0);

  if (S.initial_record) {
    M.makey2(I.y.data());
    O.order.push_back(M.order_from_y2());
    if (S.dense >= 1) O.thetas.insert(O.thetas.end(), I.y.begin(), I.y.end());
    if (S.dense >= 2) {
      M.makecoupling(floc.data());
      O.couplings.insert(O.couplings.end(), floc.begin(), floc.end());
    }
  }
  // dp45_run (dp45.cu:148-164)
  M.dydt(I.y.data(), I.k[0].data());
  int eval_i = 0;
  while (t < t1) {
    if (S.max_attempts >= 0 && O.attempts >= S.max_attempts) { O.status = 1; break; }
    O.attempts++;
    int ok = I.step(&t, &h);
    if (ok) {
      // step_eval (kuramoto.cu:164-265)
      O.steps++;
      if (S.dense >= 1) O.times.push_back((double)t);
      O.steph.push_back((double)h);
      while (eval_i < n_eval && t >= t_eval[eval_i]) {
        I.eval(t, t_eval[eval_i], false);
        M.makey2(I.yeval.data());
        O.order.push_back(M.order_from_y2());
        if (S.dense >= 1) O.thetas.insert(O.thetas.end(), I.yeval.begin(), I.yeval.end());
        if (S.dense >= 2) {
          M.makecoupling(floc.data());
          O.couplings.insert(O.couplings.end(), floc.begin(), floc.end());
        }
        eval_i++;
      }
      I.k[0] = I.k[6];
    }
  }
  // end record (kuramoto.cu:630-647)
  if (n_eval > 0) {
    I.eval(t, t_eval[n_eval - 1], true);
  } else {
    I.yeval = I.y;
  }
  M.makey2(I.yeval.data());
  M.makecoupling(floc.data());
  O.final_theta.assign(I.yeval.begin(), I.yeval.end());
  O.final_coupling.assign(floc.begin(), floc.end());
  O.final_t = (double)t;
  O.final_h = (double)h;
}

}  // namespace kora
