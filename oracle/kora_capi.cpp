// kora_capi.cpp -- C ABI of the CPU oracle (TEST INFRASTRUCTURE ONLY).
//
// Loaded with ctypes by tests/, __graft_entry__.smoke() and bench.py's CPU legs.
// Nothing in the product links or loads it.  See kora_core.hpp for the
// reference file:line each piece restates.
#include <type_traits>
#include "kora_core.hpp"

typedef struct kora_spec {
  int64_t n;
  int32_t k;
  int32_t onthefly;   // -A
  int32_t seed;
  int32_t fp64;       // 0: float (kuramoto), 1: double (kuramoto_64)
  double c1, t0, t1, dt, h0, atol, rtol;
  int32_t fixed, dense, initial_record, threads;
  int64_t max_attempts;
} kora_spec;

template <typename R>
static void setup_model(kora::Model<R>& M, std::vector<R>& Abuf, const kora_spec* s, const double* omega,
                        const double* adj, double c1) {
  M.N = s->n;
  M.K = s->k;
  M.onthefly = s->onthefly;
  M.c1 = (R)c1;
  M.omega.resize((size_t)s->n);
  for (int64_t i = 0; i < s->n; ++i) M.omega[(size_t)i] = (R)omega[i];
  if (s->onthefly) {
    M.U.resize((size_t)s->k * s->n);
    kora::volcano_factor(s->seed, s->n, s->k, M.U.data());
  } else {
    Abuf.resize((size_t)s->n * s->n);
    if (adj) {
      for (size_t i = 0; i < Abuf.size(); ++i) Abuf[i] = (R)adj[i];
    } else {
      kora::volcano_adjacency<R>(s->seed, s->n, s->k, Abuf.data());
    }
    M.A = Abuf.data();
  }
}

extern "C" {

void kora_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  kora::u32x4 c;
  for (int i = 0; i < 4; ++i) c.v[i] = ctr[i];
  kora::u32x4 o = kora::philox4x32_10(c, key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = o.v[i];
}

uint32_t kora_philox_stream_word(int32_t seed, uint64_t q) { return kora::philox_stream_word(seed, q); }

void kora_volcano_factor(int32_t seed, int64_t n, int32_t k, int8_t* u) { kora::volcano_factor(seed, n, k, u); }

void kora_volcano_adjacency_f32(int32_t seed, int64_t n, int32_t k, float* a) {
  kora::volcano_adjacency<float>(seed, n, k, a);
}
void kora_volcano_adjacency_f64(int32_t seed, int64_t n, int32_t k, double* a) {
  kora::volcano_adjacency<double>(seed, n, k, a);
}

void kora_host_random_inputs(int32_t seed, int64_t n, float init, float freq, int32_t normal, int32_t gen_theta,
                             int32_t gen_omega, float* theta0, float* omega) {
  kora::host_random_inputs(seed, n, init, freq, normal, gen_theta, gen_omega, theta0, omega);
}

void kora_set_threads(int32_t n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int32_t kora_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// RHS f = dtheta/dt at y (kuramoto.cu:118-126); couplings (2N) optional.
void kora_rhs(const kora_spec* s, const double* omega, const double* adj, const double* y, double* f,
              double* couplings) {
  auto go = [&](auto tag) {
    using R = decltype(tag);
    kora::Model<R> M;
    std::vector<R> Abuf;
    setup_model<R>(M, Abuf, s, omega, adj, s->c1);
    M.init();
    std::vector<R> yy((size_t)s->n), ff((size_t)s->n);
    for (int64_t i = 0; i < s->n; ++i) yy[(size_t)i] = (R)y[i];
    M.dydt(yy.data(), ff.data());
    for (int64_t i = 0; i < s->n; ++i) f[i] = (double)ff[(size_t)i];
    if (couplings)
      for (int64_t i = 0; i < 2 * s->n; ++i) couplings[i] = (double)M.f2[(size_t)i];
  };
  if (s->fp64) go(double()); else go(float());
}

// One whole run; returns an opaque result (free with kora_result_free).
void* kora_run(const kora_spec* s, const double* theta0, const double* omega, const double* adj) {
  kora::RunSpec S;
  S.t0 = s->t0; S.t1 = s->t1; S.dt = s->dt; S.h0 = s->h0; S.atol = s->atol; S.rtol = s->rtol;
  S.fixed = s->fixed; S.dense = s->dense; S.initial_record = s->initial_record; S.max_attempts = s->max_attempts;
  if (s->threads > 0) kora_set_threads(s->threads);
  auto* O = new kora::Outputs();
  auto go = [&](auto tag) {
    using R = decltype(tag);
    kora::Model<R> M;
    std::vector<R> Abuf;
    setup_model<R>(M, Abuf, s, omega, adj, s->c1);
    std::vector<R> th((size_t)s->n);
    for (int64_t i = 0; i < s->n; ++i) th[(size_t)i] = (R)theta0[i];
    kora::run<R>(M, th.data(), S, *O);
  };
  if (s->fp64) go(double()); else go(float());
  return O;
}

// A model kept between runs (the dense adjacency of a large network is built once): runs of
// several trajectories, or several samples of one, on the same network and frequencies.
struct kora_model {
  int fp64 = 0;
  kora::Model<float> Mf;
  kora::Model<double> Md;
  std::vector<float> Af;
  std::vector<double> Ad;
};

void* kora_model_create(const kora_spec* s, const double* omega, const double* adj) {
  if (s->threads > 0) kora_set_threads(s->threads);
  auto* m = new kora_model();
  m->fp64 = s->fp64;
  if (s->fp64) setup_model<double>(m->Md, m->Ad, s, omega, adj, s->c1);
  else setup_model<float>(m->Mf, m->Af, s, omega, adj, s->c1);
  return m;
}

// One run of the kept model from theta0 with the spec's coupling constant and horizon.
void* kora_model_run(void* model, const kora_spec* s, const double* theta0) {
  auto* m = (kora_model*)model;
  kora::RunSpec S;
  S.t0 = s->t0; S.t1 = s->t1; S.dt = s->dt; S.h0 = s->h0; S.atol = s->atol; S.rtol = s->rtol;
  S.fixed = s->fixed; S.dense = s->dense; S.initial_record = s->initial_record; S.max_attempts = s->max_attempts;
  if (s->threads > 0) kora_set_threads(s->threads);
  auto* O = new kora::Outputs();
  auto go = [&](auto& M) {
    using R = typename std::remove_reference<decltype(M)>::type::value_type;
    M.c1 = (R)s->c1;
    std::vector<R> th((size_t)s->n);
    for (int64_t i = 0; i < s->n; ++i) th[(size_t)i] = (R)theta0[i];
    kora::run<R>(M, th.data(), S, *O);
  };
  if (m->fp64) go(m->Md); else go(m->Mf);
  return O;
}

void kora_model_free(void* model) { delete (kora_model*)model; }

static const std::vector<double>* pick(kora::Outputs* O, int which) {
  switch (which) {
    case 0: return &O->order;
    case 1: return &O->thetas;
    case 2: return &O->couplings;
    case 3: return &O->times;
    case 4: return &O->steph;
    case 5: return &O->final_theta;
    case 6: return &O->final_coupling;
  }
  return nullptr;
}

int64_t kora_result_size(void* r, int32_t which) {
  auto* v = pick((kora::Outputs*)r, which);
  return v ? (int64_t)v->size() : -1;
}
void kora_result_copy(void* r, int32_t which, double* out) {
  auto* v = pick((kora::Outputs*)r, which);
  if (v) std::memcpy(out, v->data(), v->size() * sizeof(double));
}
void kora_result_scalars(void* r, double* final_t, double* final_h, int64_t* steps, int64_t* attempts,
                         int32_t* status) {
  auto* O = (kora::Outputs*)r;
  *final_t = O->final_t; *final_h = O->final_h; *steps = O->steps; *attempts = O->attempts; *status = O->status;
}
void kora_result_free(void* r) { delete (kora::Outputs*)r; }

}  // extern "C"
