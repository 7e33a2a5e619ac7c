// kora_cli.cpp -- command-line restatement of the reference program's main()
// (kuramoto.cu:267-678) on the CPU oracle.  TEST INFRASTRUCTURE ONLY: the CLI
// parity tests run it beside the product `kuramoto` on the same FILEBASE inputs.
//
// Built twice: without KORA_FP64 it mirrors `kuramoto` (float files), with
// -DKORA_FP64 it mirrors `kuramoto_64` (double files, kuramoto_64.cu).
// All FILEBASE files are written once the run has finished; their final bytes are
// what the reference leaves behind (its per-step rewrites of fs.dat are
// overwritten by the end record, kuramoto.cu:638-647).
#include <cstdio>
#include <sys/time.h>
#include <unistd.h>
#include <string>
#include "kora_core.hpp"

#ifdef KORA_FP64
typedef double R;
#else
typedef float R;
#endif

static std::string fb;
static std::string path(const char* suffix) { return fb + suffix; }

template <typename T> static void write_vec(const char* suffix, const char* mode, const std::vector<double>& v) {
  FILE* f = fopen(path(suffix).c_str(), mode);
  if (!f) return;
  std::vector<T> tmp(v.begin(), v.end());
  if (!tmp.empty()) fwrite(tmp.data(), sizeof(T), tmp.size(), f);
  fclose(f);
}

int main(int argc, char* argv[]) {
  struct timeval start, end;
  gettimeofday(&start, NULL);
  float c1f, t1f, dtf, freq, atl, rtl, I;
  int gpu, seed, fixed, A;
  unsigned long N, K;
  char* filebase = nullptr;
  N = 5000; K = 6; A = 0; I = 0; c1f = 3.0f; freq = 1.0f; t1f = 1e2f; dtf = 1e0f; gpu = 0; seed = 1;
  int verbose = 0; rtl = 0; atl = 1e-6f; fixed = 0;
  int help = 1, dense = 3, normal = 0, reload = 0;
  int c;
  while (optind < argc) {
    if ((c = getopt(argc, argv, "N:K:I:D:c:g:t:d:f:s:r:a:hvFnRA")) != -1) {
      switch (c) {
        case 'N': N = (int)atoi(optarg); break;
        case 'K': K = (int)atoi(optarg); break;
        case 'A': A = 1; break;
        case 'I': I = (float)atof(optarg); break;
        case 'c': c1f = (float)atof(optarg); break;
        case 'g': gpu = (int)atof(optarg); break;
        case 't': t1f = (float)atof(optarg); break;
        case 'd': dtf = (float)atof(optarg); break;
        case 'f': freq = (float)atof(optarg); break;
        case 's': seed = (int)atoi(optarg); break;
        case 'r': rtl = (float)atof(optarg); break;
        case 'a': atl = (float)atof(optarg); break;
        case 'D': dense = (int)atoi(optarg); break;
        case 'R': reload = 1; break;
        case 'F': fixed = 1; break;
        case 'h': help = 1; break;
        case 'v': verbose = 1; break;
        case 'n': normal = 1; break;
      }
    } else {
      filebase = argv[optind];
      optind++;
      help = 0;
    }
  }
  (void)gpu;
  if (help) {
    printf("usage:\tkuramoto_oracle [-hvnRFA] [-N N] [-K K] [-D D]\n");
    printf("\t[-c c] [-t t] [-d dt] [-f f] [-s seed] \n");
    printf("\t[-I init] [-r rtol] [-a atol] [-g gpu] filebase \n\n");
    return 0;
  }
  fb = filebase;
  // the reference keeps these in R (double in kuramoto_64.cu)
  R c1 = c1f, t1 = t1f, dt = dtf;
  R t = 0, h;
  FILE* out = fopen(path(".out").c_str(), "ab");
  std::vector<float> yl32(N), om32(N);
  std::vector<R> yloc(N), omegasloc(N);
  srand(seed);
  fprintf(out, "%lu %lu %f %f %f %i\n", N, K, (double)t1, (double)dt, (double)c1, seed);
  for (int i = 0; i < argc; i++) fprintf(out, "%s ", argv[i]);
  fprintf(out, "\n");
  size_t req = A ? 100 * N * sizeof(R) : (100 + N + 2 * K) * N * sizeof(R);
  printf("GPU Memory: %lu %lu %lu\n", (unsigned long)req, (unsigned long)req, (unsigned long)req);
  fprintf(out, "GPU Memory: %lu %lu %lu\n", (unsigned long)req, (unsigned long)req, (unsigned long)req);
  fflush(out);
  h = fixed ? dt : dt / 100;

  int reloaded = 0;
  FILE* in;
  if (reload && (in = fopen(path("fs.dat").c_str(), "r"))) {
    reloaded = 1;
    printf("Using initial conditions from file\n");
    fprintf(out, "Using initial conditions from file\n");
    size_t rd = fread(yloc.data(), sizeof(R), N, in);
    if (rd != N) {
      printf("initial conditions file not compatible with N!\n");
      fprintf(out, "initial conditions file not compatible with N!\n");
      reloaded = 0;
    }
    if (reloaded) {
      rd = fread(&t, sizeof(R), 1, in);
      rd = fread(&h, sizeof(R), 1, in);
      if (rd != 1) {
        printf("Couldn't read start time and step!\n");
        fprintf(out, "Couldn't read start time and step!\n");
        reloaded = 0;
      }
    }
    fclose(in);
    printf("Restarting at t=%f with h=%f\n", (double)t, (double)h);
    fprintf(out, "Restarting at t=%f with h=%f\n", (double)t, (double)h);
  }
  if (!reloaded) {
    printf("Using random initial conditions\n");
    fprintf(out, "Using random initial conditions\n");
    for (unsigned long j = 0; j < N; j++) yloc[j] = I / 2 * (2.0 / RAND_MAX * rand() - 1);
    in = fopen(path("fs.dat").c_str(), "wb");
    fwrite(yloc.data(), sizeof(R), N, in);
    fclose(in);
  }
  int freq_loaded = 0;
  if (reload && (in = fopen(path("frequencies.dat").c_str(), "r"))) {
    printf("Using frequencies from file\n");
    fprintf(out, "Using frequencies from file\n");
    size_t rd = fread(omegasloc.data(), sizeof(R), N, in);
    fclose(in);
    if (rd != N) {
      printf("frequencies not compatible with N!");
      fprintf(out, "frequencies not compatible with N!");
      return 0;
    }
    freq_loaded = 1;
  }
  if (!freq_loaded) {
    printf("Using random frequencies\n");
    fprintf(out, "Using random frequencies\n");
    for (unsigned long j = 0; j < N; j++) {
      if (normal) {
        R u = rand() / (R)RAND_MAX;
        R v = rand() / (R)RAND_MAX;
        omegasloc[j] = freq * std::pow(-2 * std::log(u), 0.5) * std::cos(2 * M_PI * v);
      } else {
        R u = rand() / (R)RAND_MAX;
        omegasloc[j] = freq * std::tan(M_PI * (u - 0.5));
      }
    }
    in = fopen(path("frequencies.dat").c_str(), "wb");
    fwrite(omegasloc.data(), sizeof(R), N, in);
    fclose(in);
  }

  kora::Model<R> M;
  M.N = (int64_t)N; M.K = (int32_t)K; M.onthefly = A; M.c1 = c1;
  M.omega.assign(omegasloc.begin(), omegasloc.end());
  std::vector<R> adj;
  if (!A) adj.assign((size_t)N * N, 0);
  if (!A && reload && (in = fopen(path("adj.dat").c_str(), "r"))) {
    printf("Using adjacency from file\n");
    fprintf(out, "Using adjacency from file\n");
    size_t rd = fread(adj.data(), sizeof(R), (size_t)N * N, in);
    (void)rd;
    fclose(in);
  } else {
    printf("Using random adjacency matrix\n");
    fprintf(out, "Using random adjacency matrix\n");
    if (!A) {
      kora::volcano_adjacency<R>(seed, (int64_t)N, (int32_t)K, adj.data());
      if (dense >= 3) {
        in = fopen(path("adj.dat").c_str(), "wb");
        fwrite(adj.data(), sizeof(R), (size_t)N * N, in);
        fclose(in);
      }
    }
  }
  if (A) {
    M.U.resize((size_t)K * N);
    kora::volcano_factor(seed, (int64_t)N, (int32_t)K, M.U.data());
  } else {
    M.A = adj.data();
  }
  fflush(out);
  fclose(out);

  kora::RunSpec S;
  S.t0 = (double)t; S.t1 = (double)t1; S.dt = (double)dt; S.h0 = (double)h; S.atol = atl; S.rtol = rtl;
  S.fixed = fixed; S.dense = dense; S.initial_record = !reloaded;
  kora::Outputs O;
  kora::run<R>(M, yloc.data(), S, O);

  // files (kuramoto.cu:587-626 on a fresh start, step_eval appends, end record)
  const char* mode = reloaded ? "ab" : "wb";
  write_vec<R>("order.dat", mode, O.order);
  if (dense >= 1) {
    write_vec<R>("thetas.dat", mode, O.thetas);
    write_vec<R>("times.dat", mode, O.times);
  }
  if (dense >= 2) write_vec<R>("couplings.dat", mode, O.couplings);
  FILE* fs = fopen(path("fs.dat").c_str(), "wb");
  std::vector<R> th(O.final_theta.begin(), O.final_theta.end());
  std::vector<R> cp(O.final_coupling.begin(), O.final_coupling.end());
  R ft = (R)O.final_t, fh = (R)O.final_h;
  fwrite(th.data(), sizeof(R), N, fs);
  fwrite(&ft, sizeof(R), 1, fs);
  fwrite(&fh, sizeof(R), 1, fs);
  fwrite(cp.data(), sizeof(R), 2 * N, fs);
  fclose(fs);

  out = fopen(path(".out").c_str(), "ab");
  gettimeofday(&end, NULL);
  double rt = end.tv_sec - start.tv_sec + 1e-6 * (end.tv_usec - start.tv_usec);
  if (verbose) {
    for (size_t i = 0; i < O.times.size() || i < O.steph.size(); ++i) {
      double ti = i < O.times.size() ? O.times[i] : 0;
      double hi = O.steph[i];
      fprintf(out, "%.3f\t%1.3e\t%1.3e\t%f\t%i\t\n", (ti - S.t0) / (S.t1 - S.t0), rt, 0.0, hi, (int)(i + 1));
    }
  }
  printf("\nruntime: %f\n", rt);
  fprintf(out, "\nsteps: %i\n", (int)O.steps);
  fprintf(out, "runtime: %f\n", rt);
  fclose(out);
  return 0;
}
