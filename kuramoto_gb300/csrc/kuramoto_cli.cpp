// kuramoto_cli.cpp -- the `kuramoto` command line on libkura.
//
// A drop-in for the reference program's CLI and FILEBASE files (kuramoto.cu:267-678):
// the same getopt string "N:K:I:D:c:g:t:d:f:s:r:a:hvFnRA", defaults (N=5000, K=6,
// c=3, t=100, dt=1, f=1, seed=1, atol=1e-6, rtol=0, D=3), messages and files:
//   FILEBASE.out          header "N K t1 dt c seed", argv, memory line, messages, steps, runtime
//   FILEBASEfs.dat        theta0 on a fresh start; at the end theta(t_eval[last]), t, h, couplings[2N]
//   FILEBASEorder.dat     r at t0 (fresh start) and at every t_eval
//   FILEBASEthetas.dat    (D>=1) theta0 and theta(t_eval)
//   FILEBASEtimes.dat     (D>=1) t after every accepted step
//   FILEBASEcouplings.dat (D>=2) [A cos, A sin] interleaved at t0 and every t_eval
//   FILEBASEadj.dat       (D>=3, generated dense adjacency) N*N floats
//   FILEBASEfrequencies.dat  omega
// -R reloads fs.dat (theta, t, h), frequencies.dat and adj.dat when present and
// appends to the output files, as the reference does.  The reference rewrites
// fs.dat after every accepted step for preemption; here fs.dat is rewritten after
// every persistent launch and at the end.  Two environment variables serve preemption:
//   KURA_CHECKPOINT_STEPS=k  ends a launch every k step attempts, so fs.dat is rewritten
//                            at least that often;
//   KURA_FAIL_AT_STEP=k      host-side fault injection: once k steps are accepted, the
//                            process exits with status 3 right after writing fs.dat, as a
//                            preempted job would; rerunning with -R resumes from it.
#include <cuda_runtime.h>
#include <sys/time.h>
#include <unistd.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "kura.h"

namespace {

struct Run {
  std::string base;
  int dense = 3;
  int verbose = 0;
  unsigned long n = 0;
  double t0 = 0, t1 = 0;
  struct timeval start;
  FILE* order = nullptr;
  FILE* thetas = nullptr;
  FILE* couplings = nullptr;
  FILE* times = nullptr;
  std::vector<float> floc;  // couplings last written (fs.dat checkpoint tail)
  long long steps = 0;       // accepted steps seen by on_step
  long long fail_at = 0;     // KURA_FAIL_AT_STEP
};

std::string path(const Run& R, const char* suffix) { return R.base + suffix; }

double elapsed(const Run& R) {
  struct timeval e;
  gettimeofday(&e, NULL);
  return e.tv_sec - R.start.tv_sec + 1e-6 * (e.tv_usec - R.start.tv_usec);
}

void write_fs(const Run& R, const float* theta, float t, float h, const float* coup) {
  FILE* f = fopen(path(R, "fs.dat").c_str(), "wb");
  if (!f) return;
  fwrite(theta, sizeof(float), R.n, f);
  fwrite(&t, sizeof(float), 1, f);
  fwrite(&h, sizeof(float), 1, f);
  fwrite(coup, sizeof(float), 2 * R.n, f);
  fclose(f);
}

int on_step(void* user, int32_t, double t, double h, int64_t step) {
  Run& R = *(Run*)user;
  R.steps = step;
  if (R.verbose) {
    double el = elapsed(R);
    double frac = (t - R.t0) / (R.t1 - R.t0);
    double eta = el / ((t - R.t0 + h) / (R.t1 - R.t0)) * (1 - frac);
    printf("%.3f\t%1.3e\t%1.3e\t%f\t%i\t\r", frac, el, eta, h, (int)step);
    fflush(stdout);
    FILE* out = fopen(path(R, ".out").c_str(), "ab");
    if (out) {
      fprintf(out, "%.3f\t%1.3e\t%1.3e\t%f\t%i\t\n", frac, el, eta, h, (int)step);
      fclose(out);
    }
  }
  if (R.dense >= 1 && R.times) {
    float tf = (float)t;
    fwrite(&tf, sizeof(float), 1, R.times);
  }
  return 0;
}

int on_output(void* user, int32_t, int64_t, double, float r, const float* theta, const float* coup) {
  Run& R = *(Run*)user;
  fwrite(&r, sizeof(float), 1, R.order);
  if (R.dense >= 1 && theta) fwrite(theta, sizeof(float), R.n, R.thetas);
  if (R.dense >= 2 && coup) {
    fwrite(coup, sizeof(float), 2 * R.n, R.couplings);
    std::memcpy(R.floc.data(), coup, sizeof(float) * 2 * R.n);
  }
  return 0;
}

int on_chunk(void* user, int32_t, double t, double h, const float* theta) {
  Run& R = *(Run*)user;
  for (FILE* f : {R.order, R.thetas, R.couplings, R.times})
    if (f) fflush(f);
  if (R.dense >= 0) write_fs(R, theta, (float)t, (float)h, R.floc.data());
  if (R.fail_at > 0 && R.steps >= R.fail_at) {
    for (FILE* f : {R.order, R.thetas, R.couplings, R.times})
      if (f) fclose(f);
    FILE* out = fopen(path(R, ".out").c_str(), "ab");
    if (out) {
      fprintf(out, "\ninjected fault after %lld steps at t=%f\n", R.steps, t);
      fclose(out);
    }
    exit(3);
  }
  return 0;
}

void usage() {
  printf("usage:\tkuramoto [-hvnRFA] [-N N] [-K K] [-D D]\n");
  printf("\t[-c c] [-t t] [-d dt] [-f f] [-s seed] \n");
  printf("\t[-I init] [-r rtol] [-a atol] [-g gpu] filebase \n\n");
  printf("-h for help \n");
  printf("-v for verbose \n");
  printf("-n for normal random frequencies (default is cauchy) \n");
  printf("-R to reload adjacency, frequencies, and initial conditions from files if possible\n");
  printf("-F for fixed timestep \n");
  printf("-A to regenerate volcano adjacency each step to save memory \n");
  printf("D is the output density level. 0 for minimal, 1 for phases, 2 for phases and couplings, 3 for phases, "
         "couplings, and adjacency\n");
  printf("N is number of oscillators. Default 5000. \n");
  printf("K is rank of volcano adjacency. Default 6. \n");
  printf("c is the coupling coefficient. Default 3.0. \n");
  printf("t is total integration time. Default 1e2. \n");
  printf("dt is the time between outputs. Default 1e0. \n");
  printf("f is the scale of the frequencies. Default 1e0. \n");
  printf("seed is random seed. Default 1. \n");
  printf("init is uniform random initial condition scale. Default 0. \n");
  printf("rtol is relative error tolerance. Default 0.\n");
  printf("atol is absolute error tolerance. Default 1e-6.\n");
  printf("gpu is index of the gpu. Default 0.\n");
  printf("filebase is base file name for output. \n");
}

}  // namespace

#define CHECK(call)                                                                   \
  do {                                                                                \
    int rc_ = (call);                                                                 \
    if (rc_ != KURA_OK) {                                                             \
      fprintf(stderr, "kuramoto: %s failed (%d): %s\n", #call, rc_, kura_last_error()); \
      FILE* o_ = fopen(path(R, ".out").c_str(), "ab");                               \
      if (o_) {                                                                       \
        fprintf(o_, "error: %s (%d): %s\n", #call, rc_, kura_last_error());           \
        fclose(o_);                                                                   \
      }                                                                               \
      return 1;                                                                       \
    }                                                                                 \
  } while (0)

int main(int argc, char* argv[]) {
  Run R;
  gettimeofday(&R.start, NULL);
  float c1 = 3.0f, t1 = 1e2f, dt = 1e0f, freq = 1.0f, atl = 1e-6f, rtl = 0, I = 0;
  int gpu = 0, seed = 1, fixed = 0, A = 0;
  unsigned long N = 5000, K = 6;
  char* filebase = nullptr;
  int help = 1, normal = 0, reload = 0;
  int c;
  while (optind < argc) {
    if ((c = getopt(argc, argv, "N:K:I:D:c:g:t:d:f:s:r:a:hvFnRA")) != -1) {
      switch (c) {
        case 'N': N = (int)atoi(optarg); break;
        case 'K': K = (int)atoi(optarg); break;
        case 'A': A = 1; break;
        case 'I': I = (float)atof(optarg); break;
        case 'c': c1 = (float)atof(optarg); break;
        case 'g': gpu = (int)atof(optarg); break;
        case 't': t1 = (float)atof(optarg); break;
        case 'd': dt = (float)atof(optarg); break;
        case 'f': freq = (float)atof(optarg); break;
        case 's': seed = (int)atoi(optarg); break;
        case 'r': rtl = (float)atof(optarg); break;
        case 'a': atl = (float)atof(optarg); break;
        case 'D': R.dense = (int)atoi(optarg); break;
        case 'R': reload = 1; break;
        case 'F': fixed = 1; break;
        case 'h': help = 1; break;
        case 'v': R.verbose = 1; break;
        case 'n': normal = 1; break;
      }
    } else {
      filebase = argv[optind];
      optind++;
      help = 0;
    }
  }
  if (help || !filebase) {
    usage();
    return 0;
  }
  R.base = filebase;
  R.n = N;
  R.floc.assign(2 * N, 0.f);
  float t = 0, h = fixed ? dt : dt / 100;

  FILE* out = fopen(path(R, ".out").c_str(), "ab");
  if (!out) {
    fprintf(stderr, "kuramoto: cannot open %s\n", path(R, ".out").c_str());
    return 1;
  }
  fprintf(out, "%lu %lu %f %f %f %i\n", N, K, t1, dt, c1, seed);
  for (int i = 0; i < argc; i++) fprintf(out, "%s ", argv[i]);
  fprintf(out, "\n");

  kura_config cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.n = (int64_t)N;
  cfg.k = (int32_t)K;
  cfg.coupling = A ? KURA_COUPLING_VOLCANO : KURA_COUPLING_DENSE;
  cfg.batch = 1;
  cfg.seed = seed;
  cfg.atol = atl;
  cfg.rtol = rtl;
  cfg.fixed_step = fixed;
  cfg.device = gpu;
  cfg.dense_level = R.dense;

  size_t fr = 0, total = 0;
  int64_t req = 0;
  if (cudaSetDevice(gpu) != cudaSuccess || cudaMemGetInfo(&fr, &total) != cudaSuccess) {
    printf("CUDA initialization failed\n");
    fprintf(out, "CUDA initialization failed\n");
    fclose(out);
    return EXIT_FAILURE;
  }
  if (kura_memory_required(&cfg, &req) != KURA_OK) {
    fprintf(stderr, "kuramoto: %s\n", kura_last_error());
    fprintf(out, "error: %s\n", kura_last_error());
    fclose(out);
    return 1;
  }
  printf("GPU Memory: %lu %lu %lu\n", (unsigned long)fr, (unsigned long)total, (unsigned long)req);
  fprintf(out, "GPU Memory: %lu %lu %lu\n", (unsigned long)fr, (unsigned long)total, (unsigned long)req);
  if (fr < (size_t)req) {
    printf("GPU Memory low!\n");
    fprintf(out, "GPU Memory low!\n");
    fclose(out);
    return 0;
  }
  fflush(out);

  std::vector<float> yloc(N, 0.f), omegas(N, 0.f);
  // initial state (kuramoto.cu:466-506)
  int reloaded = 0;
  FILE* in;
  if (reload && (in = fopen(path(R, "fs.dat").c_str(), "r"))) {
    reloaded = 1;
    printf("Using initial conditions from file\n");
    fprintf(out, "Using initial conditions from file\n");
    size_t rd = fread(yloc.data(), sizeof(float), N, in);
    if (rd != N) {
      printf("initial conditions file not compatible with N!\n");
      fprintf(out, "initial conditions file not compatible with N!\n");
      reloaded = 0;
    }
    if (reloaded) {
      rd = fread(&t, sizeof(float), 1, in);
      rd = fread(&h, sizeof(float), 1, in);
      if (rd != 1) {
        printf("Couldn't read start time and step!\n");
        fprintf(out, "Couldn't read start time and step!\n");
        reloaded = 0;
      }
    }
    fclose(in);
    printf("Restarting at t=%f with h=%f\n", t, h);
    fprintf(out, "Restarting at t=%f with h=%f\n", t, h);
  }
  // frequencies from file (kuramoto.cu:508-521); read before drawing so that one
  // generator call makes theta0 and then omega from the same rand() sequence
  int freq_loaded = 0, freq_bad = 0;
  if (reload && (in = fopen(path(R, "frequencies.dat").c_str(), "r"))) {
    size_t rd = fread(omegas.data(), sizeof(float), N, in);
    fclose(in);
    freq_loaded = 1;
    freq_bad = (rd != N);
  }
  std::vector<float> th_gen(N);
  if (kura_random_inputs(seed, (int64_t)N, I, freq, normal, !reloaded, !freq_loaded, th_gen.data(),
                         freq_loaded ? nullptr : omegas.data()) != KURA_OK) {
    fprintf(stderr, "kuramoto: bad random input request\n");
    return 1;
  }
  if (!reloaded) {
    printf("Using random initial conditions\n");
    fprintf(out, "Using random initial conditions\n");
    yloc = th_gen;
    in = fopen(path(R, "fs.dat").c_str(), "wb");
    if (in) {
      fwrite(yloc.data(), sizeof(float), N, in);
      fclose(in);
    }
  }
  if (freq_loaded) {
    printf("Using frequencies from file\n");
    fprintf(out, "Using frequencies from file\n");
    if (freq_bad) {
      printf("frequencies not compatible with N!");
      fprintf(out, "frequencies not compatible with N!");
      fclose(out);
      return 0;
    }
  } else {
    printf("Using random frequencies\n");
    fprintf(out, "Using random frequencies\n");
    in = fopen(path(R, "frequencies.dat").c_str(), "wb");
    if (in) {
      fwrite(omegas.data(), sizeof(float), N, in);
      fclose(in);
    }
  }

  kura_handle* H = nullptr;
  CHECK(kura_create(&cfg, &H));
  CHECK(kura_set_frequencies(H, omegas.data(), (int64_t)N));
  CHECK(kura_set_coupling(H, 0, c1));

  // adjacency (kuramoto.cu:557-581)
  if (!A && reload && (in = fopen(path(R, "adj.dat").c_str(), "r"))) {
    printf("Using adjacency from file\n");
    fprintf(out, "Using adjacency from file\n");
    std::vector<float> adj((size_t)N * N, 0.f);
    size_t rd = fread(adj.data(), sizeof(float), (size_t)N * N, in);
    (void)rd;  // a short file leaves zeros, as in the reference
    fclose(in);
    CHECK(kura_set_adjacency(H, adj.data(), (int64_t)N));
  } else {
    printf("Using random adjacency matrix\n");
    fprintf(out, "Using random adjacency matrix\n");
    if (!A) {
      CHECK(kura_generate_adjacency(H));
      if (R.dense >= 3) {
        std::vector<float> adj((size_t)N * N);
        CHECK(kura_get_adjacency(H, adj.data(), (int64_t)N));
        in = fopen(path(R, "adj.dat").c_str(), "wb");
        if (in) {
          fwrite(adj.data(), sizeof(float), (size_t)N * N, in);
          fclose(in);
        }
      }
    }
  }
  fflush(out);
  fclose(out);

  CHECK(kura_set_state(H, 0, yloc.data(), (double)t, (double)h));
  CHECK(kura_set_horizon(H, (double)t1, (double)dt, reloaded ? 0 : 1));
  R.t0 = t;
  R.t1 = t1;

  const char* mode = reloaded ? "ab" : "wb";
  R.order = fopen(path(R, "order.dat").c_str(), mode);
  if (R.dense >= 1) {
    R.thetas = fopen(path(R, "thetas.dat").c_str(), mode);
    R.times = fopen(path(R, "times.dat").c_str(), mode);
  }
  if (R.dense >= 2) R.couplings = fopen(path(R, "couplings.dat").c_str(), mode);

  if (const char* e = getenv("KURA_CHECKPOINT_STEPS")) CHECK(kura_set_launch_attempts(H, atoll(e)));
  if (const char* e = getenv("KURA_FAIL_AT_STEP")) R.fail_at = atoll(e);
  kura_callbacks cb;
  std::memset(&cb, 0, sizeof(cb));
  cb.user = &R;
  cb.on_output = on_output;
  cb.on_chunk = on_chunk;
  if (R.verbose || R.dense >= 1 || R.fail_at > 0) cb.on_step = on_step;
  CHECK(kura_run(H, &cb));
  for (FILE* f : {R.order, R.thetas, R.couplings, R.times})
    if (f) fclose(f);

  // end record (kuramoto.cu:630-647)
  std::vector<float> th(N), cp(2 * N);
  double tf = 0, hf = 0;
  CHECK(kura_final_record(H, 0, th.data(), cp.data(), &tf, &hf));
  write_fs(R, th.data(), (float)tf, (float)hf, cp.data());
  kura_stats st;
  CHECK(kura_get_stats(H, &st));
  kura_destroy(H);

  out = fopen(path(R, ".out").c_str(), "ab");
  double rt = elapsed(R);
  printf("\nruntime: %f\n", rt);
  if (out) {
    fprintf(out, "\nsteps: %i\n", (int)st.accepted);
    fprintf(out, "runtime: %f\n", rt);
    fclose(out);
  }
  return 0;
}
