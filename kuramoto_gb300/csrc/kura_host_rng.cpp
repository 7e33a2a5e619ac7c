// kura_host_rng.cpp -- host generation of the random initial phases and
// frequencies with glibc rand(), in the order and arithmetic of the reference
// program (kuramoto.cu:416, 495-541): srand(seed); N draws for theta0 when it is
// generated; then one draw per oscillator for Cauchy frequencies
// f*tan(pi*(u-1/2)) or two for normal ones f*sqrt(-2 log u)*cos(2 pi v), with
// u = rand()/(float)RAND_MAX.  The arithmetic types follow the C++ overloads the
// reference resolves to (float log; double pow, cos and tan), so the frequencies
// are bit-identical to the reference's frequencies.dat.  Compiled without FMA
// contraction so x86_64 and aarch64 agree.
#include <cmath>
#include <cstdlib>
#include "kura.h"

extern "C" int kura_random_inputs(int32_t seed, int64_t n, float init, float freq, int32_t normal,
                                  int32_t gen_theta, int32_t gen_omega, float* theta0, float* omega) {
  if (n < 0 || (gen_theta && !theta0) || (gen_omega && !omega)) return KURA_ERR_INVALID;
  srand(seed);
  if (gen_theta) {
    for (int64_t j = 0; j < n; ++j) {
      double u = 2.0 / RAND_MAX * rand() - 1;
      theta0[j] = (float)(init / 2 * u);
    }
  }
  if (gen_omega) {
    for (int64_t j = 0; j < n; ++j) {
      if (normal) {
        float u = rand() / (float)RAND_MAX;
        float v = rand() / (float)RAND_MAX;
        float lu = std::log(u);
        double amp = std::pow((double)(-2 * lu), 0.5);
        omega[j] = (float)(freq * amp * std::cos(2 * M_PI * v));
      } else {
        float u = rand() / (float)RAND_MAX;
        omega[j] = (float)(freq * std::tan(M_PI * (u - 0.5)));
      }
    }
  }
  return KURA_OK;
}
