// Test helper (checker only): the volcano factor bits drawn through the cuRAND
// device API in the call pattern of the reference's m2 kernel
// (kuramoto.cu:57-60, 83-101): curand_init(seed, 0, 0), skipahead(n), then for
// each mode m one curand() and skipahead(N-1).  Writes K*N int8 (+1/-1) to a file.
#include <curand_kernel.h>
#include <cstdio>
#include <cstdlib>
#include <vector>

__global__ void factor(int seed, int n, int k, signed char* u) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  curandStatePhilox4_32_10_t s;
  curand_init(seed, 0, 0, &s);
  skipahead((unsigned long long)i, &s);
  for (int m = 0; m < k; ++m) {
    unsigned v = curand(&s);
    u[(size_t)m * n + i] = (v % 2) ? 1 : -1;
    skipahead((unsigned long long)(n - 1), &s);
  }
}

int main(int argc, char** argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: curand_factor seed n k out\n");
    return 2;
  }
  int seed = atoi(argv[1]), n = atoi(argv[2]), k = atoi(argv[3]);
  size_t bytes = (size_t)n * k;
  signed char* d = nullptr;
  if (cudaMalloc(&d, bytes ? bytes : 1) != cudaSuccess) return 1;
  factor<<<(n + 127) / 128, 128>>>(seed, n, k, d);
  std::vector<signed char> h(bytes);
  if (cudaMemcpy(h.data(), d, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
  cudaFree(d);
  FILE* f = fopen(argv[4], "wb");
  if (!f) return 1;
  fwrite(h.data(), 1, bytes, f);
  fclose(f);
  return 0;
}
