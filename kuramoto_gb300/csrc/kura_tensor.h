// kura_tensor.h -- host interface of the tcgen05 shared-adjacency ensemble engine
// (kura_tensor.cu), used by the C ABI when a dense network carries a large batch.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>
#include "kura.h"
#include "kura_kernels.cuh"

namespace kura {

class TensorEngine {
 public:
  struct Impl;
  TensorEngine();
  ~TensorEngine();
  int init(int64_t n, int k, int batch, int seed, double atol, double rtol, int fixed, int dense_level, int device,
           cudaStream_t st);
  static size_t memory_required(int64_t n, int batch);
  int set_frequencies(const float* omega);
  int generate_adjacency();
  int set_adjacency(const float* adj_host);
  int get_adjacency(float* adj_host);
  float* staging(int b);  // device buffer of n floats for trajectory b's uploads
  int set_state(int b, const float* theta_dev, const TrajG& T);
  int set_horizon(const std::vector<float>& t_eval, int ring, std::vector<TrajG>& traj);
  // integrates until every trajectory is done or, with max_replays > 0, after that many step
  // attempts (rounded up to a multiple of four: the attempt graph is replayed four at a time)
  int run(std::vector<TrajG>& traj, kura_stats& stats, long long max_replays = -1);
  int read_order(int b, int count, float* r, int* idx);  // records: r and output index (-1: t0)
  int get_state(int b, int rot_y, float* theta);
  int evaluate(int mode, int b, float* theta_out, float* coup_out);  // 1: end record, 2: RHS
  int sync_traj(std::vector<TrajG>& traj, bool to_device);
  static const char* last_error();
  Impl* d;
};

}  // namespace kura
