// Launch interface between the C-ABI layer and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "qiw_internal.hpp"

namespace qiw {

constexpr int kMaxThreads = 128;     // samples per CTA (upper bound)
#ifndef QIW_MIN_BLOCKS
#define QIW_MIN_BLOCKS 4
#endif
constexpr int kMinBlocks = QIW_MIN_BLOCKS;  // 128-thread blocks per SM the register budget allows
constexpr int kArenaSmall = 1024;    // per-sample arena instantiations (elements)
constexpr int kArenaLarge = 8192;
constexpr int kArenaHuge = 20480;   // large-sector problems (9x9 blocks); results always kResLarge
constexpr int kResSmall = 64;        // result-size instantiations (sum of d_s^2)
constexpr int kResLarge = 512;

struct LaunchArgs {
  DevProblem pb;
  const DevGroup *groups;
  const DevWork *works;
  const int4 *cta_map;
  double *partials;
  int n_cta, threads;
  int64_t arena_max;
  int res_max;
  bool fp32;
  cudaStream_t stream;
};

struct FinishArgs {
  const DevWork *works;
  const int *cta_first;
  const double *partials;
  const int *res_sizes;
  const int *out_off;
  double *out;
  int *err_word;
  int n_work;
  cudaStream_t stream;
};

int arena_class(int64_t arena);   // 0 small, 1 large, 2 huge, -1 too large
cudaError_t launch_eval(const LaunchArgs &a);
cudaError_t launch_finish(const FinishArgs &a);
cudaError_t launch_fma_peak(bool fp32, void *out, int blocks, int threads, int iters, cudaStream_t st);

}  // namespace qiw
