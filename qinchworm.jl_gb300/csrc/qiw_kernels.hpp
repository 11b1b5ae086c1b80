// Launch interface between the C-ABI layer and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "qiw_internal.hpp"

namespace qiw {

constexpr int kMaxThreads = 128;     // samples per CTA (upper bound)
#ifndef QIW_MIN_BLOCKS
#define QIW_MIN_BLOCKS 5
#endif
constexpr int kMinBlocks = QIW_MIN_BLOCKS;  // 128-thread blocks per SM: FP64 at 94 registers, no spills
#ifndef QIW_MIN_BLOCKS_FP32
#define QIW_MIN_BLOCKS_FP32 5
#endif
constexpr int kMinBlocks32 = QIW_MIN_BLOCKS_FP32;  // the same bound for the FP32 kernels
// FP32 launches of many waves (throughput-bound) use kernels compiled for more resident blocks:
// small-block programs 7 per SM (72 registers), large-block programs 6 (80 registers).
constexpr int kMinBlocks32Dense = 7;
constexpr int kMinBlocks32DenseHuge = 6;
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
  bool extras;               // a work item has warped points or per-sample output
  bool stage;                // a group is scalar: shared-memory instruction staging buffers
  int extra_smem = 0;        // extra dynamic shared memory per CTA (occupancy tuning)
  bool tc_omul = false;      // FP32: operator multiplies of 9-wide blocks on tensor cores (large-block kernels)
  int carveout = -1;         // preferred shared-memory carveout, percent (-1: driver default)
  bool dense = false;        // FP32, many waves of tiles: the kernels with more resident blocks
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

// ---- batched solves (csrc/qiw_batch.cu): many independent inchworm loops in one launch queue

// One (solve, group) pair; its tiles hold partial slots [slot0, slot0 + n_slots).
struct BatchWork {
  int32_t group, solve, order, last_step;   // last_step: last step this work item runs
  int32_t slot0, n_slots, res_off, pad;
  uint64_t n_samples;
  double inv_n;                             // 1 / n_samples (one rank, one sequence)
  const uint32_t *m, *x0;                   // Sobol tables [D][32], [D]
};

// One solve: its grid, device P tables and the ranges of its work items.
struct BatchSolve {
  const double *taus;     // [n_tau]
  const double *P0;       // initial i*P table (FP64)
  double *P;              // i*P table, FP64 (layout of DevProblem::P)
  float *Pf;              // FP32 copy read by the FP32 kernels
  double *lam;            // [n_tau] normalisation exponent of each step (output)
  int32_t last_step;      // last bold step (1 .. n_tau - 2); 0: bare step only
  int32_t bare0, bare1;   // bare work items [bare0, bare1) of the bare list
  int32_t bold0, bold1;   // bold work items [bold0, bold1) of the bold list
  int32_t res_size, ptab_size, n_tau;
};

struct BatchArgs {
  const DevProblem *probs;   // [n_solves], views of the launch precision
  const BatchSolve *solves;
  const DevGroup *groups;
  const BatchWork *works;    // this step's list (bare for step 0, bold otherwise)
  const int4 *tiles;         // (work, batch, first sample, partial slot), heaviest first
  int *ticket;               // this step's tile counter (zero before the launch)
  double *partials;          // [slots][pstride]
  int pstride;               // elements per partial slot (largest result size)
  double *res;               // per work item result (i*P units) at res_off
  int *err_word;
  int n_tiles, n_works, n_solves, step, grid, threads;
  int64_t arena_max;
  int res_max;
  bool fp32;
  bool stage;                // a plan is scalar: shared-memory instruction staging buffers
  cudaStream_t stream;
};

cudaError_t launch_batch_eval(const BatchArgs &a);     // persistent evaluation of one step
cudaError_t launch_batch_finish(const BatchArgs &a);   // per work item results of the step
cudaError_t launch_batch_update(const BatchArgs &a);   // P(tau_{step+1}) and normalize!(P, tau)
cudaError_t launch_batch_reset(const BatchArgs &a);    // P = P0 for every solve
int batch_occupancy(const BatchArgs &a, int *blocks_per_sm);

int arena_class(int64_t arena);   // 0 small, 1 large, 2 huge, -1 too large
cudaError_t launch_eval(const LaunchArgs &a);
cudaError_t launch_eval_extras(const LaunchArgs &a);   // csrc/qiw_kernels_x.cu
cudaError_t launch_finish(const FinishArgs &a);
cudaError_t launch_fma_peak(bool fp32, void *out, int blocks, int threads, int iters, cudaStream_t st);
// out[i] = || v[i][0 .. rs) ||_2 for i < n.
cudaError_t launch_row_norms(const double *v, uint64_t n, int rs, double *out, cudaStream_t st);
cudaError_t launch_sobol_points(const uint32_t *m, const uint32_t *x0, int D, uint64_t first, uint64_t n,
                                uint32_t *out, cudaStream_t st);

}  // namespace qiw
