// CUDA kernels of the qMC diagram integration (sm_103a): the plain evaluation kernel, the
// finish kernel and the FMA-throughput probe.  The per-sample evaluation itself is in
// qiw_eval.cuh; qiw_kernels_x.cu builds its variant with warped points and per-sample
// output, qiw_batch_kernels.cu the batched-solve kernels.
#include "qiw_eval.cuh"

namespace qiw {

// out[w][e] = -i * scale_w * sum_c partials[c][e] over the CTAs of work item w (in order,
// Kahan-compensated).  Sets *err_word if a result is not finite.
__global__ void finish_kernel(const DevWork *__restrict__ works, const int *__restrict__ cta_first,
                              const double *__restrict__ partials, const int *__restrict__ res_sizes,
                              const int *__restrict__ out_off, double *__restrict__ out,
                              int *__restrict__ err_word) {
  const int wi = blockIdx.x;
  const DevWork &w = works[wi];
  const int rs = res_sizes[wi];
  const int c0 = cta_first[wi];
  for (int e = threadIdx.x; e < rs; e += blockDim.x) {
    double s = 0.0, comp = 0.0;
    for (int c = 0; c < w.n_cta; ++c) {
      double y = partials[(size_t)(c0 + c) * rs + e] - comp;
      double t = s + y;
      comp = (t - s) - y;
      s = t;
    }
    const double v = -w.scale * s;
    if (!isfinite(v)) atomicOr(err_word, 1);
    out[2 * ((size_t)out_off[wi] + e)] = 0.0;
    out[2 * ((size_t)out_off[wi] + e) + 1] = v;
  }
}

// FMA-throughput probe: 8 independent chains per thread keep the pipe full.
template <typename T>
__global__ void fma_peak_kernel(T *out, T b, T c, int iters) {
  T a0 = (T)threadIdx.x, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
  T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
#pragma unroll 1
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fmaT<T>(a0, b, c); a1 = fmaT<T>(a1, b, c); a2 = fmaT<T>(a2, b, c); a3 = fmaT<T>(a3, b, c);
      a4 = fmaT<T>(a4, b, c); a5 = fmaT<T>(a5, b, c); a6 = fmaT<T>(a6, b, c); a7 = fmaT<T>(a7, b, c);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

cudaError_t launch_fma_peak(bool fp32, void *out, int blocks, int threads, int iters, cudaStream_t st) {
  if (fp32) fma_peak_kernel<float><<<blocks, threads, 0, st>>>((float *)out, 0.999999f, 1e-7f, iters);
  else fma_peak_kernel<double><<<blocks, threads, 0, st>>>((double *)out, 0.999999999, 1e-12, iters);
  return cudaGetLastError();
}

// The kernels' Sobol integers for points first .. first + n - 1 (the same sobol_coord the
// evaluation kernels use), out[i][d] row-major.
__global__ void sobol_points_kernel(const uint32_t *__restrict__ m, const uint32_t *__restrict__ x0, int D,
                                    uint64_t first, uint64_t n, uint32_t *__restrict__ out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = first + i;
  const uint32_t gray = (uint32_t)(k ^ (k >> 1));
  for (int d = 0; d < D; ++d) out[i * D + d] = sobol_coord(m + d * 32, __ldg(x0 + d), gray);
}

cudaError_t launch_sobol_points(const uint32_t *m, const uint32_t *x0, int D, uint64_t first, uint64_t n,
                                uint32_t *out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  sobol_points_kernel<<<blocks, 256, 0, st>>>(m, x0, D, first, n, out);
  return cudaGetLastError();
}

// Euclidean norm of each row of a [n][rs] array (per-sample values -> training weights): one
// thread per row, the squares summed in row order.
__global__ void row_norms_kernel(const double *__restrict__ v, uint64_t n, int rs, double *__restrict__ out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *r = v + i * (uint64_t)rs;
  double s = 0.0;
  for (int e = 0; e < rs; ++e) s = fma(r[e], r[e], s);
  out[i] = sqrt(s);
}

cudaError_t launch_row_norms(const double *v, uint64_t n, int rs, double *out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  row_norms_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(v, n, rs, out);
  return cudaGetLastError();
}

template <typename T, int ARENA, int RESMAX, int MINB = (sizeof(T) == 4 ? kMinBlocks32 : kMinBlocks)>
static cudaError_t launch_t(const LaunchArgs &a) {
  size_t smem = eval_smem_bytes(a.threads, RESMAX, a.stage) + (size_t)a.extra_smem;
  DevProblem pb = a.pb;
  pb.tc_stage = 0;
  if (sizeof(T) == 4 && ARENA >= kArenaHuge && a.tc_omul) {   // per-warp staging after the other buffers
    smem = (smem + 15) & ~(size_t)15;
    pb.tc_stage = (int32_t)smem;
    smem += (size_t)((a.threads + 31) / 32) * kTcWarpFloats * sizeof(float);
  }
  auto *k = eval_kernel<T, ARENA, RESMAX, false, MINB>;
  cudaError_t e;
  if (smem > (48u << 10) && (e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
    return e;
  if (a.carveout >= 0 && (e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, a.carveout)))
    return e;
  k<<<a.n_cta, a.threads, smem, a.stream>>>(pb, a.groups, a.works, a.cta_map, a.partials);
  return cudaGetLastError();
}

int arena_class(int64_t arena) {
  if (arena <= kArenaSmall) return 0;
  if (arena <= kArenaLarge) return 1;
  if (arena <= kArenaHuge) return 2;
  return -1;
}

cudaError_t launch_eval(const LaunchArgs &a) {
  if (a.extras) return launch_eval_extras(a);
  const bool big_res = a.res_max > kResSmall;
  const int ac = arena_class(a.arena_max);
  if (a.fp32) {
    if (ac == 0) return big_res ? launch_t<float, kArenaSmall, kResLarge>(a) : launch_t<float, kArenaSmall, kResSmall>(a);
    if (ac == 2)
      return a.dense ? launch_t<float, kArenaHuge, kResLarge, kMinBlocks32DenseHuge>(a)
                     : launch_t<float, kArenaHuge, kResLarge>(a);
    if (a.dense)
      return big_res ? launch_t<float, kArenaLarge, kResLarge, kMinBlocks32Dense>(a)
                     : launch_t<float, kArenaLarge, kResSmall, kMinBlocks32Dense>(a);
    return big_res ? launch_t<float, kArenaLarge, kResLarge>(a) : launch_t<float, kArenaLarge, kResSmall>(a);
  }
  if (ac == 0) return big_res ? launch_t<double, kArenaSmall, kResLarge>(a) : launch_t<double, kArenaSmall, kResSmall>(a);
  if (ac == 2) return launch_t<double, kArenaHuge, kResLarge>(a);
  return big_res ? launch_t<double, kArenaLarge, kResLarge>(a) : launch_t<double, kArenaLarge, kResSmall>(a);
}

cudaError_t launch_finish(const FinishArgs &a) {
  finish_kernel<<<a.n_work, 128, 0, a.stream>>>(a.works, a.cta_first, a.partials, a.res_sizes, a.out_off,
                                               a.out, a.err_word);
  return cudaGetLastError();
}

}  // namespace qiw
