// Kernels of the batched independent solves (qiw_batch_*): persistent evaluation over the
// tiles of many solves, per-work-item finish, per-solve P update and normalisation.
#include "qiw_eval.cuh"

namespace qiw {

// ---------------------------------------------------------------------------------------
// Batched solves.  A persistent CTA takes tiles from the step's list (heaviest first) with an
// atomic ticket; tiles of solves whose loop has ended are skipped.  The times of a tile are
// those of its solve at this step: (tau_0, 0, tau_1) for the bare step 0, else
// (tau_0, tau_step, tau_{step+1}) as in src/inchworm.jl:474-493.

template <typename T, int ARENA, int RESMAX>
__global__ void __launch_bounds__(kMaxThreads, kMinBlocks)
    batch_eval_kernel(const DevProblem *__restrict__ probs, const BatchSolve *__restrict__ solves,
                      const DevGroup *__restrict__ groups, const BatchWork *__restrict__ works,
                      const int4 *__restrict__ tiles, int n_tiles, int *ticket, double *__restrict__ partials,
                      int pstride, int step) {
  __shared__ DevProblem spb;
  __shared__ int s_tile;
  for (;;) {
    __syncthreads();  // the previous tile is done with spb and s_tile
    if (threadIdx.x == 0) {
      const int t = atomicAdd(ticket, 1);
      s_tile = t;
      if (t < n_tiles) spb = probs[works[tiles[t].x].solve];
    }
    __syncthreads();
    const int t = s_tile;
    if (t >= n_tiles) return;
    const int4 cm = tiles[t];
    const BatchWork &w = works[cm.x];
    if (step > w.last_step) continue;
    const BatchSolve &so = solves[w.solve];
    const DevGroup &g = groups[w.group];
    const double t_i = so.taus[0];
    const double t_w = step == 0 ? 0.0 : so.taus[step];
    const double t_f = so.taus[step + 1];
    const TileSrc src{t_i, t_w, t_f, 0, w.n_samples, w.m, w.x0, nullptr, nullptr};
    eval_tile<T, ARENA, RESMAX, false>(spb, g, src, cm.y, (uint64_t)cm.z,
                                [=]() { return partials + (size_t)tiles[t].w * pstride; });
  }
}

// Contour Jacobian of a group at the step's times (simplex volumes, as on the host).
__device__ __forceinline__ double dev_simplex_volume(int d, double edge) {
  double v = 1.0;
  for (int i = 1; i <= d; ++i) v *= edge / (double)i;
  return d > 0 ? v : 1.0;
}

// res[w] = J/N * sum of the work item's partial slots (in order, Kahan-compensated): its
// contribution to i*P(tau_{step+1}).
__global__ void batch_finish_kernel(const BatchSolve *__restrict__ solves, const DevGroup *__restrict__ groups,
                                    const BatchWork *__restrict__ works, const double *__restrict__ partials,
                                    int pstride, double *__restrict__ res, int *err_word, int step) {
  const BatchWork &w = works[blockIdx.x];
  if (step > w.last_step) return;
  const DevGroup &g = groups[w.group];
  const BatchSolve &so = solves[w.solve];
  double scale = 1.0;  // order 0: one exact evaluation
  if (g.D > 0) {
    const double t_i = so.taus[0], t_f = so.taus[step + 1];
    const double t_w = step == 0 ? 0.0 : so.taus[step];
    const double J = (g.kind == QIW_GROUP_BARE)
                         ? dev_simplex_volume(g.D, t_f - t_i)
                         : dev_simplex_volume(g.d_before, t_w - t_i) * dev_simplex_volume(g.d_after, t_f - t_w);
    scale = J * w.inv_n;
  }
  const int rs = g.res_size;
  for (int e = threadIdx.x; e < rs; e += blockDim.x) {
    double s = 0.0, comp = 0.0;
    for (int c = 0; c < w.n_slots; ++c) {
      const double y = partials[(size_t)(w.slot0 + c) * pstride + e] - comp;
      const double t = s + y;
      comp = (t - s) - y;
      s = t;
    }
    const double v = scale * s;
    if (!isfinite(v)) atomicOr(err_word, 1);
    res[w.res_off + e] = v;
  }
}

// One CTA per solve: i*P(tau_j), j = step + 1, is the sum of the step's work items -- per
// order first, then over orders, as the host does -- (src/ppgf.jl:474-504); after a bold
// step every tau is rescaled by exp(-tau lambda), lambda = log(max_s,i i*P_s,ii(tau_j)) / tau_j
// (normalize!(P, tau), src/ppgf.jl:646-654).  The FP32 copy is refreshed.  A largest diagonal
// that is not positive and finite has no logarithm: the solve's P is left unscaled and bit 1
// of the error word is set (the host reports QIW_ERR_DEVICE, as normalize_tau raises on it).
__global__ void batch_update_kernel(const DevProblem *__restrict__ probs, const BatchSolve *__restrict__ solves,
                                    const BatchWork *__restrict__ works, const double *__restrict__ res,
                                    int *err_word, int step) {
  const BatchSolve &so = solves[blockIdx.x];
  if (step > so.last_step) return;
  const DevProblem &pb = probs[blockIdx.x];
  const bool bare = step == 0;
  const int w0 = bare ? so.bare0 : so.bold0, w1 = bare ? so.bare1 : so.bold1;
  const int j = step + 1;
  __shared__ double nv[kResLarge];
  __shared__ double s_lam;
  for (int e = threadIdx.x; e < so.res_size; e += blockDim.x) {
    double tot = 0.0, co = 0.0;
    int cur = w0 < w1 ? works[w0].order : 0;
    for (int w = w0; w < w1; ++w) {
      if (works[w].order != cur) {
        tot += co;
        co = 0.0;
        cur = works[w].order;
      }
      co += res[works[w].res_off + e];
    }
    nv[e] = tot + co;
  }
  __syncthreads();
  for (int s = 0; s < pb.S; ++s) {
    const int d = pb.dims[s];
    for (int e = threadIdx.x; e < d * d; e += blockDim.x)
      so.P[pb.ptab_off[s] + (size_t)j * d * d + e] = nv[pb.res_off[s] + e];
  }
  if (!bare) {
    if (threadIdx.x == 0) {
      double pmax = -INFINITY;
      for (int s = 0; s < pb.S; ++s) {
        const int d = pb.dims[s];
        for (int i = 0; i < d; ++i) pmax = fmax(pmax, nv[pb.res_off[s] + i * d + i]);
      }
      double lam = 0.0;
      if (pmax > 0.0 && isfinite(pmax)) lam = log(pmax) / so.taus[j];
      else atomicOr(err_word, 2);
      s_lam = lam;
      so.lam[j] = lam;
    }
    __syncthreads();
    const double lam = s_lam;
    for (int s = 0; s < pb.S; ++s) {
      const int dd = pb.dims[s] * pb.dims[s];
      const int n = pb.n_tau * dd;
      double *P = so.P + pb.ptab_off[s];
      for (int q = threadIdx.x; q < n; q += blockDim.x) P[q] *= exp(-(so.taus[q / dd] * lam));
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < so.ptab_size; q += blockDim.x) so.Pf[q] = (float)so.P[q];
}

__global__ void batch_reset_kernel(const BatchSolve *__restrict__ solves) {
  const BatchSolve &so = solves[blockIdx.x];
  for (int q = threadIdx.x; q < so.ptab_size; q += blockDim.x) {
    const double v = so.P0[q];
    so.P[q] = v;
    so.Pf[q] = (float)v;
  }
  for (int q = threadIdx.x; q < so.n_tau; q += blockDim.x) so.lam[q] = 0.0;
}

template <typename T, int ARENA, int RESMAX>
static cudaError_t launch_batch_t(const BatchArgs &a) {
  batch_eval_kernel<T, ARENA, RESMAX><<<a.grid, a.threads, eval_smem_bytes(a.threads, RESMAX, a.stage), a.stream>>>(
      a.probs, a.solves, a.groups, a.works, a.tiles, a.n_tiles, a.ticket, a.partials, a.pstride, a.step);
  return cudaGetLastError();
}

template <typename T, int ARENA, int RESMAX>
static int occ_t(int threads, bool stage) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batch_eval_kernel<T, ARENA, RESMAX>, threads,
                                                    eval_smem_bytes(threads, RESMAX, stage)) !=
      cudaSuccess)
    return 0;
  return b;
}

#define QIW_BATCH_DISPATCH(F, ...)                                                                    \
  do {                                                                                                \
    const bool big_res = a.res_max > kResSmall;                                                       \
    const int ac = arena_class(a.arena_max);                                                          \
    if (a.fp32) {                                                                                     \
      if (ac == 0) return big_res ? F<float, kArenaSmall, kResLarge>(__VA_ARGS__)                     \
                                  : F<float, kArenaSmall, kResSmall>(__VA_ARGS__);                    \
      if (ac == 1) return big_res ? F<float, kArenaLarge, kResLarge>(__VA_ARGS__)                     \
                                  : F<float, kArenaLarge, kResSmall>(__VA_ARGS__);                    \
      return F<float, kArenaHuge, kResLarge>(__VA_ARGS__);                                            \
    }                                                                                                 \
    if (ac == 0) return big_res ? F<double, kArenaSmall, kResLarge>(__VA_ARGS__)                      \
                                : F<double, kArenaSmall, kResSmall>(__VA_ARGS__);                     \
    if (ac == 1) return big_res ? F<double, kArenaLarge, kResLarge>(__VA_ARGS__)                      \
                                : F<double, kArenaLarge, kResSmall>(__VA_ARGS__);                     \
    return F<double, kArenaHuge, kResLarge>(__VA_ARGS__);                                             \
  } while (0)

cudaError_t launch_batch_eval(const BatchArgs &a) { QIW_BATCH_DISPATCH(launch_batch_t, a); }

int batch_occupancy(const BatchArgs &a, int *blocks_per_sm) {
  auto f = [&]() -> int { QIW_BATCH_DISPATCH(occ_t, a.threads, a.stage); };
  *blocks_per_sm = f();
  return *blocks_per_sm > 0 ? 0 : 1;
}

cudaError_t launch_batch_finish(const BatchArgs &a) {
  batch_finish_kernel<<<a.n_works, 128, 0, a.stream>>>(a.solves, a.groups, a.works, a.partials, a.pstride, a.res,
                                                       a.err_word, a.step);
  return cudaGetLastError();
}

cudaError_t launch_batch_reset(const BatchArgs &a) {
  batch_reset_kernel<<<a.n_solves, 256, 0, a.stream>>>(a.solves);
  return cudaGetLastError();
}

cudaError_t launch_batch_update(const BatchArgs &a) {
  batch_update_kernel<<<a.n_solves, 128, 0, a.stream>>>(a.probs, a.solves, a.works, a.res, a.err_word, a.step);
  return cudaGetLastError();
}

}  // namespace qiw
