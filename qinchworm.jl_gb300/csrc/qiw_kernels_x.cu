// Evaluation kernel with the warped-point and per-sample-output paths compiled in
// (qiw_integrate_warped, qiw_integrate_samples).
#include "qiw_eval.cuh"

namespace qiw {

template <typename T, int ARENA, int RESMAX, int MINB = (sizeof(T) == 4 ? kMinBlocks32 : kMinBlocks)>
static cudaError_t launch_x(const LaunchArgs &a) {
  eval_kernel<T, ARENA, RESMAX, true, MINB><<<a.n_cta, a.threads, eval_smem_bytes(a.threads, RESMAX, a.stage), a.stream>>>(a.pb, a.groups, a.works, a.cta_map,
                                                                             a.partials);
  return cudaGetLastError();
}

cudaError_t launch_eval_extras(const LaunchArgs &a) {
  const bool big_res = a.res_max > kResSmall;
  const int ac = arena_class(a.arena_max);
  if (a.fp32) {
    if (ac == 0) return big_res ? launch_x<float, kArenaSmall, kResLarge>(a) : launch_x<float, kArenaSmall, kResSmall>(a);
    if (ac == 2)
      return a.dense ? launch_x<float, kArenaHuge, kResLarge, kMinBlocks32DenseHuge>(a)
                     : launch_x<float, kArenaHuge, kResLarge>(a);
    if (a.dense)
      return big_res ? launch_x<float, kArenaLarge, kResLarge, kMinBlocks32Dense>(a)
                     : launch_x<float, kArenaLarge, kResSmall, kMinBlocks32Dense>(a);
    return big_res ? launch_x<float, kArenaLarge, kResLarge>(a) : launch_x<float, kArenaLarge, kResSmall>(a);
  }
  if (ac == 0) return big_res ? launch_x<double, kArenaSmall, kResLarge>(a) : launch_x<double, kArenaSmall, kResSmall>(a);
  if (ac == 2) return launch_x<double, kArenaHuge, kResLarge>(a);
  return big_res ? launch_x<double, kArenaLarge, kResLarge>(a) : launch_x<double, kArenaLarge, kResSmall>(a);
}

}  // namespace qiw
