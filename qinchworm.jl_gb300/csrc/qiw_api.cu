// C-ABI implementation: contexts, problem upload, group planning, integration calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "qiw_ctx.hpp"
#include "qiw_dispatch.hpp"

using namespace qiw;

namespace {

// Natural cubic spline of y on a uniform grid; per segment a0 + a1 f + a2 f^2 + a3 f^3.
void cubic_coeffs(const std::vector<double> &y, double h, std::vector<double> *out) {
  const int n = (int)y.size();
  std::vector<double> M(n, 0.0);
  if (n >= 3) {
    const int m = n - 2;
    std::vector<double> cp(m), dp(m);
    for (int i = 0; i < m; ++i) {
      double rhs = 6.0 * (y[i + 2] - 2.0 * y[i + 1] + y[i]) / (h * h);
      double den = (i == 0) ? 4.0 : 4.0 - cp[i - 1];
      cp[i] = 1.0 / den;
      dp[i] = (i == 0) ? rhs / den : (rhs - dp[i - 1]) / den;
    }
    M[m] = dp[m - 1];
    for (int i = m - 2; i >= 0; --i) M[i + 1] = dp[i] - cp[i] * M[i + 2];
  }
  out->assign(4 * (size_t)n, 0.0);  // n-1 segments (+1 padding segment)
  const double h2 = h * h;
  for (int j = 0; j + 1 < n; ++j) {
    (*out)[4 * j + 0] = y[j];
    (*out)[4 * j + 1] = (y[j + 1] - y[j]) - h2 * (2.0 * M[j] + M[j + 1]) / 6.0;
    (*out)[4 * j + 2] = h2 * M[j] / 2.0;
    (*out)[4 * j + 3] = h2 * (M[j + 1] - M[j]) / 6.0;
  }
}

double simplex_volume(int d, double edge) {
  double v = 1.0;
  for (int i = 1; i <= d; ++i) v *= edge / (double)i;
  return d > 0 ? v : 1.0;
}

}  // namespace

namespace qiw {

int integrate_impl(qiw_ctx *c, int32_t n_work, const qiw_work_desc *work, int32_t precision, double *out,
                   const int32_t *warp_ids, double *sample_out, double *norms_out) {
  if (!c || n_work < 0 || (n_work > 0 && (!work || !out))) return QIW_ERR_ARG;
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_integrate: cudaSetDevice");
  if (n_work == 0) return QIW_OK;
  LaunchTables t;
  int rc = prepare_launch(c, n_work, work, precision, &t);
  if (rc) return rc;
  if ((rc = sync_groups(c))) return rc;
  cudaStream_t st = c->stream;
  if ((rc = c->cuda(c->d_sobol.upload(t.sobol.data(), t.sobol.size(), st), "upload Sobol"))) return rc;
  for (auto &w : t.works) {
    w.m = c->d_sobol.p + (uintptr_t)w.m;
    w.x0 = c->d_sobol.p + (uintptr_t)w.x0;
  }
  // warped points: one buffer, one region per warped work item
  if (warp_ids) {
    size_t total = 0;
    std::vector<size_t> poff(n_work, 0);
    for (int i = 0; i < n_work; ++i) {
      const int id = warp_ids[i];
      if (id < 0) continue;
      const Plan &p = c->groups[work[i].group]->plan;
      if (id >= (int)c->warps.size() || warp_dim(c, id) != p.D)
        return c->fail(QIW_ERR_ARG, "qiw_integrate_warped: warp id invalid or of the wrong dimension");
      poff[i] = total;
      total += (size_t)t.works[i].n_samples * (p.D + 1);
    }
    if (total > 0) {
      if ((rc = c->cuda(c->d_pts.reserve(total), "alloc warped points"))) return rc;
      // the maps of different items are independent: several run concurrently on auxiliary
      // streams (each a few CTAs), joined back before the evaluation launch
      int n_warped = 0;
      for (int i = 0; i < n_work; ++i) n_warped += warp_ids[i] >= 0 && t.works[i].n_samples > 0;
      const int n_st = n_warped > 1 ? std::min(n_warped, kAuxStreams) : 0;
      if (n_st > 0 && ((rc = aux_streams(c, n_st)) || (rc = aux_fork(c, n_st)))) return rc;
      int k = 0;
      for (int i = 0; i < n_work; ++i) {
        if (warp_ids[i] < 0) continue;
        double *dst = c->d_pts.p + poff[i];
        if ((rc = warp_map_device(c, warp_ids[i], t.works[i].m, t.works[i].x0, t.works[i].first_index,
                                  t.works[i].n_samples, dst, n_st > 0 ? c->aux[k++ % n_st] : nullptr)))
          break;
        t.works[i].pts = dst;
      }
      const int rj = n_st > 0 ? aux_join(c, n_st) : QIW_OK;
      if (rc || (rc = rj)) return rc;
    }
  }
  // per-sample values: one region per work item, in work order
  size_t n_sample_vals = 0;
  if (sample_out || norms_out) {
    for (int i = 0; i < n_work; ++i) n_sample_vals += (size_t)t.works[i].n_samples * t.res_sizes[i];
    if ((rc = c->cuda(c->d_samples.reserve(n_sample_vals), "alloc samples")) ||
        (rc = c->cuda(cudaMemsetAsync(c->d_samples.p, 0, sizeof(double) * n_sample_vals, st), "clear samples")))
      return rc;
    size_t o = 0;
    for (int i = 0; i < n_work; ++i) {
      t.works[i].sample_out = c->d_samples.p + o;
      o += (size_t)t.works[i].n_samples * t.res_sizes[i];
    }
  }
  const int n_cta = (int)t.cta_map.size();
  int zero = 0;
  if ((rc = c->cuda(c->d_works.upload(t.works.data(), t.works.size(), st), "upload work")) ||
      (rc = c->cuda(c->d_cta_map.upload(t.cta_map.data(), t.cta_map.size(), st), "upload work")) ||
      (rc = c->cuda(c->d_cta_first.upload(t.cta_first.data(), t.cta_first.size(), st), "upload work")) ||
      (rc = c->cuda(c->d_res_sizes.upload(t.res_sizes.data(), t.res_sizes.size(), st), "upload work")) ||
      (rc = c->cuda(c->d_out_off.upload(t.out_off.data(), t.out_off.size(), st), "upload work")) ||
      (rc = c->cuda(c->d_err.upload(&zero, 1, st), "upload work")) ||
      (rc = c->cuda(c->d_partials.reserve((size_t)n_cta * t.res_max), "alloc partials")) ||
      (rc = c->cuda(c->d_out.reserve((size_t)2 * t.out_total), "alloc out")))
    return rc;
  const DevGroup *dgroups = t.level > 0 ? c->d_groups_split[t.level - 1].p : c->d_groups.p;
  rc = launch_tables(c, t, precision, dgroups, c->d_works.p, c->d_cta_map.p, c->d_cta_first.p,
                     c->d_res_sizes.p, c->d_out_off.p, c->d_partials.p, c->d_err.p, c->d_out.p);
  if (rc) return rc;
  int err_word = 0;
  if ((rc = c->cuda(cudaMemcpyAsync(out, c->d_out.p, sizeof(double) * 2 * t.out_total, cudaMemcpyDeviceToHost, st), "copy out")) ||
      (rc = c->cuda(cudaMemcpyAsync(&err_word, c->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st), "copy err")))
    return rc;
  if (sample_out && n_sample_vals > 0 &&
      (rc = c->cuda(cudaMemcpyAsync(sample_out, c->d_samples.p, sizeof(double) * n_sample_vals,
                                    cudaMemcpyDeviceToHost, st), "copy samples")))
    return rc;
  if (norms_out) {   // per-sample norms only: the values stay on the device
    size_t n_rows = 0;
    for (int i = 0; i < n_work; ++i) n_rows += (size_t)t.works[i].n_samples;
    if ((rc = c->cuda(c->d_norms.reserve(n_rows), "alloc norms"))) return rc;
    size_t o = 0, r = 0;
    for (int i = 0; i < n_work; ++i) {
      const uint64_t n = t.works[i].n_samples;
      if ((rc = c->cuda(launch_row_norms(c->d_samples.p + o, n, t.res_sizes[i], c->d_norms.p + r, st), "norm kernel")))
        return rc;
      o += (size_t)n * t.res_sizes[i];
      r += (size_t)n;
    }
    if (n_rows > 0 &&
        (rc = c->cuda(cudaMemcpyAsync(norms_out, c->d_norms.p, sizeof(double) * n_rows, cudaMemcpyDeviceToHost, st),
                      "copy norms")))
      return rc;
  }
  if ((rc = c->cuda(cudaStreamSynchronize(st), "integrate"))) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->last_ms = ms;
  if (err_word) return c->fail(QIW_ERR_DEVICE, "qiw_integrate: non-finite result detected on the device");
  return QIW_OK;
}

// Split level of an FP32 launch.  A thread runs its batch's instructions one after another, and
// at few waves of tiles the launch lasts as long as its longest batch; split-batch programs
// shorten that at the price of more instructions in all.  Measured on the eg inch step (ms per
// step, no split / 11000 / 9000 instructions per batch): 512 samples 13.6 / 10.9 / 9.7, 1024
// 14.3 / 13.2 / 14.5, 4096 44.7 / 47.4 / 51.4.  So: under 1.5 waves level 2, under 4 level 1,
// otherwise the plain programs.  QIW_SPLIT_LEVEL=0|1|2 fixes the level (tuning).
// *waves: the launch's tiles x threads over the SMs' resident threads (plain programs).
static int split_level(qiw_ctx *c, int32_t n_work, const qiw_work_desc *work, double *waves_out) {
  *waves_out = 0.0;
  if (c->n_sm <= 0) return 0;
  bool any = false;
  double tiles_x_threads = 0.0;   // samples in flight over the launch, tiles counted whole
  for (int i = 0; i < n_work; ++i) {
    const qiw_work_desc &wd = work[i];
    if (wd.group < 0 || wd.group >= (int)c->groups.size()) return 0;   // rejected by the caller
    const GroupRec &g = *c->groups[wd.group];
    any = any || g.split[0] != nullptr;
    const uint64_t n = g.plan.D == 0 ? 1 : wd.n_samples;
    const double tiles = (double)((n + c->threads32 - 1) / c->threads32);
    tiles_x_threads += tiles * c->threads32 * (double)(g.plan.batch_begin.size() - 1);
  }
  const double waves = tiles_x_threads / ((double)c->n_sm * kMinBlocks32 * kMaxThreads);
  *waves_out = waves;
  if (const char *e = std::getenv("QIW_SPLIT_LEVEL")) return std::max(0, std::min(kSplitLevels, std::atoi(e)));
  if (!any) return 0;
  return waves < 1.5 ? 2 : waves < 4.0 ? 1 : 0;
}

int prepare_launch(qiw_ctx *c, int32_t n_work, const qiw_work_desc *work, int32_t precision, LaunchTables *t) {
  if (precision != QIW_PREC_FP64 && precision != QIW_PREC_FP32 && precision != QIW_PREC_FP32_TC)
    return c->fail(QIW_ERR_ARG, "qiw_integrate: unknown precision");
  if (!c->has_problem) return c->fail(QIW_ERR_ARG, "qiw_integrate: no problem set");
  bool need_P = false;
  t->works.assign(n_work, DevWork());
  t->cta_first.assign(n_work, 0);
  t->res_sizes.assign(n_work, 0);
  t->out_off.assign(n_work, 0);
  const int threads = precision == QIW_PREC_FP64 ? c->threads : c->threads32;  // samples per tile
  t->level = precision == QIW_PREC_FP64 ? 0 : split_level(c, n_work, work, &t->waves);
  for (int i = 0; i < n_work; ++i) {
    const qiw_work_desc &wd = work[i];
    if (wd.group < 0 || wd.group >= (int)c->groups.size()) return c->fail(QIW_ERR_ARG, "qiw_integrate: bad group id");
    const Plan &p = c->groups[wd.group]->level(t->level).plan;
    if (p.use_bold) need_P = true;
    if (p.D > 0 && (!wd.sobol_m || !wd.sobol_x0)) return c->fail(QIW_ERR_ARG, "qiw_integrate: Sobol tables missing");
    const bool no_tw = p.kind == QIW_GROUP_BARE || p.kind == QIW_GROUP_SIGMA;
    if (!(wd.t_i <= wd.t_f) || (!no_tw && !(wd.t_i <= wd.t_w && wd.t_w <= wd.t_f)))
      return c->fail(QIW_ERR_ARG, "qiw_integrate: times must satisfy t_i <= t_w <= t_f");
    if (p.D > 0 && (wd.n_total == 0 || wd.first_index + wd.n_samples > (1ull << 32)))
      return c->fail(QIW_ERR_ARG, "qiw_integrate: Sobol index range beyond 2^32 or N_total = 0");
    DevWork &w = t->works[i];
    std::memset(&w, 0, sizeof(w));
    w.group = wd.group;
    w.t_i = wd.t_i;
    w.t_w = wd.t_w;
    w.t_f = wd.t_f;
    w.first_index = wd.first_index;
    if (wd.transform != QIW_TRANSFORM_DEFAULT) {
      if (wd.transform != QIW_TRANSFORM_SORT && wd.transform != QIW_TRANSFORM_EXPMODEL)
        return c->fail(QIW_ERR_ARG, "qiw_integrate: unknown transform");
      if (p.kind != QIW_GROUP_BARE) return c->fail(QIW_ERR_ARG, "qiw_integrate: SORT / EXPMODEL maps apply to bare groups");
      if (wd.transform == QIW_TRANSFORM_EXPMODEL && (wd.t_i != 0.0 || !(wd.t_w > 0.0)))
        return c->fail(QIW_ERR_ARG, "qiw_integrate: EXPMODEL needs t_i = 0 and the decay rate (t_w) > 0");
      w.transform = wd.transform;
      w.decay = wd.t_w;
    }
    // Phase of the result: the kernels compute real chains and the finish step returns
    // -i * scale * sum.  Bold, bare and correlator groups carry -i * parity (the reference's
    // -i parity (-1)^k times (-i)^(2k) branch factors); self-energy groups integrate 2k - 2
    // times only, which leaves +i * parity: their scale is negated.
    const double phase = (p.kind == QIW_GROUP_SIGMA) ? -1.0 : 1.0;
    if (p.D == 0) {
      w.n_samples = 1;
      w.scale = phase;  // order 0 (and order-1 self-energy): evaluated exactly, no qMC average
      w.transform = QIW_TRANSFORM_DEFAULT;
    } else {
      w.n_samples = wd.n_samples;
      double J = (p.kind == QIW_GROUP_BARE || p.kind == QIW_GROUP_SIGMA)
                     ? simplex_volume(p.D, wd.t_f - wd.t_i)
                     : simplex_volume(p.d_before, wd.t_w - wd.t_i) * simplex_volume(p.d_after, wd.t_f - wd.t_w);
      if (w.transform == QIW_TRANSFORM_EXPMODEL) J = 1.0;  // per sample in the kernel
      w.scale = phase * J / (double)wd.n_total;
    }
    const int n_tiles = (int)((w.n_samples + threads - 1) / threads);
    const int n_b = std::max(0, (int)p.batch_begin.size() - 1);
    w.n_cta = n_tiles * n_b;
    t->cta_first[i] = (int)t->cta_map.size();
    // within the work item the batches go heaviest first; every tile has its own partial row
    std::vector<int> order(n_b);
    for (int b = 0; b < n_b; ++b) order[b] = b;
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return p.batch_flops[x] > p.batch_flops[y]; });
    for (int b : order)
      for (int k = 0; k < n_tiles; ++k) {
        const int slot = (int)t->cta_map.size();  // partial row: the finish kernel sums a work item's rows in order
        t->cta_map.push_back(make_int4(i, b, k * threads, slot));
        const uint64_t s0 = (uint64_t)k * threads;
        const double n_in = (double)std::min<uint64_t>((uint64_t)threads, w.n_samples - s0);
        t->cta_cost.push_back(p.batch_flops[b] * n_in);
      }
    t->res_sizes[i] = p.res_size;
    t->out_off[i] = t->out_total;
    t->out_total += p.res_size;
    t->arena_max = std::max<int64_t>(t->arena_max, p.arena);
    t->res_max = std::max(t->res_max, p.res_size);
    // Sobol tables: offsets into t->sobol, turned into device pointers when placed
    w.m = reinterpret_cast<const uint32_t *>((uintptr_t)t->sobol.size());
    if (p.D > 0) t->sobol.insert(t->sobol.end(), wd.sobol_m, wd.sobol_m + 32 * p.D);
    w.x0 = reinterpret_cast<const uint32_t *>((uintptr_t)t->sobol.size());
    if (p.D > 0) t->sobol.insert(t->sobol.end(), wd.sobol_x0, wd.sobol_x0 + p.D);
  }
  // all tiles of the launch heaviest first: the block scheduler starts the long CTAs early
  std::vector<size_t> ord(t->cta_map.size());
  for (size_t k = 0; k < ord.size(); ++k) ord[k] = k;
  std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return t->cta_cost[a] > t->cta_cost[b]; });
  std::vector<int4> sorted(ord.size());
  for (size_t k = 0; k < ord.size(); ++k) sorted[k] = t->cta_map[ord[k]];
  t->cta_map.swap(sorted);
  if (!c->real_phase_problem || (need_P && !c->real_phase_P))
    return c->fail(QIW_ERR_UNSUPPORTED, "qiw_integrate: inputs are not real-phase (i*P, i*Delta and operator "
                                        "blocks must be real); only the real-phase kernels are built");
  if (need_P && !c->has_P) return c->fail(QIW_ERR_ARG, "qiw_integrate: bold group but qiw_ppgf_set was not called");
  if (t->res_max > kResLarge) return c->fail(QIW_ERR_UNSUPPORTED, "qiw_integrate: sum of d_s^2 above 512");
  return QIW_OK;
}

int sync_groups(qiw_ctx *c) {
  if (!c->groups_dirty) return QIW_OK;
  std::vector<DevGroup> dgs;
  for (auto *g : c->groups) dgs.push_back(g->dg);
  int rc = c->cuda(c->d_groups.upload(dgs.data(), dgs.size(), c->stream), "upload groups");
  if (rc) return rc;
  for (int L = 1; L <= kSplitLevels; ++L) {
    dgs.clear();
    for (auto *g : c->groups) dgs.push_back(g->level(L).dg);
    if ((rc = c->cuda(c->d_groups_split[L - 1].upload(dgs.data(), dgs.size(), c->stream), "upload groups")))
      return rc;
  }
  c->groups_dirty = false;
  return QIW_OK;
}

// Launches the evaluation and finish kernels on tables already placed in device memory.
int launch_tables(qiw_ctx *c, const LaunchTables &t, int32_t precision, const DevGroup *groups, const DevWork *works,
                  const int4 *cta_map, const int *cta_first, const int *res_sizes, const int *out_off,
                  double *partials, int *err, double *out) {
  const int n_cta = (int)t.cta_map.size();
  LaunchArgs la;
  la.pb = c->dev_problem(precision != QIW_PREC_FP64);
  la.groups = groups;
  la.works = works;
  la.cta_map = cta_map;
  la.partials = partials;
  la.n_cta = n_cta;
  la.threads = precision == QIW_PREC_FP64 ? c->threads : c->threads32;
  la.extra_smem = c->eval_extra_smem;
  la.carveout = c->eval_carveout;
  la.arena_max = t.arena_max;
  la.res_max = t.res_max;
  la.fp32 = precision != QIW_PREC_FP64;
  la.tc_omul = precision == QIW_PREC_FP32_TC;
  // FP32 launches of many waves are throughput-bound: kernels with more resident blocks (eg at
  // 4096 samples 39.4 -> 34.1 ms, t2g 196.0 -> 186.8 ms); launches of few waves are bound by a
  // thread's path and keep the 5-block kernels (the denser ones were 2-3 % slower there)
  la.dense = la.fp32 && t.level == 0 && t.waves >= 4.0;
  if (const char *e = std::getenv("QIW_DENSE")) la.dense = la.fp32 && std::atoi(e) != 0;
  la.extras = false;
  la.stage = false;
  for (const DevWork &w : t.works) {
    la.extras = la.extras || w.pts != nullptr || w.sample_out != nullptr || w.transform != QIW_TRANSFORM_DEFAULT;
    la.stage = la.stage || c->groups[w.group]->dg.scalar != 0;
  }
  la.stream = c->stream;
  FinishArgs fa;
  fa.works = works;
  fa.cta_first = cta_first;
  fa.partials = partials;
  fa.res_sizes = res_sizes;
  fa.out_off = out_off;
  fa.out = out;
  fa.err_word = err;
  fa.n_work = (int)t.works.size();
  fa.stream = c->stream;
  int rc;
  if ((rc = c->cuda(cudaEventRecord(c->ev0, c->stream), "event")) ||
      (n_cta > 0 && (rc = c->cuda(launch_eval(la), "eval kernel launch"))) ||
      (rc = c->cuda(launch_finish(fa), "finish kernel launch")) || (rc = c->cuda(cudaEventRecord(c->ev1, c->stream), "event")))
    return rc;
  return QIW_OK;
}

}  // namespace qiw

namespace qiw {

// Process-wide store of host plans by plan_key + planner budget.  Plans are immutable once
// stored and hold no times or tables, so every context and batch of the process shares them:
// repeated solves on one operator structure (new Delta, beta or grid) plan each group once.
constexpr int64_t kPlanCacheBytes = (int64_t)1 << 31;

struct PlanStore {
  std::mutex m;
  std::unordered_map<std::string, std::shared_ptr<const Plan>> map;
  int64_t bytes = 0, hits = 0;
};

PlanStore &plan_store() {
  static PlanStore store;
  return store;
}

std::shared_ptr<const Plan> plan_store_find(const std::string &key) {
  PlanStore &ps = plan_store();
  std::lock_guard<std::mutex> lock(ps.m);
  auto it = ps.map.find(key);
  if (it == ps.map.end()) return nullptr;
  ps.hits++;
  return it->second;
}

void plan_store_insert(std::string &&key, const Plan &p) {
  const int64_t bytes = (int64_t)(p.ins.size() * sizeof(Instr) + p.pm.size() * sizeof(PmJob) +
                                  p.wj.size() * sizeof(WJob) + key.size());
  auto sp = std::make_shared<const Plan>(p);
  PlanStore &ps = plan_store();
  std::lock_guard<std::mutex> lock(ps.m);
  if (ps.bytes + bytes > kPlanCacheBytes) {
    ps.map.clear();
    ps.bytes = 0;
  }
  if (ps.map.emplace(std::move(key), std::move(sp)).second) ps.bytes += bytes;
}

// Plans a group on c's problem (or takes the plan from c's cache), uploads its program and
// fills its device descriptor.  max_instrs > 0: batches split to at most that many instructions.
static int build_program(qiw_ctx *c, const GroupSpec &gs, int64_t max_instrs, GroupRec **out) {
  PlanOptions opt;
  opt.arena_budget = kArenaLarge;
  if (const char *b = std::getenv("QIW_ARENA_BUDGET")) opt.arena_budget = std::max<int64_t>(256, std::atoll(b));
  opt.arena_budget = std::min<int64_t>(opt.arena_budget, kArenaLarge);
  // tuning: split batches whose per-sample work exceeds this many flops (a thread runs a batch
  // serially, so the heaviest batch bounds a launch's duration from below)
  if (const char *m = std::getenv("QIW_MAX_BATCH_FLOPS")) opt.max_batch_flops = std::max(0.0, std::atof(m));
  if (const char *m = std::getenv("QIW_MAX_BATCH_INSTRS")) opt.max_batch_instrs = std::max<int64_t>(0, std::atoll(m));
  if (max_instrs > 0) opt.max_batch_instrs = max_instrs;
  std::string key = plan_key(c->hp, gs);
  key.append(reinterpret_cast<const char *>(&opt.arena_budget), sizeof(opt.arena_budget));
  key.append(reinterpret_cast<const char *>(&opt.max_batch_flops), sizeof(opt.max_batch_flops));
  key.append(reinterpret_cast<const char *>(&opt.max_batch_instrs), sizeof(opt.max_batch_instrs));
  GroupRec *g = new GroupRec();
  if (std::shared_ptr<const Plan> hit = plan_store_find(key)) {
    g->plan = *hit;
  } else {
    std::string e;
    int rc = plan_group(c->hp, gs, opt, &g->plan, &e);
    if (rc == QIW_ERR_MEMORY && opt.arena_budget == kArenaLarge) {
      // large sector blocks: one (topology, sector) tree needs more than the large arena
      opt.arena_budget = kArenaHuge;
      e.clear();
      g->plan = Plan();
      rc = plan_group(c->hp, gs, opt, &g->plan, &e);
    }
    if (rc) {
      delete g;
      return c->fail(rc, "qiw_group_create: " + e);
    }
    if (arena_class(g->plan.arena) < 0) {
      delete g;
      return c->fail(QIW_ERR_MEMORY, "qiw_group_create: per-sample arena above the largest kernel instantiation");
    }
    // flag bits: 0 = (c != 1), 1 = (c == -1); bits 2-4 come from the planner
    for (Instr &I : g->plan.ins)
      I.flags = (uint8_t)((I.flags & ~3u) | (I.c != 1.0 ? 1 : 0) | (I.c == -1.0 ? 2 : 0));
    plan_store_insert(std::move(key), g->plan);
  }
  // the FP32 copy holds c rounded to float in the low 4 bytes of c; each copy carries the flat
  // dispatch index of the kernels that run it (FP32: P products held in registers)
  std::vector<Instr> ins32(g->plan.ins);
  for (Instr &I : ins32) {
    const float f = (float)I.c;
    uint64_t bits = 0;
    std::memcpy(&bits, &f, sizeof(f));
    std::memcpy(&I.c, &bits, sizeof(bits));
    I.handler = QIW_FLAT_DISPATCH ? handler_of(I, QIW_REG_PRODUCTS) : 0;
  }
  for (Instr &I : g->plan.ins) I.handler = QIW_FLAT_DISPATCH ? handler_of(I, QIW_REG_PRODUCTS && QIW_REG_PRODUCTS_FP64) : 0;
  const Plan &p = g->plan;
  int rc;
  if ((rc = c->cuda(g->pm.upload(p.pm.data(), p.pm.size(), c->stream), "upload plan")) ||
      (rc = c->cuda(g->wj.upload(p.wj.data(), p.wj.size(), c->stream), "upload plan")) ||
      (rc = c->cuda(g->ins.upload(p.ins.data(), p.ins.size(), c->stream), "upload plan")) ||
      (rc = c->cuda(g->ins32.upload(ins32.data(), ins32.size(), c->stream), "upload plan")) ||
      (rc = c->cuda(g->batch.upload(p.batch_begin.data(), p.batch_begin.size(), c->stream), "upload plan")) ||
      (rc = c->cuda(cudaStreamSynchronize(c->stream), "upload plan"))) {
    g->release();
    delete g;
    return rc;
  }
  DevGroup &dg = g->dg;
  std::memset(&dg, 0, sizeof(dg));
  dg.kind = p.kind;
  dg.order = p.order;
  dg.n_nodes = p.n_nodes;
  dg.D = p.D;
  dg.d_before = p.d_before;
  dg.d_after = p.d_after;
  dg.use_bold = p.use_bold;
  dg.n_fixed = p.n_fixed;
  for (int f = 0; f < p.n_fixed; ++f) {
    dg.fixed_pos[f] = p.fixed_pos[f];
    dg.fixed_time[f] = p.fixed_time[f];
  }
  for (size_t j = 0; j < p.var_pos.size(); ++j) dg.var_pos[j] = p.var_pos[j];
  dg.n_pm = (int)p.pm.size();
  dg.n_w = (int)p.wj.size();
  dg.n_instr = (int)p.ins.size();
  dg.arena = (int)p.arena;
  dg.res_size = p.res_size;
  dg.n_batches = (int)p.batch_begin.size() - 1;
  dg.scalar = 1;
  for (const Instr &I : p.ins)
    if (I.rows > 1 || I.cols > 1 || I.inner > 1) dg.scalar = 0;
  dg.pm = g->pm.p;
  dg.wj = g->wj.p;
  dg.ins = g->ins.p;
  dg.ins32 = g->ins32.p;
  dg.batch_begin = g->batch.p;
  *out = g;
  return QIW_OK;
}

int build_group(qiw_ctx *c, const GroupSpec &gs, GroupRec **out, bool with_splits) {
  GroupRec *g = nullptr;
  int rc = build_program(c, gs, 0, &g);
  if (rc) return rc;
  // split-batch programs for FP32 launches of few waves: groups with small blocks (not the
  // large-block or all-scalar programs) whose longest batch is above a level's instruction cap
  if (with_splits && !g->dg.scalar && g->plan.arena <= kArenaLarge) {
    int64_t longest = 0;
    for (size_t b = 0; b + 1 < g->plan.batch_begin.size(); ++b)
      longest = std::max<int64_t>(longest, g->plan.batch_begin[b + 1] - g->plan.batch_begin[b]);
    for (int L = 0; L < kSplitLevels; ++L) {
      if (longest <= kSplitInstrs[L]) continue;
      GroupRec *sp = nullptr;
      if (build_program(c, gs, kSplitInstrs[L], &sp) == QIW_OK) {
        g->split[L] = sp;
      } else {
        c->err.clear();   // no split program for this level: launches use the plain one
      }
    }
  }
  *out = g;
  return QIW_OK;
}

}  // namespace qiw

extern "C" {

int qiw_ctx_create(qiw_ctx **out, int device) {
  if (!out) return QIW_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return QIW_ERR_CUDA;
  qiw_ctx *c = new qiw_ctx();
  c->device = device;
  if (cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) c->n_sm = 0;
  qiw::DeviceScope dev_scope(device);
  if (dev_scope.status != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
    delete c;
    return QIW_ERR_CUDA;
  }
  if (const char *t = std::getenv("QIW_THREADS")) {
    int v = std::atoi(t);
    if (v == 32 || v == 64 || v == 96 || v == 128) c->threads = c->threads32 = v;
  }
  if (const char *t = std::getenv("QIW_EVAL_EXTRA_SMEM")) c->eval_extra_smem = std::max(0, std::min(160 << 10, std::atoi(t)));
  if (const char *t = std::getenv("QIW_EVAL_CARVEOUT")) c->eval_carveout = std::max(-1, std::min(100, std::atoi(t)));
  *out = c;
  return QIW_OK;
}

void qiw_ctx_destroy(qiw_ctx *c) {
  if (!c) return;
  qiw::DeviceScope dev_scope(c->device);
  cudaStreamSynchronize(c->stream);
  for (cudaStream_t s : c->aux) cudaStreamSynchronize(s);
  c->clear_groups();
  destroy_warps(c);
  c->d_groups.release();
  for (auto &d : c->d_groups_split) d.release();
  c->d_pts.release();
  c->d_samples.release();
  c->d_norms.release();
  for (auto *b : {&c->d_dims, &c->d_ptab_off, &c->d_eoff, &c->d_res_off, &c->d_delta_kind, &c->d_delta_off,
                  &c->d_cta_first, &c->d_res_sizes, &c->d_out_off, &c->d_err})
    b->release();
  for (auto *b : {&c->d_E, &c->d_P, &c->d_opv, &c->d_delta, &c->d_partials, &c->d_out}) b->release();
  for (auto *b : {&c->d_Pf, &c->d_opvf, &c->d_deltaf}) b->release();
  c->d_works.release();
  c->d_cta_map.release();
  c->d_sobol.release();
  for (cudaStream_t s : c->aux) cudaStreamDestroy(s);
  for (cudaEvent_t e : c->aux_ev) cudaEventDestroy(e);
  cudaEventDestroy(c->ev0);
  cudaEventDestroy(c->ev1);
  cudaStreamDestroy(c->stream);
  delete c;
}

const char *qiw_last_error(const qiw_ctx *c) { return c ? c->err.c_str() : "null context"; }

double qiw_last_kernel_ms(const qiw_ctx *c) { return c ? c->last_ms : 0.0; }

int qiw_problem_set(qiw_ctx *c, const qiw_problem_desc *d) {
  if (!c || !d) return QIW_ERR_ARG;
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_problem_set: cudaSetDevice");
  if (d->n_sectors <= 0 || !d->sector_dims || d->n_tau < 2 || !(d->beta > 0.0) || d->n_ops <= 0 ||
      !d->op_n_blocks || !d->op_blocks || !d->op_value_offset || !d->op_values || d->n_pairs < 0 ||
      (d->n_pairs > 0 && (!d->pair_ops || !d->pair_prop_kind || !d->pair_prop_data)) || !d->atomic_energies)
    return c->fail(QIW_ERR_ARG, "qiw_problem_set: missing or invalid field");
  c->clear_groups();
  HostProblem &hp = c->hp;
  std::string e;
  int prc = host_problem_from_desc(d, &hp, &e);
  if (prc) return c->fail(prc, "qiw_problem_set: " + e);
  const int64_t max_val = (int64_t)hp.op_vals.size();
  c->real_phase_problem = true;
  std::vector<double> opv(max_val), E;
  std::vector<float> opvf(max_val);
  for (int64_t i = 0; i < max_val; ++i) {
    if (hp.op_vals[i].imag() != 0.0) c->real_phase_problem = false;
    opv[i] = hp.op_vals[i].real();
    opvf[i] = (float)opv[i];
  }
  c->n_tau = d->n_tau;
  c->beta = d->beta;
  c->h = d->beta / (double)(d->n_tau - 1);
  c->delta_kind.resize(hp.n_pairs);
  c->delta_off.resize(hp.n_pairs);
  std::vector<double> delta;
  for (int p = 0; p < hp.n_pairs; ++p) {
    int kind = d->pair_prop_kind[p];
    if (kind != QIW_PROP_LINEAR && kind != QIW_PROP_CUBIC) return c->fail(QIW_ERR_ARG, "qiw_problem_set: unknown propagator kind");
    std::vector<double> y(c->n_tau);
    for (int j = 0; j < c->n_tau; ++j) {
      const double re = d->pair_prop_data[2 * ((size_t)p * c->n_tau + j)];
      const double im = d->pair_prop_data[2 * ((size_t)p * c->n_tau + j) + 1];
      if (re != 0.0) c->real_phase_problem = false;
      y[j] = -im;  // i * Delta
    }
    c->delta_kind[p] = kind;
    c->delta_off[p] = (int)delta.size();
    if (kind == QIW_PROP_LINEAR) delta.insert(delta.end(), y.begin(), y.end());
    else {
      std::vector<double> co;
      cubic_coeffs(y, c->h, &co);
      delta.insert(delta.end(), co.begin(), co.end());
    }
  }
  c->dims = hp.dims;
  c->eoff.resize(hp.S);
  c->ptab_off.resize(hp.S);
  c->res_off.resize(hp.S);
  int eo = 0, ro = 0;
  int64_t po = 0;
  for (int s = 0; s < hp.S; ++s) {
    c->eoff[s] = eo;
    eo += hp.dims[s];
    c->res_off[s] = ro;
    ro += hp.dims[s] * hp.dims[s];
    c->ptab_off[s] = (int)po;
    po += (int64_t)c->n_tau * hp.dims[s] * hp.dims[s];
  }
  c->ptab_size = po;
  c->res_total = ro;
  E.assign(d->atomic_energies, d->atomic_energies + eo);
  std::vector<float> deltaf(delta.begin(), delta.end());
  cudaStream_t st = c->stream;
  int rc;
  if ((rc = c->cuda(c->d_dims.upload(hp.dims.data(), hp.S, st), "upload dims")) ||
      (rc = c->cuda(c->d_ptab_off.upload(c->ptab_off.data(), hp.S, st), "upload ptab_off")) ||
      (rc = c->cuda(c->d_eoff.upload(c->eoff.data(), hp.S, st), "upload eoff")) ||
      (rc = c->cuda(c->d_res_off.upload(c->res_off.data(), hp.S, st), "upload res_off")) ||
      (rc = c->cuda(c->d_E.upload(E.data(), E.size(), st), "upload energies")) ||
      (rc = c->cuda(c->d_opv.upload(opv.data(), opv.size(), st), "upload operators")) ||
      (rc = c->cuda(c->d_opvf.upload(opvf.data(), opvf.size(), st), "upload operators")) ||
      (rc = c->cuda(c->d_delta.upload(delta.data(), delta.size(), st), "upload delta")) ||
      (rc = c->cuda(c->d_deltaf.upload(deltaf.data(), deltaf.size(), st), "upload delta")) ||
      (rc = c->cuda(c->d_delta_kind.upload(c->delta_kind.data(), c->delta_kind.size(), st), "upload delta kind")) ||
      (rc = c->cuda(c->d_delta_off.upload(c->delta_off.data(), c->delta_off.size(), st), "upload delta off")) ||
      (rc = c->cuda(c->d_P.reserve(po), "alloc P")) || (rc = c->cuda(c->d_Pf.reserve(po), "alloc P")) ||
      (rc = c->cuda(cudaStreamSynchronize(st), "problem upload")))
    return rc;
  c->has_problem = true;
  c->has_P = false;
  return QIW_OK;
}

int qiw_ppgf_set(qiw_ctx *c, const double *P) {
  if (!c || !P) return QIW_ERR_ARG;
  if (!c->has_problem) return c->fail(QIW_ERR_ARG, "qiw_ppgf_set: no problem set");
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_ppgf_set: cudaSetDevice");
  std::vector<double> t(c->ptab_size);
  std::vector<float> tf(c->ptab_size);
  c->real_phase_P = true;
  for (int64_t i = 0; i < c->ptab_size; ++i) {
    if (P[2 * i] != 0.0) c->real_phase_P = false;
    t[i] = -P[2 * i + 1];  // i * P
    tf[i] = (float)t[i];
  }
  int rc;
  if ((rc = c->cuda(c->d_P.upload(t.data(), t.size(), c->stream), "upload P")) ||
      (rc = c->cuda(c->d_Pf.upload(tf.data(), tf.size(), c->stream), "upload P")) ||
      (rc = c->cuda(cudaStreamSynchronize(c->stream), "upload P")))
    return rc;
  c->has_P = true;
  return QIW_OK;
}

int qiw_group_create(qiw_ctx *c, const qiw_group_desc *d, int32_t *group_id) {
  if (!c || !d || !group_id) return QIW_ERR_ARG;
  if (!c->has_problem) return c->fail(QIW_ERR_ARG, "qiw_group_create: no problem set");
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_group_create: cudaSetDevice");
  GroupSpec gs;
  {
    std::string e;
    int grc = group_spec_from_desc(d, &gs, &e);
    if (grc) return c->fail(grc, "qiw_group_create: " + e);
  }
  GroupRec *g = nullptr;
  int rc = build_group(c, gs, &g, true);
  if (rc) return rc;
  c->groups.push_back(g);
  c->groups_dirty = true;
  *group_id = (int32_t)c->groups.size() - 1;
  return QIW_OK;
}

int qiw_plan_cache_info(int64_t *entries, int64_t *hits, int64_t *bytes) {
  PlanStore &ps = plan_store();
  std::lock_guard<std::mutex> lock(ps.m);
  if (entries) *entries = (int64_t)ps.map.size();
  if (hits) *hits = ps.hits;
  if (bytes) *bytes = ps.bytes;
  return QIW_OK;
}

int qiw_plan_cache_clear(void) {
  PlanStore &ps = plan_store();
  std::lock_guard<std::mutex> lock(ps.m);
  ps.map.clear();
  ps.bytes = 0;
  return QIW_OK;
}

int qiw_group_stats_get(qiw_ctx *c, int32_t gid, qiw_group_stats *out) {
  if (!c || !out || gid < 0 || gid >= (int)c->groups.size()) return QIW_ERR_ARG;
  const Plan &p = c->groups[gid]->plan;
  out->n_nodes_dag = p.dag_nodes;
  out->n_instructions = (int64_t)p.ins.size();
  out->arena_elements = p.arena;
  out->flops_per_sample = p.flops;
  out->tree_flops_per_sample = p.tree_flops;
  out->n_leaves_tree = p.tree_leaves;
  return QIW_OK;
}

int qiw_integrate(qiw_ctx *c, int32_t n_work, const qiw_work_desc *work, int32_t precision, double *out) {
  return integrate_impl(c, n_work, work, precision, out, nullptr, nullptr);
}

int qiw_integrate_warped(qiw_ctx *c, int32_t n_work, const qiw_work_desc *work, const int32_t *warp_ids,
                         int32_t precision, double *out) {
  return integrate_impl(c, n_work, work, precision, out, warp_ids, nullptr);
}

int qiw_integrate_samples(qiw_ctx *c, const qiw_work_desc *work, int32_t precision, double *out, double *samples) {
  if (!c || !work || !samples) return QIW_ERR_ARG;
  return integrate_impl(c, 1, work, precision, out, nullptr, samples);
}

int qiw_integrate_samples_batch(qiw_ctx *c, int32_t n_work, const qiw_work_desc *work, int32_t precision,
                                double *out, double *samples) {
  if (!c || n_work < 0 || (n_work > 0 && (!work || !out || !samples))) return QIW_ERR_ARG;
  return integrate_impl(c, n_work, work, precision, out, nullptr, samples);
}

int qiw_integrate_sample_norms(qiw_ctx *c, int32_t n_work, const qiw_work_desc *work, int32_t precision,
                               double *out, double *norms) {
  if (!c || n_work < 0 || (n_work > 0 && (!work || !out || !norms))) return QIW_ERR_ARG;
  return integrate_impl(c, n_work, work, precision, out, nullptr, nullptr, norms);
}

int qiw_sobol_points(qiw_ctx *c, int32_t D, const uint32_t *m, const uint32_t *x0, uint64_t first, uint64_t n,
                     uint32_t *out) {
  if (!c || !m || !x0 || (n > 0 && !out)) return QIW_ERR_ARG;
  if (D < 1 || D > kMaxDim) return c->fail(QIW_ERR_ARG, "qiw_sobol_points: D must lie in 1..32");
  if (first > (1ull << 32) || n > (1ull << 32) - first)
    return c->fail(QIW_ERR_ARG, "qiw_sobol_points: points beyond index 2^32 - 1 (32 direction numbers)");
  if (n > (1ull << 26)) return c->fail(QIW_ERR_ARG, "qiw_sobol_points: at most 2^26 points per call");
  if (n == 0) return QIW_OK;
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_sobol_points: cudaSetDevice");
  DevBuf<uint32_t> dm, dx, dout;
  int rc;
  if ((rc = c->cuda(dm.upload(m, (size_t)D * 32, c->stream), "qiw_sobol_points: upload")) ||
      (rc = c->cuda(dx.upload(x0, (size_t)D, c->stream), "qiw_sobol_points: upload")) ||
      (rc = c->cuda(dout.reserve((size_t)n * D), "qiw_sobol_points: alloc")) ||
      (rc = c->cuda(launch_sobol_points(dm.p, dx.p, D, first, n, dout.p, c->stream), "qiw_sobol_points: launch")) ||
      (rc = c->cuda(cudaMemcpyAsync(out, dout.p, sizeof(uint32_t) * n * D, cudaMemcpyDeviceToHost, c->stream),
                    "qiw_sobol_points: download")) ||
      (rc = c->cuda(cudaStreamSynchronize(c->stream), "qiw_sobol_points"))) {
    cudaStreamSynchronize(c->stream);
    dm.release(); dx.release(); dout.release();
    return rc;
  }
  dm.release();
  dx.release();
  dout.release();
  return QIW_OK;
}

int qiw_measure_fma_peak(qiw_ctx *c, int32_t precision, double *tflops) {
  if (!c || !tflops) return QIW_ERR_ARG;
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_measure_fma_peak: cudaSetDevice");
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  const int threads = 256, blocks = sms * 8, iters = 2048;
  DevBuf<double> out;
  int rc;
  if ((rc = c->cuda(out.reserve((size_t)blocks * threads), "alloc"))) return rc;
  const bool fp32 = precision != QIW_PREC_FP64;
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {
    if ((rc = c->cuda(cudaEventRecord(c->ev0, c->stream), "event")) ||
        (rc = c->cuda(launch_fma_peak(fp32, out.p, blocks, threads, iters, c->stream), "fma peak")) ||
        (rc = c->cuda(cudaEventRecord(c->ev1, c->stream), "event")) ||
        (rc = c->cuda(cudaEventSynchronize(c->ev1), "fma peak"))) {
      out.release();
      return rc;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
    if (rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  out.release();
  *tflops = best;
  return QIW_OK;
}

}  // extern "C"
