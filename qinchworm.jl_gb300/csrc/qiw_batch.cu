// Batched independent solves: many whole inchworm! loops in one launch queue per step.
//
// Each solve keeps its own problem tables and P table in device memory (a qiw_ctx of its
// own, set up through the regular qiw_problem_set / qiw_ppgf_set).  Group programs are
// planned once per distinct (operator structure, topology group) and shared by every solve
// with that structure -- the Anderson solves of a parameter sweep differ only in energies,
// hybridisation tables and grids, which the programs do not contain.
//
// Per step s the device runs three launches: the persistent evaluation kernel over the tiles
// of every (solve, group) still running, one CTA per work item to finish its qMC sum, and one
// CTA per solve to write i*P(tau_{s+1}) and normalise (src/inchworm.jl:474-493,
// src/ppgf.jl:474-504, 646-654).  The whole loop can be captured once as a CUDA graph.
// Tiles of all solves are ordered heaviest first; CTAs take them with an atomic ticket.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "qiw_ctx.hpp"

using namespace qiw;

namespace {

struct PlanEntry {
  std::string key;
  GroupRec *rec = nullptr;
  int n_tops = 0;
};

struct SolveRec {
  qiw_ctx *ctx = nullptr;
  std::vector<int> bare, bold;   // indices into the plan table
  uint64_t N = 0;
  int n_steps = 0, n_tau = 0;
  std::vector<double> taus;
  DevBuf<double> d_taus, d_P0, d_lam;
};

// Tile lists of one step kind (bare or bold) for a given tile size.
struct TileSet {
  std::vector<BatchWork> works;
  std::vector<int4> tiles;
  int slots = 0, res_total = 0;
};

}  // namespace

struct qiw_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  std::vector<PlanEntry> plans;
  std::vector<SolveRec *> solves;
  DevBuf<DevProblem> d_probs;
  DevBuf<BatchSolve> d_solves;
  DevBuf<DevGroup> d_groups;
  DevBuf<BatchWork> d_bare, d_bold;
  DevBuf<int4> d_tiles_bare, d_tiles_bold;
  DevBuf<double> d_partials, d_res;
  DevBuf<int> d_err, d_ticket;
  DevBuf<uint32_t> d_sobol, d_zero;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int tuned_threads = 0, tuned_persistent = 1;
  int tuned_precision = -1;
  qiw_batch_stats st{};

  int fail(int code, const std::string &m) {
    err = m;
    return code;
  }
  int cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return QIW_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return QIW_ERR_CUDA;
  }
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
};

namespace {

// Work items and tiles of one step kind.  Within a work item the batches go heaviest first
// and the partial slots follow that order (the finish kernel sums them in it); the tile list
// of all work items is then sorted by estimated cost, heaviest first.
TileSet build_tiles(const qiw_batch *b, bool bare, int threads, const uint32_t *sobol, const uint32_t *zero) {
  TileSet ts;
  struct Cost {
    double c;
    size_t i;
  };
  std::vector<Cost> cost;
  for (size_t si = 0; si < b->solves.size(); ++si) {
    const SolveRec *s = b->solves[si];
    const std::vector<int> &gl = bare ? s->bare : s->bold;
    for (int pi : gl) {
      const Plan &p = b->plans[pi].rec->plan;
      BatchWork w;
      std::memset(&w, 0, sizeof(w));
      w.group = pi;
      w.solve = (int)si;
      w.order = p.order;
      w.last_step = bare ? 0 : s->n_steps;
      w.n_samples = p.D > 0 ? s->N : 1;
      w.inv_n = 1.0 / (double)w.n_samples;
      w.m = sobol;
      w.x0 = zero;
      w.res_off = ts.res_total;
      ts.res_total += p.res_size;
      w.slot0 = ts.slots;
      const int n_t = (int)((w.n_samples + threads - 1) / threads);
      const int n_b = std::max(0, (int)p.batch_begin.size() - 1);
      std::vector<int> order(n_b);
      for (int k = 0; k < n_b; ++k) order[k] = k;
      std::stable_sort(order.begin(), order.end(),
                       [&](int x, int y) { return p.batch_flops[x] > p.batch_flops[y]; });
      int slot = ts.slots;
      for (int bb : order)
        for (int k = 0; k < n_t; ++k) {
          const uint64_t s0 = (uint64_t)k * threads;
          const double n_in = (double)std::min<uint64_t>((uint64_t)threads, w.n_samples - s0);
          cost.push_back({p.batch_flops[bb] * n_in * (double)(bare ? 1 : std::max(1, s->n_steps)), ts.tiles.size()});
          ts.tiles.push_back(make_int4((int)ts.works.size(), bb, (int)s0, slot++));
        }
      w.n_slots = slot - ts.slots;
      ts.slots = slot;
      ts.works.push_back(w);
    }
  }
  std::stable_sort(cost.begin(), cost.end(), [](const Cost &x, const Cost &y) { return x.c > y.c; });
  std::vector<int4> sorted(ts.tiles.size());
  for (size_t i = 0; i < cost.size(); ++i) sorted[i] = ts.tiles[cost[i].i];
  ts.tiles.swap(sorted);
  return ts;
}

struct RunCfg {
  int threads = 64;
  bool persistent = true;
};

struct Prepared {
  TileSet bare, bold;
  int64_t arena_max = 0;
  int res_max = 0, pstride = 0, max_steps = 0;
  int grid_bare = 0, grid_bold = 0;
  bool stage = false;
};

int prepare(qiw_batch *b, int precision, const RunCfg &cfg, Prepared *pp) {
  Prepared &P = *pp;
  P.bare = build_tiles(b, true, cfg.threads, b->d_sobol.p, b->d_zero.p);
  P.bold = build_tiles(b, false, cfg.threads, b->d_sobol.p, b->d_zero.p);
  for (const PlanEntry &e : b->plans) {
    P.arena_max = std::max<int64_t>(P.arena_max, e.rec->plan.arena);
    P.res_max = std::max(P.res_max, e.rec->plan.res_size);
  }
  P.pstride = std::max(1, P.res_max);
  P.stage = false;
  for (const PlanEntry &e : b->plans) P.stage = P.stage || e.rec->dg.scalar != 0;
  for (const SolveRec *s : b->solves) P.max_steps = std::max(P.max_steps, s->n_steps);
  const size_t slots = (size_t)std::max(P.bare.slots, P.bold.slots);
  const size_t res = (size_t)std::max(P.bare.res_total, P.bold.res_total);
  int rc;
  if ((rc = b->cuda(b->d_bare.upload(P.bare.works.data(), P.bare.works.size(), b->stream), "upload works")) ||
      (rc = b->cuda(b->d_bold.upload(P.bold.works.data(), P.bold.works.size(), b->stream), "upload works")) ||
      (rc = b->cuda(b->d_tiles_bare.upload(P.bare.tiles.data(), P.bare.tiles.size(), b->stream), "upload tiles")) ||
      (rc = b->cuda(b->d_tiles_bold.upload(P.bold.tiles.data(), P.bold.tiles.size(), b->stream), "upload tiles")) ||
      (rc = b->cuda(b->d_partials.reserve(slots * P.pstride), "alloc partials")) ||
      (rc = b->cuda(b->d_res.reserve(std::max<size_t>(res, 1)), "alloc results")) ||
      (rc = b->cuda(b->d_ticket.reserve((size_t)P.max_steps + 2), "alloc tickets")))
    return rc;
  // grid: resident CTAs (persistent) or one CTA per tile
  BatchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.threads = cfg.threads;
  a.arena_max = P.arena_max;
  a.res_max = P.res_max;
  a.fp32 = precision == QIW_PREC_FP32;
  a.stage = P.stage;
  int occ = 0;
  if (batch_occupancy(a, &occ)) return b->fail(QIW_ERR_CUDA, "qiw_batch_run: occupancy query failed");
  int n_sm = 0;
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, b->device);
  const int resident = std::max(1, occ * n_sm);
  auto grid_of = [&](size_t n_tiles) {
    if (n_tiles == 0) return 0;
    return cfg.persistent ? (int)std::min<size_t>(n_tiles, (size_t)resident) : (int)n_tiles;
  };
  P.grid_bare = grid_of(P.bare.tiles.size());
  P.grid_bold = grid_of(P.bold.tiles.size());
  return QIW_OK;
}

BatchArgs step_args(qiw_batch *b, const Prepared &P, int precision, int threads, int step) {
  BatchArgs a;
  std::memset(&a, 0, sizeof(a));
  const bool bare = step == 0;
  a.probs = b->d_probs.p + (precision == QIW_PREC_FP32 ? b->solves.size() : 0);
  a.solves = b->d_solves.p;
  a.groups = b->d_groups.p;
  a.works = bare ? b->d_bare.p : b->d_bold.p;
  a.tiles = bare ? b->d_tiles_bare.p : b->d_tiles_bold.p;
  a.n_tiles = (int)(bare ? P.bare.tiles.size() : P.bold.tiles.size());
  a.n_works = (int)(bare ? P.bare.works.size() : P.bold.works.size());
  a.n_solves = (int)b->solves.size();
  a.ticket = b->d_ticket.p + step;
  a.partials = b->d_partials.p;
  a.pstride = P.pstride;
  a.res = b->d_res.p;
  a.err_word = b->d_err.p;
  a.step = step;
  a.grid = bare ? P.grid_bare : P.grid_bold;
  a.threads = threads;
  a.arena_max = P.arena_max;
  a.res_max = P.res_max;
  a.fp32 = precision == QIW_PREC_FP32;
  a.stage = P.stage;
  a.stream = b->stream;
  return a;
}

// The launches of a whole run (reset, then every step).
int enqueue_run(qiw_batch *b, const Prepared &P, int precision, int threads) {
  int rc;
  if ((rc = b->cuda(cudaMemsetAsync(b->d_ticket.p, 0, sizeof(int) * ((size_t)P.max_steps + 2), b->stream), "ticket")))
    return rc;
  BatchArgs a0 = step_args(b, P, precision, threads, 0);
  if ((rc = b->cuda(launch_batch_reset(a0), "reset kernel"))) return rc;
  for (int step = 0; step <= P.max_steps; ++step) {
    BatchArgs a = step_args(b, P, precision, threads, step);
    if (a.n_works == 0) continue;
    if (a.n_tiles > 0 && (rc = b->cuda(launch_batch_eval(a), "batch eval kernel"))) return rc;
    if ((rc = b->cuda(launch_batch_finish(a), "batch finish kernel")) ||
        (rc = b->cuda(launch_batch_update(a), "batch update kernel")))
      return rc;
  }
  return QIW_OK;
}

// Autotuner: device time of one bold step (step 1: every solve is still running) for each
// tile size x grid mode; the fastest is kept for the batch.
int autotune(qiw_batch *b, int precision) {
  const int cand_threads[3] = {32, 64, 128};
  double best = 1e300;
  int rc;
  for (int ti = 0; ti < 3; ++ti)
    for (int pm = 0; pm < 2; ++pm) {
      RunCfg cfg;
      cfg.threads = cand_threads[ti];
      cfg.persistent = pm == 0;
      Prepared P;
      if ((rc = prepare(b, precision, cfg, &P))) return rc;
      if (P.max_steps < 1 || P.bold.tiles.empty()) {
        b->tuned_threads = 64;
        b->tuned_persistent = 1;
        return QIW_OK;
      }
      double t_min = 1e300;
      for (int rep = 0; rep < 2; ++rep) {
        BatchArgs a = step_args(b, P, precision, cfg.threads, 1);
        float ms = 0.f;
        if ((rc = b->cuda(cudaMemsetAsync(a.ticket, 0, sizeof(int), b->stream), "ticket")) ||
            (rc = b->cuda(cudaEventRecord(b->ev0, b->stream), "event")) ||
            (rc = b->cuda(launch_batch_eval(a), "batch eval kernel")) ||
            (rc = b->cuda(cudaEventRecord(b->ev1, b->stream), "event")) ||
            (rc = b->cuda(cudaEventSynchronize(b->ev1), "autotune")) ||
            (rc = b->cuda(cudaEventElapsedTime(&ms, b->ev0, b->ev1), "event")))
          return rc;
        t_min = std::min(t_min, (double)ms);
      }
      b->st.tune_ms[ti * 2 + pm] = t_min;
      if (t_min < best) {
        best = t_min;
        b->tuned_threads = cfg.threads;
        b->tuned_persistent = cfg.persistent ? 1 : 0;
      }
    }
  return QIW_OK;
}

}  // namespace

extern "C" {

int qiw_batch_create(qiw_batch **out, int device) {
  if (!out) return QIW_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return QIW_ERR_CUDA;
  qiw_batch *b = new qiw_batch();
  b->device = device;
  qiw::DeviceScope dev_scope(device);
  if (dev_scope.status != cudaSuccess || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) {
    qiw_batch_destroy(b);
    return QIW_ERR_CUDA;
  }
  *out = b;
  return QIW_OK;
}

void qiw_batch_destroy(qiw_batch *b) {
  if (!b) return;
  qiw::DeviceScope dev_scope(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  b->drop_graph();
  for (SolveRec *s : b->solves) {
    s->d_taus.release();
    s->d_P0.release();
    s->d_lam.release();
    qiw_ctx_destroy(s->ctx);
    delete s;
  }
  for (PlanEntry &e : b->plans) {
    e.rec->release();
    delete e.rec;
  }
  b->d_probs.release();
  b->d_solves.release();
  b->d_groups.release();
  b->d_bare.release();
  b->d_bold.release();
  b->d_tiles_bare.release();
  b->d_tiles_bold.release();
  b->d_partials.release();
  b->d_res.release();
  b->d_err.release();
  b->d_ticket.release();
  b->d_sobol.release();
  b->d_zero.release();
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

const char *qiw_batch_last_error(const qiw_batch *b) { return b ? b->err.c_str() : "null batch"; }

int qiw_batch_add(qiw_batch *b, const qiw_solve_desc *d, int32_t *solve_id) {
  if (!b || !d || !solve_id || !d->problem || !d->taus || !d->P_init || d->n_bare < 0 || d->n_bold < 0 ||
      (d->n_bare > 0 && !d->bare) || (d->n_bold > 0 && !d->bold))
    return QIW_ERR_ARG;
  if (d->n_samples == 0 || (d->n_samples & (d->n_samples - 1)) || d->n_samples > (1ull << 32))
    return b->fail(QIW_ERR_ARG, "qiw_batch_add: n_samples must be a power of 2 <= 2^32");
  qiw::DeviceScope dev_scope(b->device);
  if (dev_scope.status != cudaSuccess) return b->fail(QIW_ERR_CUDA, std::string("qiw_batch_add: cudaSetDevice: ") + cudaGetErrorString(dev_scope.status));
  SolveRec *s = new SolveRec();
  int rc = qiw_ctx_create(&s->ctx, b->device);
  if (rc) {
    delete s;
    return b->fail(rc, "qiw_batch_add: context");
  }
  auto bail = [&](int code, const std::string &m) {
    qiw_ctx_destroy(s->ctx);
    s->d_taus.release();
    s->d_P0.release();
    s->d_lam.release();
    delete s;
    return b->fail(code, m);
  };
  if ((rc = qiw_problem_set(s->ctx, d->problem))) return bail(rc, std::string("qiw_batch_add: ") + s->ctx->err);
  if ((rc = qiw_ppgf_set(s->ctx, d->P_init))) return bail(rc, std::string("qiw_batch_add: ") + s->ctx->err);
  if (!s->ctx->real_phase_problem || !s->ctx->real_phase_P)
    return bail(QIW_ERR_UNSUPPORTED, "qiw_batch_add: inputs are not real-phase");
  if (s->ctx->res_total > kResLarge) return bail(QIW_ERR_UNSUPPORTED, "qiw_batch_add: sum of d_s^2 above 512");
  s->n_tau = s->ctx->n_tau;
  if (d->n_steps < 0 || d->n_steps > s->n_tau - 2) return bail(QIW_ERR_ARG, "qiw_batch_add: n_steps outside 0 .. n_tau - 2");
  s->n_steps = d->n_steps;
  s->N = d->n_samples;
  s->taus.assign(d->taus, d->taus + s->n_tau);
  for (int j = 1; j < s->n_tau; ++j)
    if (!(s->taus[j] > s->taus[j - 1])) return bail(QIW_ERR_ARG, "qiw_batch_add: taus must increase");
  // the initial table, kept for re-runs
  std::vector<double> p0(s->ctx->ptab_size);
  for (int64_t i = 0; i < s->ctx->ptab_size; ++i) p0[i] = -d->P_init[2 * i + 1];
  if ((rc = b->cuda(s->d_taus.upload(s->taus.data(), s->taus.size(), b->stream), "upload taus")) ||
      (rc = b->cuda(s->d_P0.upload(p0.data(), p0.size(), b->stream), "upload P0")) ||
      (rc = b->cuda(s->d_lam.reserve(s->n_tau), "alloc lambda")) ||
      (rc = b->cuda(cudaStreamSynchronize(b->stream), "upload")))
    return bail(rc, b->err);
  // group programs, shared through the plan cache
  for (int kind = 0; kind < 2; ++kind) {
    const int n = kind == 0 ? d->n_bare : d->n_bold;
    const qiw_group_desc *gd = kind == 0 ? d->bare : d->bold;
    int last_order = -1;
    for (int i = 0; i < n; ++i) {
      GroupSpec gs;
      std::string e;
      if ((rc = group_spec_from_desc(&gd[i], &gs, &e))) return bail(rc, "qiw_batch_add: " + e);
      if ((kind == 0) != (gs.kind == QIW_GROUP_BARE) || gs.kind == QIW_GROUP_CORRELATOR)
        return bail(QIW_ERR_ARG, "qiw_batch_add: bare list takes bare groups, bold list bold groups");
      if (kind == 1 && gs.order < last_order) return bail(QIW_ERR_ARG, "qiw_batch_add: bold groups must be by ascending order");
      last_order = gs.order;
      const std::string key = plan_key(s->ctx->hp, gs);
      int pi = -1;
      for (size_t k = 0; k < b->plans.size(); ++k)
        if (b->plans[k].key == key) {
          pi = (int)k;
          break;
        }
      if (pi < 0) {
        GroupRec *g = nullptr;
        if ((rc = build_group(s->ctx, gs, &g))) return bail(rc, std::string("qiw_batch_add: ") + s->ctx->err);
        b->plans.push_back({key, g, (int)gs.tops.size()});
        pi = (int)b->plans.size() - 1;
      }
      (kind == 0 ? s->bare : s->bold).push_back(pi);
    }
  }
  b->solves.push_back(s);
  b->tuned_threads = 0;  // the workload changed
  b->drop_graph();
  *solve_id = (int32_t)b->solves.size() - 1;
  return QIW_OK;
}

int qiw_batch_run(qiw_batch *b, int32_t precision, int32_t flags, const uint32_t *sobol_m, int32_t sobol_dims) {
  if (!b || !sobol_m || sobol_dims <= 0) return QIW_ERR_ARG;
  if (precision != QIW_PREC_FP64 && precision != QIW_PREC_FP32) return b->fail(QIW_ERR_ARG, "qiw_batch_run: precision");
  if (b->solves.empty()) return QIW_OK;
  qiw::DeviceScope dev_scope(b->device);
  if (dev_scope.status != cudaSuccess) return b->fail(QIW_ERR_CUDA, std::string("qiw_batch_run: cudaSetDevice: ") + cudaGetErrorString(dev_scope.status));
  int rc;
  for (const PlanEntry &e : b->plans)
    if (e.rec->plan.D > sobol_dims) return b->fail(QIW_ERR_ARG, "qiw_batch_run: Sobol table has too few dimensions");
  // problem views (FP64 then FP32), solves, groups, Sobol tables
  const size_t ns = b->solves.size();
  std::vector<DevProblem> probs(2 * ns);
  std::vector<BatchSolve> sol(ns);
  int bare_at = 0, bold_at = 0;
  for (size_t i = 0; i < ns; ++i) {
    SolveRec *s = b->solves[i];
    probs[i] = s->ctx->dev_problem(false);
    probs[ns + i] = s->ctx->dev_problem(true);
    BatchSolve &so = sol[i];
    std::memset(&so, 0, sizeof(so));
    so.taus = s->d_taus.p;
    so.P0 = s->d_P0.p;
    so.P = s->ctx->d_P.p;
    so.Pf = s->ctx->d_Pf.p;
    so.lam = s->d_lam.p;
    so.last_step = s->n_steps;
    so.bare0 = bare_at;
    so.bare1 = bare_at += (int)s->bare.size();
    so.bold0 = bold_at;
    so.bold1 = bold_at += (int)s->bold.size();
    so.res_size = s->ctx->res_total;
    so.ptab_size = (int)s->ctx->ptab_size;
    so.n_tau = s->n_tau;
  }
  std::vector<DevGroup> groups;
  for (const PlanEntry &e : b->plans) groups.push_back(e.rec->dg);
  std::vector<uint32_t> zero(sobol_dims, 0u);
  const int err0 = 0;
  if ((rc = b->cuda(b->d_probs.upload(probs.data(), probs.size(), b->stream), "upload problems")) ||
      (rc = b->cuda(b->d_solves.upload(sol.data(), sol.size(), b->stream), "upload solves")) ||
      (rc = b->cuda(b->d_groups.upload(groups.data(), groups.size(), b->stream), "upload groups")) ||
      (rc = b->cuda(b->d_sobol.upload(sobol_m, (size_t)sobol_dims * 32, b->stream), "upload Sobol")) ||
      (rc = b->cuda(b->d_zero.upload(zero.data(), zero.size(), b->stream), "upload Sobol")) ||
      (rc = b->cuda(b->d_err.upload(&err0, 1, b->stream), "upload error word")))
    return rc;
  b->drop_graph();
  std::memset(b->st.tune_ms, 0, sizeof(b->st.tune_ms));
  if ((flags & QIW_BATCH_AUTOTUNE) && (b->tuned_threads == 0 || b->tuned_precision != precision)) {
    if ((rc = autotune(b, precision))) return rc;
    b->tuned_precision = precision;
  }
  RunCfg cfg;
  if (b->tuned_threads) {
    cfg.threads = b->tuned_threads;
    cfg.persistent = b->tuned_persistent != 0;
  }
  Prepared P;
  if ((rc = prepare(b, precision, cfg, &P))) return rc;
  int nodes = 0;
  if (flags & QIW_BATCH_GRAPH) {
    if ((rc = b->cuda(cudaStreamSynchronize(b->stream), "sync")) ||
        (rc = b->cuda(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "graph capture")))
      return rc;
    rc = enqueue_run(b, P, precision, cfg.threads);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if ((rc = b->cuda(ec, "graph capture"))) return rc;
    b->graph = g;
    size_t nn = 0;
    cudaGraphGetNodes(g, nullptr, &nn);
    nodes = (int)nn;
    if ((rc = b->cuda(cudaGraphInstantiate(&b->exec, g, 0), "graph instantiate")) ||
        (rc = b->cuda(cudaGraphUpload(b->exec, b->stream), "graph upload")) ||
        (rc = b->cuda(cudaStreamSynchronize(b->stream), "sync")) ||
        (rc = b->cuda(cudaEventRecord(b->ev0, b->stream), "event")) ||
        (rc = b->cuda(cudaGraphLaunch(b->exec, b->stream), "graph launch")) ||
        (rc = b->cuda(cudaEventRecord(b->ev1, b->stream), "event")))
      return rc;
  } else {
    if ((rc = b->cuda(cudaEventRecord(b->ev0, b->stream), "event")) || (rc = enqueue_run(b, P, precision, cfg.threads)) ||
        (rc = b->cuda(cudaEventRecord(b->ev1, b->stream), "event")))
      return rc;
  }
  int errw = 0;
  float ms = 0.f;
  if ((rc = b->cuda(cudaEventSynchronize(b->ev1), "batch run")) ||
      (rc = b->cuda(cudaEventElapsedTime(&ms, b->ev0, b->ev1), "event")) ||
      (rc = b->cuda(cudaMemcpy(&errw, b->d_err.p, sizeof(int), cudaMemcpyDeviceToHost), "error word")))
    return rc;
  // statistics of the run
  double flops = 0.0, tsamp = 0.0;
  for (const SolveRec *s : b->solves) {
    for (int pi : s->bare) {
      const Plan &p = b->plans[pi].rec->plan;
      const double n = p.D > 0 ? (double)s->N : 1.0;
      flops += p.flops * n;
      tsamp += b->plans[pi].n_tops * n;
    }
    for (int pi : s->bold) {
      const Plan &p = b->plans[pi].rec->plan;
      const double n = (p.D > 0 ? (double)s->N : 1.0) * s->n_steps;
      flops += p.flops * n;
      tsamp += b->plans[pi].n_tops * n;
    }
  }
  b->st.kernel_ms = ms;
  b->st.flops = flops;
  b->st.topology_samples = tsamp;
  b->st.threads = cfg.threads;
  b->st.grid = P.grid_bold;
  b->st.persistent = cfg.persistent ? 1 : 0;
  b->st.n_steps_max = P.max_steps;
  b->st.graph_nodes = nodes;
  b->st.n_plans = (int)b->plans.size();
  b->st.n_tiles_bold = (int64_t)P.bold.tiles.size();
  b->st.n_tiles_bare = (int64_t)P.bare.tiles.size();
  if (errw & 2)
    return b->fail(QIW_ERR_DEVICE, "qiw_batch_run: normalize!: the largest diagonal of P is not positive (no log)");
  if (errw) return b->fail(QIW_ERR_DEVICE, "qiw_batch_run: non-finite result");
  return QIW_OK;
}

int qiw_batch_get_P(qiw_batch *b, int32_t id, double *P) {
  if (!b || !P || id < 0 || id >= (int)b->solves.size()) return QIW_ERR_ARG;
  qiw::DeviceScope dev_scope(b->device);
  if (dev_scope.status != cudaSuccess) return b->fail(QIW_ERR_CUDA, std::string("qiw_batch_get_P: cudaSetDevice: ") + cudaGetErrorString(dev_scope.status));
  SolveRec *s = b->solves[id];
  std::vector<double> t(s->ctx->ptab_size);
  int rc;
  if ((rc = b->cuda(cudaStreamSynchronize(b->stream), "sync")) ||
      (rc = b->cuda(cudaMemcpy(t.data(), s->ctx->d_P.p, sizeof(double) * t.size(), cudaMemcpyDeviceToHost), "P")))
    return rc;
  for (size_t i = 0; i < t.size(); ++i) {  // P = -i * (i P)
    P[2 * i] = 0.0;
    P[2 * i + 1] = -t[i];
  }
  return QIW_OK;
}

int qiw_batch_stats_get(const qiw_batch *b, qiw_batch_stats *out) {
  if (!b || !out) return QIW_ERR_ARG;
  *out = b->st;
  return QIW_OK;
}

}  // extern "C"
