// Host-only access to the group planner (no CUDA): lets CPU tests execute a plan's
// instruction stream against the CPU oracle.  Not part of the public ABI in include/qiw.h.
#include <cstdlib>
#include <cstring>
#include <string>

#include "qiw.h"
#include "qiw_plan.hpp"

using namespace qiw;

extern "C" int qiwp_plan(const qiw_problem_desc *pd, const qiw_group_desc *gd, int64_t arena_budget,
                         Instr *ins, int64_t ins_cap, PmJob *pm, int64_t pm_cap, WJob *wj, int64_t w_cap,
                         int64_t *counts /* [3]: n_ins, n_pm, n_w */, int32_t *meta /* [64] */,
                         double *stats /* [5] */, char *err, int err_cap) {
  std::string e;
  HostProblem hp;
  GroupSpec gs;
  int rc = host_problem_from_desc(pd, &hp, &e);
  if (!rc) rc = group_spec_from_desc(gd, &gs, &e);
  Plan p;
  if (!rc) {
    PlanOptions opt;
    opt.arena_budget = arena_budget;
    if (const char *m = std::getenv("QIW_MAX_BATCH_FLOPS")) opt.max_batch_flops = std::atof(m);
    if (const char *m = std::getenv("QIW_MAX_BATCH_INSTRS")) opt.max_batch_instrs = std::atoll(m);
    rc = plan_group(hp, gs, opt, &p, &e);
  }
  if (rc) {
    if (err && err_cap > 0) {
      std::strncpy(err, e.c_str(), err_cap - 1);
      err[err_cap - 1] = 0;
    }
    return rc;
  }
  counts[0] = (int64_t)p.ins.size();
  counts[1] = (int64_t)p.pm.size();
  counts[2] = (int64_t)p.wj.size();
  if ((int64_t)p.ins.size() > ins_cap || (int64_t)p.pm.size() > pm_cap || (int64_t)p.wj.size() > w_cap)
    return QIW_ERR_MEMORY;  // caller retries with the sizes in counts
  std::memcpy(ins, p.ins.data(), p.ins.size() * sizeof(Instr));
  std::memcpy(pm, p.pm.data(), p.pm.size() * sizeof(PmJob));
  std::memcpy(wj, p.wj.data(), p.wj.size() * sizeof(WJob));
  std::memset(meta, 0, 64 * sizeof(int32_t));
  meta[0] = p.kind; meta[1] = p.order; meta[2] = p.n_nodes; meta[3] = p.D;
  meta[4] = p.d_before; meta[5] = p.d_after; meta[6] = p.use_bold; meta[7] = (int32_t)p.arena;
  meta[8] = p.res_size; meta[9] = p.n_fixed;
  for (int f = 0; f < kMaxFixed; ++f) { meta[10 + f] = p.fixed_pos[f]; meta[14 + f] = p.fixed_time[f]; }
  for (size_t j = 0; j < p.var_pos.size() && j < 32; ++j) meta[18 + j] = p.var_pos[j];
  stats[0] = p.flops; stats[1] = p.tree_flops; stats[2] = (double)p.tree_leaves;
  stats[3] = (double)p.dag_nodes; stats[4] = (double)p.n_batches;
  return 0;
}

// Per-batch flops per sample of a planned group (load-balance studies in the CPU tests).
extern "C" int qiwp_batch_flops(const qiw_problem_desc *pd, const qiw_group_desc *gd, int64_t arena_budget,
                                double *out, int cap) {
  std::string e;
  HostProblem hp;
  GroupSpec gs;
  int rc = host_problem_from_desc(pd, &hp, &e);
  if (!rc) rc = group_spec_from_desc(gd, &gs, &e);
  Plan p;
  if (!rc) {
    PlanOptions opt;
    opt.arena_budget = arena_budget;
    if (const char *m = std::getenv("QIW_MAX_BATCH_FLOPS")) opt.max_batch_flops = std::atof(m);
    if (const char *m = std::getenv("QIW_MAX_BATCH_INSTRS")) opt.max_batch_instrs = std::atoll(m);
    rc = plan_group(hp, gs, opt, &p, &e);
  }
  if (rc) return -rc;
  const int n = (int)p.batch_flops.size();
  for (int i = 0; i < n && i < cap; ++i) out[i] = p.batch_flops[i];
  return n;
}

// Instruction index where each batch of a planned group starts (n_batches + 1 entries).
extern "C" int qiwp_batch_begin(const qiw_problem_desc *pd, const qiw_group_desc *gd, int64_t arena_budget,
                                int32_t *out, int cap) {
  std::string e;
  HostProblem hp;
  GroupSpec gs;
  int rc = host_problem_from_desc(pd, &hp, &e);
  if (!rc) rc = group_spec_from_desc(gd, &gs, &e);
  Plan p;
  if (!rc) {
    PlanOptions opt;
    opt.arena_budget = arena_budget;
    if (const char *m = std::getenv("QIW_MAX_BATCH_FLOPS")) opt.max_batch_flops = std::atof(m);
    if (const char *m = std::getenv("QIW_MAX_BATCH_INSTRS")) opt.max_batch_instrs = std::atoll(m);
    rc = plan_group(hp, gs, opt, &p, &e);
  }
  if (rc) return -rc;
  const int n = (int)p.batch_begin.size();
  for (int i = 0; i < n && i < cap; ++i) out[i] = p.batch_begin[i];
  return n;
}
