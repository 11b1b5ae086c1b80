// Host-side planner: turns one topology group into a sample-independent program.
#pragma once
#include <complex>
#include <string>
#include <vector>

#include "qiw_internal.hpp"

namespace qiw {

using cd = std::complex<double>;

struct HostProblem {
  int S = 0;
  std::vector<int> dims;
  int n_ops = 0;
  std::vector<int> op_target;          // [n_ops * S], -1: no block
  std::vector<int64_t> op_valoff;      // [n_ops * S] complex-element offset, column-major d_f x d_i
  std::vector<cd> op_vals;
  int identity_op = 0;
  int n_pairs = 0;
  std::vector<int> pair_op_i, pair_op_f;
  int target(int op, int s) const { return op_target[(size_t)op * S + s]; }
};

struct GroupSpec {
  int kind = 0, order = 0, n_pts_after = 0;
  int corr_A = -1, corr_B = -1;
  std::vector<std::vector<std::pair<int, int>>> tops;   // 1-based vertex pairs
  std::vector<int> parity;
};

struct PlanOptions {
  int64_t arena_budget = 4096;   // per-sample working-set budget (elements)
  bool fold_scalar_ops = true;   // fold 1x1 operator blocks into coefficients
  bool fuse_scalar = true;       // all sectors 1-dimensional: fuse a P multiply into its only AXPY
  double max_batch_flops = 0.0;  // > 0: split batches above this many flops per sample (topology halves)
  int64_t max_batch_instrs = 0;  // > 0: split batches above this many instructions (topology halves)
};

struct Plan {
  int kind = 0, order = 0, n_nodes = 0, D = 0, d_before = 0, d_after = 0;
  int use_bold = 1;
  int n_fixed = 0;
  int fixed_pos[kMaxFixed] = {0, 0, 0, 0};
  int fixed_time[kMaxFixed] = {0, 0, 0, 0};
  std::vector<int> var_pos;
  std::vector<Instr> ins;
  std::vector<PmJob> pm;
  std::vector<WJob> wj;
  int64_t arena = 0;
  int res_size = 0;
  int64_t dag_nodes = 0;
  double flops = 0.0;            // per sample, real-phase count (x4 for complex)
  double tree_flops = 0.0;       // per sample, reference tree (complex arithmetic)
  int64_t tree_leaves = 0;
  int n_batches = 0;
  std::vector<int32_t> batch_begin;   // instruction index of each batch start, + end sentinel
  std::vector<double> batch_flops;    // flops per sample of each batch
};

// Returns 0 on success, a QIW_ERR_* code otherwise (message in *err).
int plan_group(const HostProblem &pb, const GroupSpec &g, const PlanOptions &opt, Plan *out,
               std::string *err);

// Everything a group program depends on, as bytes: the operator structure of the problem
// (sector dimensions, block targets and values, pair operators) and the group (kind, order,
// n_pts_after, correlator operators, topologies, parities).  Equal keys give equal plans for
// equal PlanOptions; the times, P and Delta tables are not part of a plan.
std::string plan_key(const HostProblem &hp, const GroupSpec &gs);

}  // namespace qiw

namespace qiw {
// Conversions from the C-ABI descriptors (no CUDA involved).
int host_problem_from_desc(const void *problem_desc, HostProblem *hp, std::string *err);
int group_spec_from_desc(const void *group_desc, GroupSpec *gs, std::string *err);

}  // namespace qiw
