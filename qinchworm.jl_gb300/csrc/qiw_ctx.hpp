// Internal: the context object behind the C ABI (shared by the API translation units).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include "qiw.h"
#include "qiw_internal.hpp"
#include "qiw_kernels.hpp"
#include "qiw_plan.hpp"

namespace qiw {

template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t reserve(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    size_t c = std::max<size_t>(count, 1);
    cudaError_t e = cudaMalloc(&p, c * sizeof(T));
    if (e == cudaSuccess) n = c;
    return e;
  }
  cudaError_t upload(const T *h, size_t count, cudaStream_t s) {
    cudaError_t e = reserve(count);
    if (e != cudaSuccess || count == 0) return e;
    return cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s);
  }
};

// Makes a context's device current for one library call and gives the caller's thread its
// previous current device back when the call returns, so no entry point leaves another device
// current behind.  `status` is the result of the switch; a call that needs the device checks it.
struct DeviceScope {
  int prev = -1;
  cudaError_t status = cudaSuccess;
  explicit DeviceScope(int device) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != device) status = cudaSetDevice(device);
    if (status != cudaSuccess || prev == device) prev = -1;   // nothing to give back
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope &) = delete;
  DeviceScope &operator=(const DeviceScope &) = delete;
};

// FP32 launches of few waves are bound by the longest batch a thread runs (its instruction
// count), not by throughput: a group may carry programs whose batches are split to at most
// kSplitInstrs[L] instructions (topology halves; more instructions in all), chosen per launch.
constexpr int kSplitLevels = 2;
constexpr int64_t kSplitInstrs[kSplitLevels] = {11000, 9000};

struct GroupRec {
  Plan plan;
  DevBuf<PmJob> pm;
  DevBuf<WJob> wj;
  DevBuf<Instr> ins, ins32;
  DevBuf<int32_t> batch;
  DevGroup dg;
  GroupRec *split[kSplitLevels] = {nullptr, nullptr};   // split-batch programs (null: same as this one)
  void release() {
    pm.release();
    wj.release();
    ins.release();
    ins32.release();
    batch.release();
    for (GroupRec *&s : split) {
      if (s) {
        s->release();
        delete s;
      }
      s = nullptr;
    }
  }
  // the program of split level L (0: this one)
  const GroupRec &level(int L) const { return (L > 0 && split[L - 1]) ? *split[L - 1] : *this; }
};

struct WarpRec;
constexpr int kAuxStreams = 16;   // most warps trained concurrently, one stream each

// Host-side launch tables of one qiw_integrate call.
struct LaunchTables {
  std::vector<DevWork> works;         // Sobol pointers hold offsets into `sobol` until placed
  std::vector<int4> cta_map;          // (work item, batch, first sample, partial row), heaviest first
  std::vector<double> cta_cost;        // estimated flops of each tile (before sorting)
  std::vector<int> cta_first, res_sizes, out_off;
  std::vector<uint32_t> sobol;
  int64_t arena_max = 0;
  int res_max = 0, out_total = 0;
  int level = 0;                      // split level of the programs the tables refer to
  double waves = 0.0;                 // FP32: tiles x threads over the SMs' resident threads
};

}  // namespace qiw

struct qiw_ctx {
  // (definition below uses qiw:: types)
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  double last_ms = 0.0;

  bool has_problem = false, has_P = false;
  bool real_phase_problem = true, real_phase_P = true;
  qiw::HostProblem hp;
  int n_tau = 0;
  double beta = 0.0, h = 0.0;
  std::vector<int> dims, eoff, ptab_off, res_off, delta_kind, delta_off;
  int64_t ptab_size = 0;
  int res_total = 0;

  qiw::DevBuf<int> d_dims, d_ptab_off, d_eoff, d_res_off, d_delta_kind, d_delta_off;
  qiw::DevBuf<double> d_E, d_P, d_opv, d_delta;
  qiw::DevBuf<float> d_Pf, d_opvf, d_deltaf;

  std::vector<qiw::GroupRec *> groups;
  qiw::DevBuf<qiw::DevGroup> d_groups;
  qiw::DevBuf<qiw::DevGroup> d_groups_split[qiw::kSplitLevels];   // per split level (parallel to d_groups)
  int n_sm = 0;                 // multiprocessors of the device
  bool groups_dirty = true;

  qiw::DevBuf<qiw::DevWork> d_works;
  qiw::DevBuf<int4> d_cta_map;
  qiw::DevBuf<double> d_partials, d_out;
  qiw::DevBuf<int> d_cta_first, d_res_sizes, d_out_off, d_err;
  qiw::DevBuf<uint32_t> d_sobol;
  qiw::DevBuf<double> d_pts, d_samples, d_norms;
  std::vector<qiw::WarpRec *> warps;
  std::vector<cudaStream_t> aux;   // streams of concurrent warp training (created on first use)
  std::vector<cudaEvent_t> aux_ev; // their fork / join events
  int threads = 64;            // samples per tile of the FP64 launches
  int threads32 = 128;         // samples per tile of the FP32 launches (eg step 15.2 -> 14.6 ms against 64)
  int eval_extra_smem = 0;     // tuning: extra dynamic shared memory per CTA (limits CTAs per SM)
  int eval_carveout = -1;      // tuning: preferred shared-memory carveout in percent (-1: driver default)

  int fail(int code, const std::string &msg) {
    err = msg;
    return code;
  }
  int cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return QIW_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return QIW_ERR_CUDA;
  }
  void clear_groups() {
    for (auto *g : groups) {
      g->release();
      delete g;
    }
    groups.clear();
    groups_dirty = true;
  }
  qiw::DevProblem dev_problem(bool fp32) const {
    qiw::DevProblem p;
    std::memset(&p, 0, sizeof(p));
    p.S = hp.S;
    p.n_tau = n_tau;
    p.n_pairs = hp.n_pairs;
    p.h = h;
    p.inv_h = 1.0 / h;
    p.beta = beta;
    p.dims = d_dims.p;
    p.ptab_off = d_ptab_off.p;
    p.eoff = d_eoff.p;
    p.res_off = d_res_off.p;
    p.E = d_E.p;
    p.P = fp32 ? (const void *)d_Pf.p : (const void *)d_P.p;
    p.opv = fp32 ? (const void *)d_opvf.p : (const void *)d_opv.p;
    p.delta = fp32 ? (const void *)d_deltaf.p : (const void *)d_delta.p;
    p.delta_kind = d_delta_kind.p;
    p.delta_off = d_delta_off.p;
    return p;
  }
};


namespace qiw {
// Validates the work items and builds the launch tables (no device memory touched).
int prepare_launch(qiw_ctx *c, int32_t n_work, const qiw_work_desc *work, int32_t precision, LaunchTables *t);
// Plans a group on c's problem, uploads its program and fills its device descriptor.
// with_splits: also plan the split-batch programs of FP32 launches (kSplitInstrs).
int build_group(qiw_ctx *c, const GroupSpec &gs, GroupRec **out, bool with_splits = false);
// Uploads the group descriptor table if groups changed.
int sync_groups(qiw_ctx *c);
// Learned warps (csrc/qiw_warp.cu).
void destroy_warps(qiw_ctx *c);
int warp_dim(qiw_ctx *c, int id);
int warp_map_device(qiw_ctx *c, int id, const uint32_t *m_dev, const uint32_t *x0_dev, uint64_t first, uint64_t n,
                    double *pts_dev, cudaStream_t st = nullptr);   // st null: the context stream
// Auxiliary streams of a context: create up to n, fork them from the context stream (they wait
// for its work so far), join them back (the context stream waits for theirs).
int aux_streams(qiw_ctx *c, int n);
int aux_fork(qiw_ctx *c, int n);
int aux_join(qiw_ctx *c, int n);
// qiw_integrate with optional learned warps per work item and optional per-sample results.
int integrate_impl(qiw_ctx *c, int32_t n_work, const qiw_work_desc *work, int32_t precision, double *out,
                   const int32_t *warp_ids, double *sample_out, double *norms_out = nullptr);
// Launches the kernels on launch tables already in device memory (timed by ev0/ev1).
int launch_tables(qiw_ctx *c, const LaunchTables &t, int32_t precision, const DevGroup *groups, const DevWork *works,
                  const int4 *cta_map, const int *cta_first, const int *res_sizes, const int *out_off,
                  double *partials, int *err, double *out);
}  // namespace qiw
