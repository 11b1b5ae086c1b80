// qiw_integrate_noalloc: the integration entry point for callers that cannot allocate device
// memory while they run (for example code that executes between the phases of a host
// framework that owns every device allocation, or inside a region where cudaMalloc is not
// permitted).  It runs the same kernels as qiw_integrate, but its scratch -- work
// descriptors, CTA map, Sobol tables, per-CTA partial sums and the error word -- lives in the
// file-scope device array below, and the result is written straight into a device buffer
// the caller owns.  It calls no cudaMalloc, cudaFree or other allocating routine.
//
// The array is QIW_NOALLOC_SCRATCH_BYTES (16 MiB) on every GPU that loads this library and
// stays reserved until the process exits.  Calls whose launch tables and partial sums would
// not fit are rejected with QIW_ERR_MEMORY.  All calls share the one array and it keeps the
// previous call's contents: the launch tables and the error word are rewritten in full by
// every call (the partial sums are overwritten by the kernels), so nothing stale is read;
// calls that overlap on the GPU (from several host threads or contexts on the same device)
// race on the array and must be serialised by the caller.
//
// The group descriptor table is staged into the array as well, so the call works right after
// qiw_group_create.  The device address of the array is looked up once per device, with that device current,
// by the first call on that device (cudaGetSymbolAddress); make that first call before any
// stream capture.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <vector>

#include "qiw_ctx.hpp"

#define QIW_NOALLOC_SCRATCH_BYTES (16u << 20)

static __device__ __align__(256) unsigned char g_qiw_noalloc_scratch[QIW_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of g_qiw_noalloc_scratch on `device`, which must be the current device
// (looked up once per device and cached; a lookup made with another device current would
// cache that device's copy, so it is refused).
cudaError_t scratch_address(int device, unsigned char **out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_scratch_mutex);
  if (!g_scratch_addr[device]) {
    int cur = -1;
    cudaError_t e0 = cudaGetDevice(&cur);
    if (e0 != cudaSuccess) return e0;
    if (cur != device) return cudaErrorInvalidDevice;
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_qiw_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device] = p;
  }
  *out = static_cast<unsigned char *>(g_scratch_addr[device]);
  return cudaSuccess;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

extern "C" int qiw_integrate_noalloc(qiw_ctx *c, int32_t n_work, const qiw_work_desc *work, int32_t precision,
                                     double *out_device) {
  using namespace qiw;
  if (!c || n_work < 0 || (n_work > 0 && (!work || !out_device))) return QIW_ERR_ARG;
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_integrate_noalloc: cudaSetDevice");
  if (n_work == 0) return QIW_OK;
  LaunchTables t;
  int rc = prepare_launch(c, n_work, work, precision, &t);
  if (rc) return rc;
  const int n_cta = (int)t.cta_map.size();
  // scratch layout: groups | works | cta_map | cta_first | res_sizes | out_off | sobol | err | partials
  std::vector<DevGroup> dgs;
  for (auto *g : c->groups) dgs.push_back(g->level(t.level).dg);
  size_t o = 0;
  const size_t o_groups = o;    o = align256(o + sizeof(DevGroup) * dgs.size());
  const size_t o_works = o;     o = align256(o + sizeof(DevWork) * t.works.size());
  const size_t o_map = o;       o = align256(o + sizeof(int4) * t.cta_map.size());
  const size_t o_first = o;     o = align256(o + sizeof(int) * t.cta_first.size());
  const size_t o_rs = o;        o = align256(o + sizeof(int) * t.res_sizes.size());
  const size_t o_off = o;       o = align256(o + sizeof(int) * t.out_off.size());
  const size_t o_sob = o;       o = align256(o + sizeof(uint32_t) * t.sobol.size());
  const size_t o_err = o;       o = align256(o + sizeof(int));
  const size_t staged = o;
  const size_t o_part = o;      o = align256(o + sizeof(double) * (size_t)n_cta * t.res_max);
  if (o > QIW_NOALLOC_SCRATCH_BYTES)
    return c->fail(QIW_ERR_MEMORY, "qiw_integrate_noalloc: the call needs " + std::to_string(o) +
                                       " bytes of scratch, the maximum is " +
                                       std::to_string((size_t)QIW_NOALLOC_SCRATCH_BYTES) +
                                       " (use fewer samples per call or qiw_integrate)");
  unsigned char *base = nullptr;
  if ((rc = c->cuda(scratch_address(c->device, &base), "qiw_integrate_noalloc: cudaGetSymbolAddress"))) return rc;
  // Stage every table (and a zero error word) in one host buffer, then one copy.
  std::vector<unsigned char> host(staged, 0);
  const uint32_t *sob_dev = reinterpret_cast<const uint32_t *>(base + o_sob);
  for (auto &w : t.works) {
    w.m = sob_dev + (uintptr_t)w.m;
    w.x0 = sob_dev + (uintptr_t)w.x0;
  }
  std::memcpy(host.data() + o_groups, dgs.data(), sizeof(DevGroup) * dgs.size());
  std::memcpy(host.data() + o_works, t.works.data(), sizeof(DevWork) * t.works.size());
  std::memcpy(host.data() + o_map, t.cta_map.data(), sizeof(int4) * t.cta_map.size());
  std::memcpy(host.data() + o_first, t.cta_first.data(), sizeof(int) * t.cta_first.size());
  std::memcpy(host.data() + o_rs, t.res_sizes.data(), sizeof(int) * t.res_sizes.size());
  std::memcpy(host.data() + o_off, t.out_off.data(), sizeof(int) * t.out_off.size());
  if (!t.sobol.empty()) std::memcpy(host.data() + o_sob, t.sobol.data(), sizeof(uint32_t) * t.sobol.size());
  cudaStream_t st = c->stream;
  if ((rc = c->cuda(cudaMemcpyAsync(base, host.data(), staged, cudaMemcpyHostToDevice, st), "stage tables")))
    return rc;
  rc = launch_tables(c, t, precision, reinterpret_cast<const DevGroup *>(base + o_groups),
                     reinterpret_cast<const DevWork *>(base + o_works),
                     reinterpret_cast<const int4 *>(base + o_map), reinterpret_cast<const int *>(base + o_first),
                     reinterpret_cast<const int *>(base + o_rs), reinterpret_cast<const int *>(base + o_off),
                     reinterpret_cast<double *>(base + o_part), reinterpret_cast<int *>(base + o_err), out_device);
  if (rc) return rc;
  int err_word = 0;
  if ((rc = c->cuda(cudaMemcpyAsync(&err_word, base + o_err, sizeof(int), cudaMemcpyDeviceToHost, st), "copy err")) ||
      (rc = c->cuda(cudaStreamSynchronize(st), "qiw_integrate_noalloc")))
    return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->last_ms = ms;
  if (err_word) return c->fail(QIW_ERR_DEVICE, "qiw_integrate_noalloc: non-finite result detected on the device");
  return QIW_OK;
}
