// CUDA kernels of the qMC diagram integration (sm_103a).
//
// One thread evaluates one qMC sample of one topology group:
//   1. Sobol point by Gray-code jump   x = x0 ^ XOR_{b in bits(n ^ n>>1)} m[:, b]
//      (src/scrambled_sobol.jl:158-173, bit-exact UInt32 arithmetic);
//   2. Root / DoubleSimplexRoot map onto ordered times (src/qmc_integrate.jl:229-238, 425-449);
//   3. i*P(t_{j+1}-t_j) blocks by linear interpolation of the P table, or the exact atomic
//      i*P0 = exp(-dt E) for the bare step (src/topology_eval.jl:357-374,
//      src/exact_atomic_ppgf.jl:109-118); i*Delta_p weights (src/topology_eval.jl:412-415);
//   4. the group's program: the merged configuration DAG built by the host planner.
// All threads of a CTA run the same (warp-uniform) instruction stream, so control flow never
// diverges; per-sample matrices live in the thread's arena (local memory, L1 resident).
//
// Real-phase arithmetic: on the imaginary branch i*P, i*Delta and the operator blocks are
// real, so every complex product of the reference has exactly zero cross terms; the host
// verifies that and the kernels compute the real parts only (the result is -i times it).
//
// Reduction: per-thread sector-block sums -> warp shuffles -> CTA shared memory (fixed
// order) -> per-CTA partials -> one CTA per work item sums its partials in order with
// Kahan compensation.  Re-runs are bit-identical.
#include <cuda_runtime.h>

#include <cstdint>

#include "qiw.h"
#include "qiw_internal.hpp"
#include "qiw_kernels.hpp"

namespace qiw {

template <typename T>
__device__ __forceinline__ T fmaT(T a, T b, T c);
template <>
__device__ __forceinline__ double fmaT<double>(double a, double b, double c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float fmaT<float>(float a, float b, float c) { return fmaf(a, b, c); }

__device__ __forceinline__ Instr load_instr(const Instr *p) {
  const int4 *q = reinterpret_cast<const int4 *>(p);
  int4 a = __ldg(q), b = __ldg(q + 1);
  Instr I;
  int4 *o = reinterpret_cast<int4 *>(&I);
  o[0] = a;
  o[1] = b;
  return I;
}

// Linear interpolation of a uniform-grid table at dt >= 0 (rule of qiw/gf.py: linear_interp).
__device__ __forceinline__ void lin_index(double dt, double inv_h, int n_tau, int *i, double *f) {
  double x = dt * inv_h;
  int k = (int)floor(x);
  k = k > n_tau - 2 ? n_tau - 2 : k;
  k = k < 0 ? 0 : k;
  *i = k;
  *f = x - (double)k;
}


// ---------------------------------------------------------------------------------------
// Matrix instructions.  Block dimensions 1, 2 and 4 (every sector of the Anderson and eg
// models) take fully unrolled paths: all operands are loaded into registers first, so the
// arena reads of one instruction are in flight together, then 4..64 independent FMAs run.
// Other dimensions use the generic loops.

__device__ __forceinline__ int dcode(int d) { return d == 1 ? 0 : d == 2 ? 1 : d == 4 ? 2 : -1; }

template <typename T, int R, int C>
__device__ __forceinline__ void pmul_u(T *A, int dst, int pm, int src) {
  T p[R * R], x[R * C];
#pragma unroll
  for (int i = 0; i < R * R; ++i) p[i] = A[pm + i];
#pragma unroll
  for (int i = 0; i < R * C; ++i) x[i] = A[src + i];
#pragma unroll
  for (int j = 0; j < C; ++j)
#pragma unroll
    for (int r = 0; r < R; ++r) {
      T acc = p[r] * x[j * R];
#pragma unroll
      for (int k = 1; k < R; ++k) acc = fmaT<T>(p[k * R + r], x[j * R + k], acc);
      A[dst + j * R + r] = acc;
    }
}

template <typename T, int R, int C>
__device__ __forceinline__ void pmuld_u(T *A, int dst, int pm, int src) {
  T p[R], x[R * C];
#pragma unroll
  for (int i = 0; i < R; ++i) p[i] = A[pm + i];
#pragma unroll
  for (int i = 0; i < R * C; ++i) x[i] = A[src + i];
#pragma unroll
  for (int j = 0; j < C; ++j)
#pragma unroll
    for (int r = 0; r < R; ++r) A[dst + j * R + r] = p[r] * x[j * R + r];
}

// dst (=|+=) coef * O * src.  MODE 0: no coefficient (coef == 1 exactly), MODE 1: the
// coefficient scales the smaller of src (K x C) and the product (R x C).
template <typename T, int R, int K, int C, int MODE>
__device__ __forceinline__ void omul_m(T *A, const T *O, int dst, int oa, int src, T coef, bool accf) {
  T o[R * K], x[K * C];
#pragma unroll
  for (int i = 0; i < R * K; ++i) o[i] = __ldg(O + oa + i);
#pragma unroll
  for (int i = 0; i < K * C; ++i) x[i] = A[src + i];
  constexpr bool scale_src = (MODE == 1) && (K < R);
  if (scale_src) {
#pragma unroll
    for (int i = 0; i < K * C; ++i) x[i] *= coef;
  }
#pragma unroll
  for (int j = 0; j < C; ++j)
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int d = dst + j * R + r;
      T acc;
      if (accf && !(MODE == 1 && !scale_src)) {
        // accumulate into the destination: the chain starts from its value (K FMAs)
        acc = A[d];
#pragma unroll
        for (int k = 0; k < K; ++k) acc = fmaT<T>(o[k * R + r], x[j * K + k], acc);
      } else {
        acc = o[r] * x[j * K];
#pragma unroll
        for (int k = 1; k < K; ++k) acc = fmaT<T>(o[k * R + r], x[j * K + k], acc);
        if (MODE == 1 && !scale_src) acc = accf ? fmaT<T>(coef, acc, A[d]) : coef * acc;
      }
      A[d] = acc;
    }
}

template <typename T, int R, int K, int C>
__device__ __forceinline__ void omul_u(T *A, const T *O, int dst, int oa, int src, T coef, bool accf,
                                       bool has_coef) {
  if (has_coef) omul_m<T, R, K, C, 1>(A, O, dst, oa, src, coef, accf);
  else omul_m<T, R, K, C, 0>(A, O, dst, oa, src, coef, accf);
}

template <typename T, int N>
__device__ __forceinline__ void axpy_u(T *A, int dst, int src, T coef, bool accf, bool has_coef) {
  T x[N];
#pragma unroll
  for (int i = 0; i < N; ++i) x[i] = A[src + i];
  if (has_coef) {
#pragma unroll
    for (int i = 0; i < N; ++i) A[dst + i] = accf ? fmaT<T>(coef, x[i], A[dst + i]) : coef * x[i];
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) A[dst + i] = accf ? x[i] + A[dst + i] : x[i];
  }
}

#define QIW_D3(F, ...)                                                                            \
  switch (code) {                                                                                 \
    case 0: F<T, 1, 1, 1>(__VA_ARGS__); break;  case 1: F<T, 1, 1, 2>(__VA_ARGS__); break;        \
    case 2: F<T, 1, 1, 4>(__VA_ARGS__); break;  case 3: F<T, 1, 2, 1>(__VA_ARGS__); break;        \
    case 4: F<T, 1, 2, 2>(__VA_ARGS__); break;  case 5: F<T, 1, 2, 4>(__VA_ARGS__); break;        \
    case 6: F<T, 1, 4, 1>(__VA_ARGS__); break;  case 7: F<T, 1, 4, 2>(__VA_ARGS__); break;        \
    case 8: F<T, 1, 4, 4>(__VA_ARGS__); break;  case 9: F<T, 2, 1, 1>(__VA_ARGS__); break;        \
    case 10: F<T, 2, 1, 2>(__VA_ARGS__); break; case 11: F<T, 2, 1, 4>(__VA_ARGS__); break;       \
    case 12: F<T, 2, 2, 1>(__VA_ARGS__); break; case 13: F<T, 2, 2, 2>(__VA_ARGS__); break;       \
    case 14: F<T, 2, 2, 4>(__VA_ARGS__); break; case 15: F<T, 2, 4, 1>(__VA_ARGS__); break;       \
    case 16: F<T, 2, 4, 2>(__VA_ARGS__); break; case 17: F<T, 2, 4, 4>(__VA_ARGS__); break;       \
    case 18: F<T, 4, 1, 1>(__VA_ARGS__); break; case 19: F<T, 4, 1, 2>(__VA_ARGS__); break;       \
    case 20: F<T, 4, 1, 4>(__VA_ARGS__); break; case 21: F<T, 4, 2, 1>(__VA_ARGS__); break;       \
    case 22: F<T, 4, 2, 2>(__VA_ARGS__); break; case 23: F<T, 4, 2, 4>(__VA_ARGS__); break;       \
    case 24: F<T, 4, 4, 1>(__VA_ARGS__); break; case 25: F<T, 4, 4, 2>(__VA_ARGS__); break;       \
    default: F<T, 4, 4, 4>(__VA_ARGS__); break;                                                   \
  }

#define QIW_D2(F, ...)                                                                            \
  switch (code) {                                                                                 \
    case 0: F<T, 1, 1>(__VA_ARGS__); break; case 1: F<T, 1, 2>(__VA_ARGS__); break;               \
    case 2: F<T, 1, 4>(__VA_ARGS__); break; case 3: F<T, 2, 1>(__VA_ARGS__); break;               \
    case 4: F<T, 2, 2>(__VA_ARGS__); break; case 5: F<T, 2, 4>(__VA_ARGS__); break;               \
    case 6: F<T, 4, 1>(__VA_ARGS__); break; case 7: F<T, 4, 2>(__VA_ARGS__); break;               \
    default: F<T, 4, 4>(__VA_ARGS__); break;                                                      \
  }

template <typename T, int RESMAX>
__device__ __forceinline__ void exec_instr(const Instr &I, T *A, const T *O, double *R) {
  const int rows = I.rows, cols = I.cols;
  switch (I.op) {
    case OP_LOADP: {
      const T c = (T)I.c;
      if (I.inner) {
#pragma unroll 1
        for (int j = 0; j < rows; ++j)
#pragma unroll 1
          for (int r = 0; r < rows; ++r) A[I.dst + j * rows + r] = (r == j) ? c * A[I.a + r] : (T)0;
      } else {
#pragma unroll 1
        for (int e = 0; e < rows * rows; ++e) A[I.dst + e] = c * A[I.a + e];
      }
      break;
    }
    case OP_LOADC: {
      const T c = (T)I.c;
#pragma unroll 1
      for (int e = 0; e < rows * cols; ++e) A[I.dst + e] = c * __ldg(O + I.a + e);
      break;
    }
    case OP_PMUL: {
      const int cr = dcode(rows), cc = dcode(cols);
      if (cr >= 0 && cc >= 0) {
        const int code = cr * 3 + cc;
        QIW_D2(pmul_u, A, I.dst, I.a, I.src)
      } else {
#pragma unroll 1
        for (int j = 0; j < cols; ++j)
#pragma unroll 1
          for (int r = 0; r < rows; ++r) {
            T acc = (T)0;
#pragma unroll 4
            for (int k = 0; k < rows; ++k) acc = fmaT<T>(A[I.a + k * rows + r], A[I.src + j * rows + k], acc);
            A[I.dst + j * rows + r] = acc;
          }
      }
      break;
    }
    case OP_PMULD: {
      const int cr = dcode(rows), cc = dcode(cols);
      if (cr >= 0 && cc >= 0) {
        const int code = cr * 3 + cc;
        QIW_D2(pmuld_u, A, I.dst, I.a, I.src)
      } else {
#pragma unroll 1
        for (int j = 0; j < cols; ++j)
#pragma unroll 1
          for (int r = 0; r < rows; ++r) A[I.dst + j * rows + r] = A[I.a + r] * A[I.src + j * rows + r];
      }
      break;
    }
    case OP_OMUL: {
      const int inner = I.inner;
      const bool has_coef = (I.w >= 0) || (I.c != 1.0);
      const T coef = (I.w >= 0) ? (I.c == 1.0 ? A[I.w] : (T)I.c * A[I.w]) : (T)I.c;
      const int cr = dcode(rows), ck = dcode(inner), cc = dcode(cols);
      if (cr >= 0 && ck >= 0 && cc >= 0) {
        const int code = cr * 9 + ck * 3 + cc;
        QIW_D3(omul_u, A, O, I.dst, I.a, I.src, coef, I.acc != 0, has_coef)
      } else {
#pragma unroll 1
        for (int j = 0; j < cols; ++j)
#pragma unroll 1
          for (int r = 0; r < rows; ++r) {
            T acc = (T)0;
#pragma unroll 4
            for (int k = 0; k < inner; ++k) acc = fmaT<T>(__ldg(O + I.a + k * rows + r), A[I.src + j * inner + k], acc);
            const int o = I.dst + j * rows + r;
            A[o] = I.acc ? fmaT<T>(coef, acc, A[o]) : coef * acc;
          }
      }
      break;
    }
    case OP_AXPY: {
      const bool has_coef = (I.w >= 0) || (I.c != 1.0);
      const T coef = (I.w >= 0) ? (I.c == 1.0 ? A[I.w] : (T)I.c * A[I.w]) : (T)I.c;
      const int n = rows * cols;
      const bool accf = I.acc != 0;
      switch (n) {
        case 1: axpy_u<T, 1>(A, I.dst, I.src, coef, accf, has_coef); break;
        case 2: axpy_u<T, 2>(A, I.dst, I.src, coef, accf, has_coef); break;
        case 4: axpy_u<T, 4>(A, I.dst, I.src, coef, accf, has_coef); break;
        case 8: axpy_u<T, 8>(A, I.dst, I.src, coef, accf, has_coef); break;
        case 16: axpy_u<T, 16>(A, I.dst, I.src, coef, accf, has_coef); break;
        default:
#pragma unroll 1
          for (int e = 0; e < n; ++e) {
            const int o = I.dst + e;
            A[o] = accf ? fmaT<T>(coef, A[I.src + e], A[o]) : coef * A[I.src + e];
          }
      }
      break;
    }
    case OP_LEAF: {
#pragma unroll 1
      for (int e = 0; e < rows * cols; ++e) R[I.a + e] += (double)A[I.src + e];
      break;
    }
    default:
      break;
  }
}

// Times and sample range of one tile: t_i, t_w, t_f of the work item, the Sobol index of its
// first sample (first_index), the work item's sample count, the Sobol tables and the optional
// warped points / per-sample output of qiw_integrate_warped / qiw_integrate_samples.
struct TileSrc {
  double t_i, t_w, t_f;
  uint64_t first_index, n_samples;
  const uint32_t *m, *x0;
  const double *pts;
  double *sample_out;
};

// One tile: blockDim.x samples [s0, s0 + blockDim.x) of batch `batch` of group g, reduced to
// the CTA's partial sums prow[0 .. res_size).  Every thread of the CTA must call it.
template <typename T, int ARENA, int RESMAX>
__device__ __forceinline__ void eval_tile(const DevProblem &pb, const DevGroup &g, const TileSrc &w, int batch,
                                          uint64_t s0, double *__restrict__ prow) {
  const uint64_t sidx = s0 + threadIdx.x;
  const bool active = sidx < w.n_samples;
  const int res_size = g.res_size;

  T A[ARENA];
  double R[RESMAX];
#pragma unroll 1
  for (int e = 0; e < res_size; ++e) R[e] = 0.0;

  double wt = 1.0;
  if (active) {
    double tm[kMaxNodes];
    const double tsel[3] = {w.t_i, w.t_w, w.t_f};
#pragma unroll 1
    for (int f = 0; f < g.n_fixed; ++f) tm[g.fixed_pos[f]] = tsel[g.fixed_time[f]];
    const int D = g.D;
    if (D > 0) {
      const uint64_t n = w.first_index + sidx;
      const uint32_t gray = (uint32_t)(n ^ (n >> 1));
      double u[kMaxDim];
#pragma unroll 1
      if (w.pts) {  // warped point x = w(y) of a learned change of variables, weight 1/q(x)
        const double *pp = w.pts + sidx * (uint64_t)(D + 1);
#pragma unroll 1
        for (int d = 0; d < D; ++d) u[d] = pp[d];
        wt = pp[D];
      } else {
#pragma unroll 1
        for (int d = 0; d < D; ++d) {
          uint32_t v = __ldg(w.x0 + d);
          const uint32_t *md = w.m + d * 32;
#pragma unroll 8
          for (int b = 0; b < 32; ++b)
            if ((gray >> b) & 1u) v ^= __ldg(md + b);
          u[d] = ldexp((double)v, -32);  // exact: ldexp(Float64(x), -32)
        }
      }
      if (g.kind == 1) {  // RootTransform over [t_i, t_f]
        const double u_diff = w.t_f - w.t_i;
        double acc = pow(u[0], 1.0 / (double)D);
        u[0] = acc;
#pragma unroll 1
        for (int i = 2; i <= D; ++i) {
          acc = acc * pow(u[i - 1], 1.0 / (double)(D - i + 1));
          u[i - 1] = acc;
        }
#pragma unroll 1
        for (int i = 0; i < D; ++i) u[i] = w.t_i + u[i] * u_diff;
      } else {  // DoubleSimplexRootTransform
        const int dg = g.d_after, dl = g.d_before;
        const double fw = w.t_f - w.t_w, wi = w.t_w - w.t_i;
        double acc = pow(u[0], 1.0 / (double)dg);
        u[0] = acc;
#pragma unroll 1
        for (int i = 2; i <= dg; ++i) {
          acc = acc * pow(u[i - 1], 1.0 / (double)(dg - i + 1));
          u[i - 1] = acc;
        }
#pragma unroll 1
        for (int i = 0; i < dg; ++i) u[i] = u[i] * fw + w.t_w;
        if (dl > 0) {
          acc = pow(u[dg], 1.0 / (double)dl);
          u[dg] = acc;
#pragma unroll 1
          for (int i = dg + 2; i <= D; ++i) {
            acc = acc * pow(u[i - 1], 1.0 / (double)(D - i + 1));
            u[i - 1] = acc;
          }
#pragma unroll 1
          for (int i = dg; i < D; ++i) u[i] = u[i] * wi + w.t_i;
        }
      }
#pragma unroll 1
      for (int j = 0; j < D; ++j) tm[g.var_pos[j]] = u[j];
    }

    // i*P blocks of the intervals the program uses.
    const T *Ptab = reinterpret_cast<const T *>(pb.P);
#pragma unroll 1
    for (int j = 0; j < g.n_pm; ++j) {
      const PmJob job = g.pm[j];
      double dt = tm[job.iv + 1] - tm[job.iv];
      dt = dt < 0.0 ? 0.0 : dt;  // time-ordering violations from rounding (topology_eval.jl:361-364)
      const int d = pb.dims[job.s];
      if (g.use_bold) {
        int i;
        double f;
        lin_index(dt, pb.inv_h, pb.n_tau, &i, &f);
        const T *a = Ptab + pb.ptab_off[job.s] + (size_t)i * d * d;
        const T ff = (T)f;
#pragma unroll 1
        for (int e = 0; e < d * d; ++e) {
          const T lo = __ldg(a + e), hi = __ldg(a + d * d + e);
          A[job.off + e] = fmaT<T>(ff, hi - lo, lo);
        }
      } else {
        const double *E = pb.E + pb.eoff[job.s];
#pragma unroll 1
        for (int e = 0; e < d; ++e) A[job.off + e] = (T)exp(-dt * __ldg(E + e));
      }
    }
    // i*Delta weights.
    const T *Dtab = reinterpret_cast<const T *>(pb.delta);
#pragma unroll 1
    for (int j = 0; j < g.n_w; ++j) {
      const WJob job = g.wj[j];
      double dt = tm[job.tail] - tm[job.head];
      dt = dt < 0.0 ? 0.0 : dt;  // topology_eval.jl:407-410
      int i;
      double f;
      lin_index(dt, pb.inv_h, pb.n_tau, &i, &f);
      const T *t = Dtab + pb.delta_off[job.pair];
      T val;
      if (pb.delta_kind[job.pair] == 0) {
        const T lo = __ldg(t + i), hi = __ldg(t + i + 1);
        val = fmaT<T>((T)f, hi - lo, lo);
      } else {  // natural cubic spline, per-segment polynomial in f
        const T *c = t + 4 * i;
        const T ff = (T)f;
        val = fmaT<T>(ff, fmaT<T>(ff, fmaT<T>(ff, __ldg(c + 3), __ldg(c + 2)), __ldg(c + 1)), __ldg(c));
      }
      A[job.off] = val;
    }

    // The group's program: instructions of this CTA's batch.
    const T *O = reinterpret_cast<const T *>(pb.opv);
    const int i0 = __ldg(g.batch_begin + batch), i1 = __ldg(g.batch_begin + batch + 1);
#pragma unroll 1
    for (int ip = i0; ip < i1; ++ip) {
      const Instr I = load_instr(g.ins + ip);
      exec_instr<T, RESMAX>(I, A, O, R);
    }
    if (w.pts) {
#pragma unroll 1
      for (int e = 0; e < res_size; ++e) R[e] *= wt;
    }
    if (w.sample_out) {  // per-sample values (batches of one sample add up)
#pragma unroll 1
      for (int e = 0; e < res_size; ++e) atomicAdd(w.sample_out + sidx * (uint64_t)res_size + e, R[e]);
    }
  }

  // Deterministic CTA reduction of R -> prow[0 .. res_size).
  __shared__ double red[kMaxThreads / 32][RESMAX];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n_warps = (blockDim.x + 31) >> 5;
#pragma unroll 1
  for (int e = 0; e < res_size; ++e) {
    double v = R[e];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][e] = v;
  }
  __syncthreads();
#pragma unroll 1
  for (int e = threadIdx.x; e < res_size; e += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < n_warps; ++k) s += red[k][e];
    prow[e] = s;
  }
}

template <typename T, int ARENA, int RESMAX>
__global__ void __launch_bounds__(kMaxThreads, kMinBlocks)
    eval_kernel(DevProblem pb, const DevGroup *__restrict__ groups, const DevWork *__restrict__ works,
                const int4 *__restrict__ cta_map, double *__restrict__ partials) {
  const int4 cm = cta_map[blockIdx.x];   // (work item, batch, first sample of the tile, -)
  const DevWork &w = works[cm.x];
  const DevGroup &g = groups[w.group];
  const TileSrc src{w.t_i, w.t_w, w.t_f, w.first_index, w.n_samples, w.m, w.x0, w.pts, w.sample_out};
  eval_tile<T, ARENA, RESMAX>(pb, g, src, cm.y, (uint64_t)cm.z, partials + (size_t)blockIdx.x * g.res_size);
}

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
    eval_tile<T, ARENA, RESMAX>(spb, g, src, cm.y, (uint64_t)cm.z, partials + (size_t)cm.w * pstride);
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
// (normalize!(P, tau), src/ppgf.jl:646-654).  The FP32 copy is refreshed.
__global__ void batch_update_kernel(const DevProblem *__restrict__ probs, const BatchSolve *__restrict__ solves,
                                    const BatchWork *__restrict__ works, const double *__restrict__ res,
                                    int step) {
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
      const double lam = log(pmax) / so.taus[j];
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
  batch_eval_kernel<T, ARENA, RESMAX><<<a.grid, a.threads, 0, a.stream>>>(
      a.probs, a.solves, a.groups, a.works, a.tiles, a.n_tiles, a.ticket, a.partials, a.pstride, a.step);
  return cudaGetLastError();
}

template <typename T, int ARENA, int RESMAX>
static int occ_t(int threads) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batch_eval_kernel<T, ARENA, RESMAX>, threads, 0) !=
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
  auto f = [&]() -> int { QIW_BATCH_DISPATCH(occ_t, a.threads); };
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
  batch_update_kernel<<<a.n_solves, 128, 0, a.stream>>>(a.probs, a.solves, a.works, a.res, a.step);
  return cudaGetLastError();
}

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

template <typename T, int ARENA, int RESMAX>
static cudaError_t launch_t(const LaunchArgs &a) {
  eval_kernel<T, ARENA, RESMAX><<<a.n_cta, a.threads, 0, a.stream>>>(a.pb, a.groups, a.works, a.cta_map,
                                                                       a.partials);
  return cudaGetLastError();
}

int arena_class(int64_t arena) {
  if (arena <= kArenaSmall) return 0;
  if (arena <= kArenaLarge) return 1;
  if (arena <= kArenaHuge) return 2;
  return -1;
}

cudaError_t launch_eval(const LaunchArgs &a) {
  const bool big_res = a.res_max > kResSmall;
  const int ac = arena_class(a.arena_max);
  if (a.fp32) {
    if (ac == 0) return big_res ? launch_t<float, kArenaSmall, kResLarge>(a) : launch_t<float, kArenaSmall, kResSmall>(a);
    if (ac == 2) return launch_t<float, kArenaHuge, kResLarge>(a);
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
