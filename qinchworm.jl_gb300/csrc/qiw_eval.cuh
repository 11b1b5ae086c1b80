// Device code of the qMC diagram integration (sm_103a), shared by the kernel translation units.
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
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "qiw.h"
#include "qiw_dispatch.hpp"
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

// Register copy of a P multiply's product for the out-edges that follow it: blocks of at most
// kRegTmp elements (dims 1, 2, 4).  Instruction flag bits set by the planner: 2 = the source is
// the register copy, 3 = keep the product in registers, 4 = skip the product's arena store.
constexpr int kRegTmp = 16;
#ifndef QIW_BLOCK3
#define QIW_BLOCK3 1
#endif
#ifndef QIW_PREFETCH_INSTR
#define QIW_PREFETCH_INSTR 1
#endif

// Dynamic shared memory of the evaluation kernels: the reduction rows [warps][RESMAX] doubles,
// then (launches with scalar programs) two instruction chunks of blockDim.x entries.
extern __shared__ __align__(16) unsigned char qiw_dyn_smem[];
__host__ __device__ constexpr size_t eval_smem_bytes(int threads, int resmax, bool stage) {
  return (size_t)((threads + 31) / 32) * resmax * sizeof(double) + (stage ? 2 * (size_t)threads * 32 : 0);
}

// Instruction staging: thread t copies instruction start + t (if < end) into dst[t] with two
// 16-byte cp.async (Instr is 16-byte aligned, 32 bytes).
__device__ __forceinline__ void stage_instr(Instr *dst, const Instr *src, int start, int end) {
  const int i = start + (int)threadIdx.x;
  if (i < end) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst + threadIdx.x);
    const char *gp = reinterpret_cast<const char *>(src + i);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gp) : "memory");
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s + 16u), "l"(gp + 16) : "memory");
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Coordinate of Sobol point n (0-based) by the Gray-code jump: x0 ^ XOR of md[b] over the set
// bits b of gray = n ^ (n >> 1).  It is the value the reference's next! returns on its (n+1)-th
// call (src/scrambled_sobol.jl:158-173: the first call returns the shift, call n+1 XORs column
// ctz(n) into it), so skip!(seq, k, exact=true) becomes a start at n = k (src/scrambled_sobol.jl:189-208).
__device__ __forceinline__ uint32_t sobol_coord(const uint32_t *__restrict__ md, uint32_t x0d, uint32_t gray) {
  uint32_t v = x0d;
#pragma unroll 8
  for (int b = 0; b < 32; ++b)
    if ((gray >> b) & 1u) v ^= __ldg(md + b);
  return v;
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

// The same product kept in registers t[] for the out-edges that follow it (flag bit 3); the
// arena copy is written unless no later instruction reads it (flag bit 4).  Same roundings.
template <typename T, int R, int C>
__device__ __forceinline__ void pmul_r(T *A, T (&t)[kRegTmp], int dst, int pm, int src, bool store) {
  static_assert(R * C <= kRegTmp, "register product");
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
      t[j * R + r] = acc;
    }
  if (store) {
#pragma unroll
    for (int i = 0; i < R * C; ++i) A[dst + i] = t[i];
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
// XR: src is the register copy t[] of the preceding P multiply (flag bit 2), not the arena.
template <typename T, int R, int K, int C, int MODE, bool XR>
__device__ __forceinline__ void omul_m(T *A, const T *O, int dst, int oa, int src, T coef, bool accf,
                                       const T (&t)[kRegTmp]) {
  T o[R * K], x[K * C];
#pragma unroll
  for (int i = 0; i < R * K; ++i) o[i] = __ldg(O + oa + i);
#pragma unroll
  for (int i = 0; i < K * C; ++i) x[i] = XR ? t[i] : A[src + i];
  constexpr bool scale_src = (MODE == 1) && (K < R);
  if (scale_src) {
#pragma unroll
    for (int i = 0; i < K * C; ++i) x[i] *= coef;
  }
  // One body for both accumulation modes: the chain starts from the destination's value, or from
  // zero when overwriting (fma(a, b, 0) is the rounded product a*b, so the roundings are those of
  // a chain that starts with a multiply; only the sign of an exact zero can differ).
#pragma unroll
  for (int j = 0; j < C; ++j)
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int d = dst + j * R + r;
      const T base = accf ? A[d] : (T)0;
      T acc;
      if constexpr (MODE == 1 && !scale_src) {   // coef * (O x), added to the destination
        T sum = o[r] * x[j * K];
#pragma unroll
        for (int k = 1; k < K; ++k) sum = fmaT<T>(o[k * R + r], x[j * K + k], sum);
        acc = fmaT<T>(coef, sum, base);
      } else {                                    // the chain starts from the destination
        acc = base;
#pragma unroll
        for (int k = 0; k < K; ++k) acc = fmaT<T>(o[k * R + r], x[j * K + k], acc);
      }
      A[d] = acc;
    }
}

template <typename T, int R, int K, int C>
__device__ __forceinline__ void omul_u(T *A, const T *O, int dst, int oa, int src, T coef, bool accf,
                                       bool has_coef, const T (&t)[kRegTmp]) {
  if (has_coef) omul_m<T, R, K, C, 1, false>(A, O, dst, oa, src, coef, accf, t);
  else omul_m<T, R, K, C, 0, false>(A, O, dst, oa, src, coef, accf, t);
}

template <typename T, int R, int K, int C>
__device__ __forceinline__ void omul_ur(T *A, const T *O, int dst, int oa, int src, T coef, bool accf,
                                        bool has_coef, const T (&t)[kRegTmp]) {
  if constexpr (K * C <= kRegTmp) {
    if (has_coef) omul_m<T, R, K, C, 1, true>(A, O, dst, oa, src, coef, accf, t);
    else omul_m<T, R, K, C, 0, true>(A, O, dst, oa, src, coef, accf, t);
  }
}

template <typename T, int N, bool XR>
__device__ __forceinline__ void axpy_u(T *A, int dst, int src, T coef, bool accf, bool has_coef,
                                       const T (&t)[kRegTmp]) {
  T x[N];
#pragma unroll
  for (int i = 0; i < N; ++i) x[i] = XR ? t[i] : A[src + i];
  if (has_coef) {   // fma(coef, x, 0) = coef * x
#pragma unroll
    for (int i = 0; i < N; ++i) A[dst + i] = fmaT<T>(coef, x[i], accf ? A[dst + i] : (T)0);
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) A[dst + i] = x[i] + (accf ? A[dst + i] : (T)0);
  }
}

// Products whose row count is a multiple of 3 (sector dimensions 3 and 9, the t2g model): three
// rows of the left factor are held in registers and every column of the right factor is read
// once per row block, instead of one left and one right arena load per multiply-add.  The sums
// run over k in the same order from zero as the plain loops, so the results are identical.
// LEFT_O: the left factor is an operator block (read-only table) instead of an arena block.
template <typename T, bool LEFT_O>
__device__ __forceinline__ void mul_rows3(T *A, const T *O, int dst, int la, int src, int rows, int inner,
                                          int cols, T coef, bool scale, bool accf) {
  constexpr int KB = 9;   // inner dimension held per pass
#pragma unroll 1
  for (int r0 = 0; r0 < rows; r0 += 3) {
#pragma unroll 1
    for (int k0 = 0; k0 < inner; k0 += KB) {
      const int kn = min(KB, inner - k0);
      T l0[KB], l1[KB], l2[KB];
#pragma unroll
      for (int k = 0; k < KB; ++k) {
        if (k < kn) {
          const int e = la + (k0 + k) * rows + r0;
          l0[k] = LEFT_O ? __ldg(O + e) : A[e];
          l1[k] = LEFT_O ? __ldg(O + e + 1) : A[e + 1];
          l2[k] = LEFT_O ? __ldg(O + e + 2) : A[e + 2];
        }
      }
#pragma unroll 1
      for (int j = 0; j < cols; ++j) {
        const int o = dst + j * rows + r0;
        T a0, a1, a2;
        if (k0 == 0) {
          a0 = (T)0; a1 = (T)0; a2 = (T)0;
        } else {   // partial sums of the previous pass (kept in the destination)
          a0 = A[o]; a1 = A[o + 1]; a2 = A[o + 2];
        }
#pragma unroll
        for (int k = 0; k < KB; ++k) {
          if (k < kn) {
            const T x = A[src + j * inner + k0 + k];
            a0 = fmaT<T>(l0[k], x, a0);
            a1 = fmaT<T>(l1[k], x, a1);
            a2 = fmaT<T>(l2[k], x, a2);
          }
        }
        if (k0 + KB < inner) {   // more passes: keep the raw partial sums
          A[o] = a0; A[o + 1] = a1; A[o + 2] = a2;
        } else if (!scale) {
          A[o] = a0; A[o + 1] = a1; A[o + 2] = a2;
        } else {
          A[o] = accf ? fmaT<T>(coef, a0, A[o]) : coef * a0;
          A[o + 1] = accf ? fmaT<T>(coef, a1, A[o + 1]) : coef * a1;
          A[o + 2] = accf ? fmaT<T>(coef, a2, A[o + 2]) : coef * a2;
        }
      }
    }
  }
}

// Tensor-core operator multiply of the large-block FP32 kernels (sector dimension 9 in the
// inner index; opt-in, DevProblem::tc_stage > 0).  All 32 samples of a warp apply the same
// operator block O (rows x 9) to their own blocks X_s (9 x cols): per output column j that is
// one GEMM Y[:, (s, j)] = O . X[:, (s, j)] over the warp's samples, run as mma.sync m16n8k8 TF32
// (M = rows padded to 16, K = 9 padded to 16, N = 32 samples in 4 tiles of 8) with the 3xTF32
// split a = a_hi + a_lo (a_hi = tf32(a), a_lo = tf32(a - a_hi); products a_hi b_hi + a_hi b_lo +
// a_lo b_hi, FP32 accumulation).  The samples' blocks are staged in the warp's shared-memory
// area [32][9 * cols]; column j of the results overwrites column j of the staged blocks once
// every lane has read it.  Every lane of the warp must execute this (the kernel runs the
// program on all lanes when tc_stage > 0).  Fragment layouts (PTX ISA, m16n8k8 .tf32): lane
// 4g + t holds A[g][t], A[g+8][t], A[g][t+4], A[g+8][t+4]; B[t][g], B[t+4][g]; C[g][2t],
// C[g][2t+1], C[g+8][2t], C[g+8][2t+1].
constexpr int kTcK = 9, kTcMaxCols = 9, kTcWarpFloats = 32 * kTcK * kTcMaxCols;

__device__ __forceinline__ uint32_t tf32_bits(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void tf32_split(float x, uint32_t &hi, uint32_t &lo) {
  hi = tf32_bits(x);
  lo = tf32_bits(x - __uint_as_float(hi));
}
__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

static __device__ __noinline__ void omul_tc(float *A, const float *O, float *X, int dst, int oa, int src, int rows,
                                        int cols, float coef, bool accf) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int KC = kTcK * cols;
#pragma unroll 1
  for (int i = 0; i < KC; ++i) X[lane * KC + i] = A[src + i];
  uint32_t ah[2][4], al[2][4];
#pragma unroll
  for (int ks = 0; ks < 2; ++ks) {
    const int k0 = 8 * ks + t, k1 = k0 + 4;
    const float v0 = (g < rows && k0 < kTcK) ? __ldg(O + oa + k0 * rows + g) : 0.f;
    const float v1 = (g + 8 < rows && k0 < kTcK) ? __ldg(O + oa + k0 * rows + g + 8) : 0.f;
    const float v2 = (g < rows && k1 < kTcK) ? __ldg(O + oa + k1 * rows + g) : 0.f;
    const float v3 = (g + 8 < rows && k1 < kTcK) ? __ldg(O + oa + k1 * rows + g + 8) : 0.f;
    tf32_split(v0, ah[ks][0], al[ks][0]);
    tf32_split(v1, ah[ks][1], al[ks][1]);
    tf32_split(v2, ah[ks][2], al[ks][2]);
    tf32_split(v3, ah[ks][3], al[ks][3]);
  }
  __syncwarp();
#pragma unroll 1
  for (int j = 0; j < cols; ++j) {
    float c[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) c[q][0] = c[q][1] = c[q][2] = c[q][3] = 0.f;
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
      const int k0 = 8 * ks + t, k1 = k0 + 4;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float *xs = X + (8 * q + g) * KC + j * kTcK;
        uint32_t bh0, bl0, bh1, bl1;
        tf32_split(k0 < kTcK ? xs[k0] : 0.f, bh0, bl0);
        tf32_split(k1 < kTcK ? xs[k1] : 0.f, bh1, bl1);
        mma_tf32(c[q], ah[ks], bh0, bh1);
        mma_tf32(c[q], ah[ks], bl0, bl1);
        mma_tf32(c[q], al[ks], bh0, bh1);
      }
    }
    __syncwarp();   // column j of every sample has been read
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int s0 = 8 * q + 2 * t;
      if (g < rows) {
        X[s0 * KC + j * kTcK + g] = c[q][0];
        X[(s0 + 1) * KC + j * kTcK + g] = c[q][1];
      }
      if (g + 8 < rows) {
        X[s0 * KC + j * kTcK + g + 8] = c[q][2];
        X[(s0 + 1) * KC + j * kTcK + g + 8] = c[q][3];
      }
    }
  }
  __syncwarp();
#pragma unroll 1
  for (int j = 0; j < cols; ++j)
#pragma unroll 1
    for (int r = 0; r < rows; ++r) {
      const float y = X[lane * KC + j * kTcK + r];
      const int o = dst + j * rows + r;
      A[o] = accf ? fmaf(coef, y, A[o]) : coef * y;
    }
  __syncwarp();   // the staging area is reused by the next instruction
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

// Instruction coefficient in the compute type: FP64 programs hold c as a double, FP32 programs
// (DevGroup::ins32) hold it rounded to float in the low 4 bytes of the same slot, so neither
// path spends FP64-pipe work (compare or convert) per instruction.  Flag bit 0: c != 1.
template <typename T>
__device__ __forceinline__ T coef_c(const Instr &I);
template <>
__device__ __forceinline__ double coef_c<double>(const Instr &I) { return I.c; }
template <>
__device__ __forceinline__ float coef_c<float>(const Instr &I) {
  return __int_as_float((int)(unsigned)(__double_as_longlong(I.c) & 0xffffffffull));
}
__device__ __forceinline__ bool has_c(const Instr &I) { return (I.flags & 1u) != 0; }  // bit 1: c == -1

// Coefficient of an edge: c (flag bit 0: c != 1) times the per-sample weight A[w] when w >= 0.
// c == -1 exactly (flag bit 1) is a sign flip, which the consuming FMA takes for free.
// EAGER (block routines): the weight is loaded unconditionally (arena slot 0 always exists), so
// the load issues with the instruction's other operand loads (FP32 eg step -4 %); the scalar
// executor loads it only when the edge has one (its programs are bound by arena loads).
template <typename T, bool EAGER = true>
__device__ __forceinline__ T edge_coef(const Instr &I, const T *A) {
  T w;
  if constexpr (EAGER) {
    w = A[I.w < 0 ? 0 : I.w];
    if (I.w < 0) return coef_c<T>(I);
  } else {
    if (I.w < 0) return coef_c<T>(I);
    w = A[I.w];
  }
  if (!has_c(I)) return w;
  return (I.flags & 2u) ? -w : coef_c<T>(I) * w;
}

// Programs whose blocks are all 1x1 (single-orbital models): about 1.5 flops per
// instruction, so decoding and fetching the stream dominate; this executor has one short path
// per opcode and no block-shape dispatch.
template <typename T>
__device__ __forceinline__ void exec_scalar(const Instr &I, T *A, const T *O, double *R) {
  switch (I.op) {
    case OP_LOADP:
      A[I.dst] = has_c(I) ? coef_c<T>(I) * A[I.a] : A[I.a];
      break;
    case OP_LOADC:
      A[I.dst] = has_c(I) ? coef_c<T>(I) * __ldg(O + I.a) : __ldg(O + I.a);
      break;
    case OP_LOADI:
      A[I.dst] = coef_c<T>(I);
      break;
    case OP_PMUL:
    case OP_PMULD:
      A[I.dst] = A[I.a] * A[I.src];
      break;
    case OP_OMUL: {  // the roundings of omul_m<T, 1, 1, 1, MODE>
      const T o = __ldg(O + I.a), x = A[I.src];
      if (I.w < 0 && !has_c(I)) {
        A[I.dst] = I.acc ? fmaT<T>(o, x, A[I.dst]) : o * x;
      } else {
        const T coef = edge_coef<T, false>(I, A);
        const T p = o * x;
        A[I.dst] = I.acc ? fmaT<T>(coef, p, A[I.dst]) : coef * p;
      }
      break;
    }
    case OP_AXPY: {  // the roundings of axpy_u<T, 1>
      const T x = A[I.src];
      if (I.w < 0 && !has_c(I)) {
        A[I.dst] = I.acc ? x + A[I.dst] : x;
      } else {
        const T coef = edge_coef<T, false>(I, A);
        A[I.dst] = I.acc ? fmaT<T>(coef, x, A[I.dst]) : coef * x;
      }
      break;
    }
    case OP_PMAXPY: {  // PMUL then AXPY, the same roundings
      const T x = A[I.a] * A[I.src];
      if (I.w < 0 && !has_c(I)) {
        A[I.dst] = I.acc ? x + A[I.dst] : x;
      } else {
        const T coef = edge_coef<T, false>(I, A);
        A[I.dst] = I.acc ? fmaT<T>(coef, x, A[I.dst]) : coef * x;
      }
      break;
    }
    case OP_LEAF:
      R[I.a] += (double)A[I.src];
      break;
    default:
      break;
  }
}

// Flat dispatch (Instr::handler, computed on upload by handler_of): one jump to the routine
// instance for the instruction's opcode, block shape, coefficient mode and operand source.
// REG: this kernel keeps P products in registers; kernels that do not (FP64, large-block) run
// the register-source entries through the arena, as they ignore flag bits 2-4 everywhere.
#define QIW_RC9(M, B) M(B + 0, 1, 1) M(B + 1, 1, 2) M(B + 2, 1, 4) M(B + 3, 2, 1) M(B + 4, 2, 2) \
  M(B + 5, 2, 4) M(B + 6, 4, 1) M(B + 7, 4, 2) M(B + 8, 4, 4)
#define QIW_RKC27(M, B) \
  M(B + 0, 1, 1, 1) M(B + 1, 1, 1, 2) M(B + 2, 1, 1, 4) M(B + 3, 1, 2, 1) M(B + 4, 1, 2, 2) M(B + 5, 1, 2, 4) \
  M(B + 6, 1, 4, 1) M(B + 7, 1, 4, 2) M(B + 8, 1, 4, 4) M(B + 9, 2, 1, 1) M(B + 10, 2, 1, 2) M(B + 11, 2, 1, 4) \
  M(B + 12, 2, 2, 1) M(B + 13, 2, 2, 2) M(B + 14, 2, 2, 4) M(B + 15, 2, 4, 1) M(B + 16, 2, 4, 2) M(B + 17, 2, 4, 4) \
  M(B + 18, 4, 1, 1) M(B + 19, 4, 1, 2) M(B + 20, 4, 1, 4) M(B + 21, 4, 2, 1) M(B + 22, 4, 2, 2) M(B + 23, 4, 2, 4) \
  M(B + 24, 4, 4, 1) M(B + 25, 4, 4, 2) M(B + 26, 4, 4, 4)

template <typename T, bool REG>
__device__ __forceinline__ void exec_flat(const Instr &I, T *A, const T *O, T (&t)[kRegTmp]) {
  const bool accf = I.acc != 0;
  switch (I.handler) {
#define QIW_H_PMULR(H, R, C) \
  case H:                    \
    if constexpr (REG) pmul_r<T, R, C>(A, t, I.dst, I.a, I.src, (I.flags & 16u) == 0); \
    else pmul_u<T, R, C>(A, I.dst, I.a, I.src); \
    break;
#define QIW_H_PMUL(H, R, C) \
  case H:                   \
    pmul_u<T, R, C>(A, I.dst, I.a, I.src); \
    break;
#define QIW_H_PMULD(H, R, C) \
  case H:                    \
    pmuld_u<T, R, C>(A, I.dst, I.a, I.src); \
    break;
#define QIW_H_OMUL(H, R, K, C, MODE, XR) \
  case H:                                 \
    omul_m<T, R, K, C, MODE, XR && REG>(A, O, I.dst, I.a, I.src, MODE ? edge_coef<T>(I, A) : (T)1, accf, t); \
    break;
#define QIW_H_OMULRC(H, R, K, C) QIW_H_OMUL(H, R, K, C, 1, true)
#define QIW_H_OMULR1(H, R, K, C) QIW_H_OMUL(H, R, K, C, 0, true)
#define QIW_H_OMULC(H, R, K, C) QIW_H_OMUL(H, R, K, C, 1, false)
#define QIW_H_OMUL1(H, R, K, C) QIW_H_OMUL(H, R, K, C, 0, false)
    QIW_RC9(QIW_H_PMULR, kHPmulReg)
    QIW_RC9(QIW_H_PMUL, kHPmul)
    QIW_RC9(QIW_H_PMULD, kHPmulD)
    QIW_RKC27(QIW_H_OMULRC, kHOmulRegC)
    QIW_RKC27(QIW_H_OMULR1, kHOmulReg1)
    QIW_RKC27(QIW_H_OMULC, kHOmulC)
    QIW_RKC27(QIW_H_OMUL1, kHOmul1)
#undef QIW_H_PMULR
#undef QIW_H_PMUL
#undef QIW_H_PMULD
#undef QIW_H_OMUL
#undef QIW_H_OMULRC
#undef QIW_H_OMULR1
#undef QIW_H_OMULC
#undef QIW_H_OMUL1
#define QIW_H_AXPY(H, N, XR)                                                                   \
  case H:                                                                                      \
    axpy_u<T, N, XR && REG>(A, I.dst, I.src, edge_coef<T>(I, A), accf, (I.w >= 0) || has_c(I), t); \
    break;
    QIW_H_AXPY(kHAxpyReg + 0, 1, true) QIW_H_AXPY(kHAxpyReg + 1, 2, true) QIW_H_AXPY(kHAxpyReg + 2, 4, true)
    QIW_H_AXPY(kHAxpyReg + 3, 8, true) QIW_H_AXPY(kHAxpyReg + 4, 16, true)
    QIW_H_AXPY(kHAxpy + 0, 1, false) QIW_H_AXPY(kHAxpy + 1, 2, false) QIW_H_AXPY(kHAxpy + 2, 4, false)
    QIW_H_AXPY(kHAxpy + 3, 8, false) QIW_H_AXPY(kHAxpy + 4, 16, false)
#undef QIW_H_AXPY
    default:
      break;
  }
}
#undef QIW_RC9
#undef QIW_RKC27

// LARGE: the instantiation for problems with large sector blocks (the largest arena class, e.g.
// t2g's 9 x 9 blocks), whose products take the 3-row register blocking; the others keep products
// of dims 1, 2, 4 in registers.  Both only in the FP32 kernels: the FP64 kernels are DFMA-bound
// and at the register budget of their launch bound, so they ignore flag bits 2-4 and keep
// every product in the arena.  (One register budget cannot hold both paths without spills.)
template <typename T, int RESMAX, bool LARGE>
__device__ __forceinline__ void exec_instr(const Instr &I, T *A, const T *O, double *R, T (&t)[kRegTmp],
                                           float *tcx) {
  constexpr bool REG = QIW_REG_PRODUCTS && (sizeof(T) == 4 || QIW_REG_PRODUCTS_FP64) && !LARGE;
  constexpr bool BLOCK3 = QIW_BLOCK3 && sizeof(T) == 4 && LARGE;
  if constexpr (QIW_FLAT_DISPATCH) {
    if (I.handler) {   // blocks of dims 1, 2, 4: the decoded cases below are the rest
      exec_flat<T, REG>(I, A, O, t);
      return;
    }
  }
  constexpr bool DECODE_SMALL = !QIW_FLAT_DISPATCH;   // the small-block cases, when not dispatched flat
  const int rows = I.rows, cols = I.cols;
  switch (I.op) {
    case OP_LOADP: {  // c == 1 copies (x * 1 is exact)
      const T c = coef_c<T>(I);
      const bool hc = has_c(I);
      if (I.inner) {
#pragma unroll 1
        for (int j = 0; j < rows; ++j)
#pragma unroll 1
          for (int r = 0; r < rows; ++r)
            A[I.dst + j * rows + r] = (r == j) ? (hc ? c * A[I.a + r] : A[I.a + r]) : (T)0;
      } else {
#pragma unroll 1
        for (int e = 0; e < rows * rows; ++e) A[I.dst + e] = hc ? c * A[I.a + e] : A[I.a + e];
      }
      break;
    }
    case OP_LOADI: {  // c * identity
      const T c = coef_c<T>(I);
#pragma unroll 1
      for (int j = 0; j < rows; ++j)
#pragma unroll 1
        for (int r = 0; r < rows; ++r) A[I.dst + j * rows + r] = (r == j) ? c : (T)0;
      break;
    }
    case OP_LOADC: {
      const T c = coef_c<T>(I);
      const bool hc = has_c(I);
#pragma unroll 1
      for (int e = 0; e < rows * cols; ++e) A[I.dst + e] = hc ? c * __ldg(O + I.a + e) : __ldg(O + I.a + e);
      break;
    }
    case OP_PMUL: {
      const int cr = dcode(rows), cc = dcode(cols);
      if (DECODE_SMALL && REG && (I.flags & 8u)) {   // dims 1, 2, 4 by construction (planner)
        if constexpr (DECODE_SMALL) {
          const int code = cr * 3 + cc;
          const bool store = (I.flags & 16u) == 0;
          QIW_D2(pmul_r, A, t, I.dst, I.a, I.src, store)
        }
      } else if (DECODE_SMALL && cr >= 0 && cc >= 0) {
        if constexpr (DECODE_SMALL) {
          const int code = cr * 3 + cc;
          QIW_D2(pmul_u, A, I.dst, I.a, I.src)
        }
      } else if (BLOCK3 && rows % 3 == 0 && rows <= 9) {
        mul_rows3<T, false>(A, O, I.dst, I.a, I.src, rows, rows, cols, (T)1, false, false);
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
      if (DECODE_SMALL && cr >= 0 && cc >= 0) {
        if constexpr (DECODE_SMALL) {
          const int code = cr * 3 + cc;
          QIW_D2(pmuld_u, A, I.dst, I.a, I.src)
        }
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
      const bool has_coef = (I.w >= 0) || has_c(I);
      const T coef = edge_coef<T>(I, A);
      const int cr = dcode(rows), ck = dcode(inner), cc = dcode(cols);
      if (DECODE_SMALL && REG && (I.flags & 4u)) {   // source in registers: dims 1, 2, 4 by construction (planner)
        if constexpr (DECODE_SMALL) {
          const int code = cr * 9 + ck * 3 + cc;
          QIW_D3(omul_ur, A, O, I.dst, I.a, I.src, coef, I.acc != 0, has_coef, t)
        }
      } else if (DECODE_SMALL && cr >= 0 && ck >= 0 && cc >= 0) {
        if constexpr (DECODE_SMALL) {
          const int code = cr * 9 + ck * 3 + cc;
          QIW_D3(omul_u, A, O, I.dst, I.a, I.src, coef, I.acc != 0, has_coef, t)
        }
      } else if (BLOCK3 && tcx && inner == kTcK && rows <= 16 && cols <= kTcMaxCols) {
        if constexpr (BLOCK3) omul_tc(A, O, tcx, I.dst, I.a, I.src, rows, cols, coef, I.acc != 0);
      } else if (BLOCK3 && rows % 3 == 0 && inner <= 9 && !(I.acc && I.dst == I.src)) {
        mul_rows3<T, true>(A, O, I.dst, I.a, I.src, rows, inner, cols, coef, true, I.acc != 0);
      } else {
#pragma unroll 1
        for (int j = 0; j < cols; ++j)
#pragma unroll 1
          for (int r = 0; r < rows; ++r) {
            T acc = (T)0;
#pragma unroll 4
            for (int k = 0; k < inner; ++k) acc = fmaT<T>(__ldg(O + I.a + k * rows + r), A[I.src + j * inner + k], acc);
            const int o = I.dst + j * rows + r;
            A[o] = fmaT<T>(coef, acc, I.acc ? A[o] : (T)0);   // fma(c, a, 0) = c * a
          }
      }
      break;
    }
    case OP_AXPY: {
      const bool has_coef = (I.w >= 0) || has_c(I);
      const T coef = edge_coef<T>(I, A);
      const int n = rows * cols;
      const bool accf = I.acc != 0;
      if (DECODE_SMALL && REG && (I.flags & 4u)) {   // source in registers (n in 1, 2, 4, 8, 16 by construction)
        if constexpr (DECODE_SMALL) switch (n) {
          case 1: axpy_u<T, 1, true>(A, I.dst, I.src, coef, accf, has_coef, t); break;
          case 2: axpy_u<T, 2, true>(A, I.dst, I.src, coef, accf, has_coef, t); break;
          case 4: axpy_u<T, 4, true>(A, I.dst, I.src, coef, accf, has_coef, t); break;
          case 8: axpy_u<T, 8, true>(A, I.dst, I.src, coef, accf, has_coef, t); break;
          default: axpy_u<T, 16, true>(A, I.dst, I.src, coef, accf, has_coef, t); break;
        }
        break;
      }
      if constexpr (DECODE_SMALL) {
        switch (n) {
          case 1: axpy_u<T, 1, false>(A, I.dst, I.src, coef, accf, has_coef, t); break;
          case 2: axpy_u<T, 2, false>(A, I.dst, I.src, coef, accf, has_coef, t); break;
          case 4: axpy_u<T, 4, false>(A, I.dst, I.src, coef, accf, has_coef, t); break;
          case 8: axpy_u<T, 8, false>(A, I.dst, I.src, coef, accf, has_coef, t); break;
          case 16: axpy_u<T, 16, false>(A, I.dst, I.src, coef, accf, has_coef, t); break;
          default:
#pragma unroll 1
            for (int e = 0; e < n; ++e) {
              const int o = I.dst + e;
              A[o] = accf ? fmaT<T>(coef, A[I.src + e], A[o]) : coef * A[I.src + e];
            }
        }
      } else {   // sizes other than 1, 2, 4, 8, 16 (the others are dispatched flat)
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
// warped points / per-sample output of qiw_integrate_warped / qiw_integrate_samples.  The
// single-problem kernel passes its DevWork (same field names) straight from global memory.
struct TileSrc {
  double t_i, t_w, t_f;
  uint64_t first_index, n_samples;
  const uint32_t *m, *x0;
  const double *pts;
  double *sample_out;
};

// One tile: blockDim.x samples [s0, s0 + blockDim.x) of batch `batch` of group g, reduced to
// the CTA's partial sums at partial_row()[0 .. res_size).  Every thread of the CTA must call it.
// EXTRAS compiles in the warped points and the per-sample output (qiw_integrate_warped /
// qiw_integrate_samples); the plain kernels are built without them (fewer live registers).
// Per-sample setup of one tile slot: Sobol point (or warped point), domain map, the i*P blocks
// of the intervals the program uses and the i*Delta weights, into the sample's arena A.
// `active` is cleared for samples a domain map discards; `wt` collects per-sample weights.
template <typename T, bool EXTRAS, typename Src>
__device__ __forceinline__ void sample_setup(const DevProblem &pb, const DevGroup &g, const Src &w,
                                             uint64_t sidx, T *__restrict__ A, double &wt, bool &active) {
    double tm[kMaxNodes];
    const double tsel[3] = {w.t_i, w.t_w, w.t_f};
#pragma unroll 1
    for (int f = 0; f < g.n_fixed; ++f) tm[g.fixed_pos[f]] = tsel[g.fixed_time[f]];
    const int D = g.D;
    if (D > 0) {
      const uint64_t n = w.first_index + sidx;
      const uint32_t gray = (uint32_t)(n ^ (n >> 1));
      double u[kMaxDim];
      if (EXTRAS && w.pts) {  // warped point x = w(y) of a learned change of variables, weight 1/q(x)
        const double *pp = w.pts + sidx * (uint64_t)(D + 1);
#pragma unroll 1
        for (int d = 0; d < D; ++d) u[d] = pp[d];
        wt = pp[D];
      } else {
#pragma unroll 1
        for (int d = 0; d < D; ++d)
          u[d] = ldexp((double)sobol_coord(w.m + d * 32, __ldg(w.x0 + d), gray), -32);  // exact: ldexp(Float64(x), -32)
      }
      bool mapped = false;  // the alternative maps of bare groups live in the extras kernel
      if constexpr (EXTRAS) {
        if (g.kind == QIW_GROUP_BARE && w.transform == QIW_TRANSFORM_SORT) {  // SortTransform (src/qmc_integrate.jl:319-321)
          const double u_diff = w.t_f - w.t_i;
#pragma unroll 1
          for (int i = 1; i < D; ++i)  // insertion sort, descending
#pragma unroll 1
            for (int j = i; j > 0 && u[j] > u[j - 1]; --j) {
              const double t = u[j];
              u[j] = u[j - 1];
              u[j - 1] = t;
            }
#pragma unroll 1
          for (int i = 0; i < D; ++i) u[i] = w.t_i + u[i] * u_diff;
          mapped = true;
        } else if (g.kind == QIW_GROUP_BARE && w.transform == QIW_TRANSFORM_EXPMODEL) {
          // ExpModelFunctionTransform (src/qmc_integrate.jl:138-164): per-sample Jacobian
          // tau^d / exp(-(u_f - u_d) / tau); samples below the contour start are discarded
          const double tau = w.decay;
          u[0] = w.t_f + tau * log(1.0 - u[0]);
#pragma unroll 1
          for (int i = 1; i < D; ++i) u[i] = u[i - 1] + tau * log(1.0 - u[i]);
          if (u[D - 1] < 0.0) active = false;
          wt *= pow(tau, (double)D) / exp(-(w.t_f - u[D - 1]) / tau);
          mapped = true;
        }
      }
      if (mapped) {
      } else if (g.kind == QIW_GROUP_BARE || g.kind == QIW_GROUP_SIGMA) {  // RootTransform over [t_i, t_f]
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

  }

template <typename T, int ARENA, int RESMAX, bool EXTRAS, typename Src, typename RowFn>
__device__ __forceinline__ void eval_tile(const DevProblem &pb, const DevGroup &g, const Src &w, int batch,
                                          uint64_t s0, RowFn partial_row) {
  const int res_size = g.res_size;
  const uint64_t sidx = s0 + threadIdx.x;
  bool active = sidx < w.n_samples;   // cleared for samples a domain map discards
  double wt = 1.0;
  T A[ARENA];
  // this warp's tensor-core staging area (FP32 large-block kernels, opt-in), else null
  float *tcx = (sizeof(T) == 4 && ARENA >= kArenaHuge && pb.tc_stage > 0)
                   ? reinterpret_cast<float *>(qiw_dyn_smem + pb.tc_stage) + (threadIdx.x >> 5) * kTcWarpFloats
                   : nullptr;
  T tr[kRegTmp];   // register copy of the last P multiply's product (flag bits 2-4)
#pragma unroll
  for (int i = 0; i < kRegTmp; ++i) tr[i] = (T)0;
  double R[RESMAX];
#pragma unroll 1
  for (int e = 0; e < res_size; ++e) R[e] = 0.0;
  if (active) sample_setup<T, EXTRAS>(pb, g, w, sidx, A, wt, active);

  // The group's program: the instructions of this CTA's batch.  Scalar programs (all blocks
  // 1x1) stream them through shared memory in chunks of blockDim.x: each thread copies one
  // 32-byte instruction of the next chunk with cp.async while the current chunk executes (the
  // streams are MBs, far beyond L1, and every thread reads every instruction); the waits are
  // cp.async.wait_group and CTA barriers.  Other programs spend thousands of cycles per
  // instruction and read them directly.
  {
    const T *O = reinterpret_cast<const T *>(pb.opv);
    const int i0 = __ldg(g.batch_begin + batch), i1 = __ldg(g.batch_begin + batch + 1);
    const Instr *ins = sizeof(T) == 4 ? g.ins32 : g.ins;
    if (g.scalar) {  // the launch provides the staging buffers for every scalar group
      const int ch = blockDim.x;
      Instr *const ibuf = reinterpret_cast<Instr *>(qiw_dyn_smem + (size_t)((blockDim.x + 31) >> 5) * RESMAX * sizeof(double));
      stage_instr(ibuf, ins, i0, i1);
      cp_async_commit();
      int b = 0;
#pragma unroll 1
      for (int base = i0; base < i1; base += ch, b ^= 1) {
        if (base + ch < i1) stage_instr(ibuf + (b ^ 1) * ch, ins, base + ch, i1);
        cp_async_commit();
        cp_async_wait_1();   // this thread's copies of the current chunk have landed
        __syncthreads();     // and everyone's
        const int n = min(ch, i1 - base);
        if (active) {
#pragma unroll 1
          for (int k = 0; k < n; ++k) {
            const Instr I = ibuf[b * ch + k];
            exec_scalar<T>(I, A, O, R);
          }
        }
        __syncthreads();     // the buffer is refilled two chunks later
      }
      cp_async_wait_0();
    } else if (active || tcx) {   // with tensor-core multiplies every lane runs the program
#if QIW_PREFETCH_INSTR
      // the next instruction's load is in flight while the current one executes (FP32 eg step
      // 15.4 -> 15.0 ms, t2g 149 -> 105 ms at 2048 samples, FP64 unchanged)
      Instr nx = i0 < i1 ? load_instr(ins + i0) : Instr{};
#pragma unroll 1
      for (int ip = i0; ip < i1; ++ip) {
        const Instr I = nx;
        if (ip + 1 < i1) nx = load_instr(ins + ip + 1);
        exec_instr<T, RESMAX, (ARENA >= kArenaHuge)>(I, A, O, R, tr, tcx);
      }
#else
#pragma unroll 1
      for (int ip = i0; ip < i1; ++ip) {
        const Instr I = load_instr(ins + ip);
        exec_instr<T, RESMAX, (ARENA >= kArenaHuge)>(I, A, O, R, tr, tcx);
      }
#endif
      if (!active) {   // a lane without a sample ran the program on an unset arena: no result
#pragma unroll 1
        for (int e = 0; e < res_size; ++e) R[e] = 0.0;
      }
    }
  }
  if (active) {
    if (EXTRAS && wt != 1.0) {  // warp weight 1/q(x) and / or the ExpModel Jacobian
#pragma unroll 1
      for (int e = 0; e < res_size; ++e) R[e] *= wt;
    }
    if (EXTRAS && w.sample_out) {  // per-sample values (batches of one sample add up)
#pragma unroll 1
      for (int e = 0; e < res_size; ++e) atomicAdd(w.sample_out + sidx * (uint64_t)res_size + e, R[e]);
    }
  }

  // Deterministic CTA reduction of R -> prow[0 .. res_size).
  double(*red)[RESMAX] = reinterpret_cast<double(*)[RESMAX]>(qiw_dyn_smem);
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
  double *prow = partial_row();  // formed only now: nothing holds it across the tile
#pragma unroll 1
  for (int e = threadIdx.x; e < res_size; e += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < n_warps; ++k) s += red[k][e];
    prow[e] = s;
  }
}

// MINB: resident 128-thread blocks per SM the registers are sized for (the launch bound).
template <typename T, int ARENA, int RESMAX, bool EXTRAS, int MINB = (sizeof(T) == 4 ? kMinBlocks32 : kMinBlocks)>
__global__ void __launch_bounds__(kMaxThreads, MINB)
    eval_kernel(DevProblem pb, const DevGroup *__restrict__ groups, const DevWork *__restrict__ works,
                const int4 *__restrict__ cta_map, double *__restrict__ partials) {
  const int4 cm = cta_map[blockIdx.x];   // (work item, batch, first sample of the tile, partial row)
  const DevWork &w = works[cm.x];
  const DevGroup &g = groups[w.group];
  eval_tile<T, ARENA, RESMAX, EXTRAS>(pb, g, w, cm.y, (uint64_t)cm.z,
                              [=]() { return partials + (size_t)cm.w * g.res_size; });
}

}  // namespace qiw
