// Internal data structures shared by the host planner and the CUDA kernels.
#pragma once
#include <cstdint>

namespace qiw {

// Limits of the device program representation.
constexpr int kMaxNodes = 32;    // configuration positions (2*order + fixed nodes)
constexpr int kMaxDim = 32;      // Sobol dimensions per sample (2*order)
constexpr int kMaxFixed = 4;

// Instruction opcodes of the per-sample program.  Every thread (one qMC sample) runs
// the same stream; matrices live in the thread's arena, column-major.
enum Opcode : uint8_t {
  OP_LOADP = 1,   // dst[rows x rows] = c * Pm[a]                         (root with identity)
  OP_LOADC = 2,   // dst[rows x cols] = c * O[a]                          (root with an operator)
  OP_PMUL = 3,    // dst[rows x cols] = Pm[a] (rows x rows) * src[rows x cols]
  OP_PMULD = 4,   // dst[rows x cols] = diag(Pm[a]) * src                 (exact atomic P0)
  OP_OMUL = 5,    // dst (=|+=) c*w * O[a] (rows x inner) * src[inner x cols]
  OP_AXPY = 6,    // dst (=|+=) c*w * src    (rows*cols elements)
  OP_LEAF = 7,    // R[a ...] += src         (rows*cols elements)
  OP_LOADI = 8,   // dst[rows x rows] = c * identity      (root before a zero-length interval)
  OP_PMAXPY = 9,  // 1x1 programs only: dst (=|+=) c*w * (Pm[a] * src)  (a P multiply fused into its one AXPY)
};

struct alignas(16) Instr {     // 32 bytes
  uint8_t op, rows, inner, cols;
  uint8_t acc;                 // 1: accumulate into dst, 0: overwrite
  uint8_t flags;               // bit 0: c != 1, bit 1: c == -1 (set on upload; the kernels test no doubles)
  uint8_t handler;             // flat dispatch index of the kernels (0: decode the fields), set on upload
  uint8_t pad2;
  int32_t dst;                 // arena offset (elements)
  int32_t src;                 // arena offset (elements)
  int32_t a;                   // Pm offset (arena) / operator value offset / result offset
  int32_t w;                   // weight slot offset in the arena, -1: none
  double c;                    // constant coefficient
};
static_assert(sizeof(Instr) == 32, "Instr layout");

// Per-sample propagator evaluation jobs: Pm[iv][s] = i*P_s(t_{iv+1} - t_iv).
struct PmJob {
  int16_t iv, s;
  int32_t off;                 // arena offset
};

// Per-sample hybridisation weights: W = i*Delta_p(t_tail - t_head).
struct WJob {
  int16_t head, tail;
  int16_t pair;
  int16_t pad;
  int32_t off;
};

enum TimeSel : int32_t { T_I = 0, T_W = 1, T_F = 2 };

struct DevGroup {
  int32_t kind, order, n_nodes, D;
  int32_t d_before, d_after;
  int32_t use_bold;
  int32_t n_fixed;
  int32_t fixed_pos[kMaxFixed];
  int32_t fixed_time[kMaxFixed];
  int32_t var_pos[kMaxDim];
  int32_t n_pm, n_w, n_instr;
  int32_t arena;               // elements of the compute type
  int32_t res_size;            // sum d^2 (result elements)
  int32_t n_batches;           // independent instruction ranges (one per initial sector or split)
  int32_t scalar;              // 1: every block of the program is 1x1 (scalar executor, staged stream)
  int32_t pad_g;
  const PmJob *pm;
  const WJob *wj;
  const Instr *ins;
  const Instr *ins32;          // the same program with c rounded to float in the low 4 bytes of c
  const int32_t *batch_begin;  // [n_batches + 1]
};

struct DevWork {
  int32_t group;
  int32_t n_cta;
  double t_i, t_w, t_f;
  double scale;                // J / N_total (contour Jacobian and 1/N)
  uint64_t first_index;
  uint64_t n_samples;
  const uint32_t *m;           // [D][32]
  const uint32_t *x0;          // [D]
  const double *pts;           // optional [n_samples][D + 1]: warped points x and weights 1/q(x)
  double *sample_out;          // optional [n_samples][res_size]: per-sample integrand values
  int32_t transform;           // QIW_TRANSFORM_* of a bare group (SORT, EXPMODEL: extras kernel)
  int32_t pad_w;
  double decay;                // EXPMODEL decay rate
};

// Device view of the problem data.  Tables hold i*P and i*Delta (real in the
// real-phase kernel: T = double/float, complex otherwise).
struct DevProblem {
  int32_t S, n_tau, n_pairs;
  int32_t tc_stage;            // > 0: byte offset of the tensor-core staging area in dynamic shared memory (FP32 large blocks)
  double h, inv_h, beta;
  const int32_t *dims;
  const int32_t *ptab_off;     // [S] offset of sector s in the P table (elements)
  const int32_t *eoff;         // [S] offset into atomic energies
  const int32_t *res_off;      // [S] offset of sector s in the result vector
  const double *E;             // atomic energies (E + lambda)
  const void *P;               // i*P table: sector s at ptab_off[s]: [n_tau][d][d] col-major
  const void *opv;             // operator values (compute type), column-major blocks
  const void *delta;           // i*Delta per pair: linear [n_tau]; cubic [n_tau-1][4]
  const int32_t *delta_kind;   // [n_pairs]
  const int32_t *delta_off;    // [n_pairs]
};

}  // namespace qiw
