// Flat dispatch index of an instruction (Instr::handler), computed on upload.
//
// The evaluation kernels of small-block programs (sector dimensions 1, 2, 4; not the
// large-block instantiation) jump once on this index to the instance of the matrix routine for
// the instruction's opcode, block shape, coefficient mode and operand source, instead of
// decoding opcode, dimensions and flags per instruction.  Index 0 means "decode the fields" (the
// generic loops and everything the table does not cover); the large-block kernels always decode.
#pragma once
#include <cstdint>

#include "qiw_internal.hpp"

// Register-held P products (FP32 small-block kernels; FP64 opt-in), shared by the kernels and
// the upload step that computes the dispatch index.
#ifndef QIW_REG_PRODUCTS
#define QIW_REG_PRODUCTS 1
#endif
#ifndef QIW_REG_PRODUCTS_FP64
#define QIW_REG_PRODUCTS_FP64 0
#endif
#ifndef QIW_FLAT_DISPATCH
#define QIW_FLAT_DISPATCH 1
#endif

namespace qiw {

constexpr int kHPmulReg = 1;      // + rc (9): P multiply kept in registers (flag bit 3)
constexpr int kHPmul = 10;        // + rc (9): P multiply through the arena
constexpr int kHPmulD = 19;       // + rc (9): diagonal P multiply
constexpr int kHOmulRegC = 28;    // + rkc (27): operator multiply, source in registers, with coefficient
constexpr int kHOmulReg1 = 55;    // + rkc (27): the same without coefficient
constexpr int kHOmulC = 82;       // + rkc (27): operator multiply, source in the arena, with coefficient
constexpr int kHOmul1 = 109;      // + rkc (27): the same without coefficient
constexpr int kHAxpyReg = 136;    // + log2(n) (5): axpy, source in registers
constexpr int kHAxpy = 141;       // + log2(n) (5): axpy, source in the arena
constexpr int kHandlers = 146;
static_assert(kHPmul == kHPmulReg + 9 && kHPmulD == kHPmul + 9 && kHOmulRegC == kHPmulD + 9 &&
                  kHOmulReg1 == kHOmulRegC + 27 && kHOmulC == kHOmulReg1 + 27 && kHOmul1 == kHOmulC + 27 &&
                  kHAxpyReg == kHOmul1 + 27 && kHAxpy == kHAxpyReg + 5 && kHandlers == kHAxpy + 5,
              "dispatch ranges are contiguous and disjoint");
static_assert(kHandlers <= 256, "the dispatch index is one byte");

inline int small_code(int d) { return d == 1 ? 0 : d == 2 ? 1 : d == 4 ? 2 : -1; }
inline int pow2_code(int n) { return n == 1 ? 0 : n == 2 ? 1 : n == 4 ? 2 : n == 8 ? 3 : n == 16 ? 4 : -1; }

// reg: the kernels that run this copy keep P products in registers (flag bits 2-4 honoured).
inline uint8_t handler_of(const Instr &I, bool reg) {
  const int r = small_code(I.rows), k = small_code(I.inner), c = small_code(I.cols);
  const bool has_coef = I.w >= 0 || (I.flags & 1u);
  switch (I.op) {
    case OP_PMUL:
      if (r < 0 || c < 0) return 0;
      return (uint8_t)((reg && (I.flags & 8u) ? kHPmulReg : kHPmul) + r * 3 + c);
    case OP_PMULD:
      if (r < 0 || c < 0) return 0;
      return (uint8_t)(kHPmulD + r * 3 + c);
    case OP_OMUL: {
      if (r < 0 || k < 0 || c < 0) return 0;
      const int rkc = r * 9 + k * 3 + c;
      if (reg && (I.flags & 4u)) return (uint8_t)((has_coef ? kHOmulRegC : kHOmulReg1) + rkc);
      return (uint8_t)((has_coef ? kHOmulC : kHOmul1) + rkc);
    }
    case OP_AXPY: {
      const int n = pow2_code(I.rows * I.cols);
      if (n < 0) return 0;
      return (uint8_t)((reg && (I.flags & 4u) ? kHAxpyReg : kHAxpy) + n);
    }
    default:
      return 0;
  }
}

}  // namespace qiw
