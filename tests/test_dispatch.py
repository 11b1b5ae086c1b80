"""The flat dispatch index of the evaluation kernels (csrc/qiw_dispatch.hpp, computed on upload):
every instruction with blocks of dims 1, 2, 4 gets an index in the range of its opcode, block
shape, coefficient mode and operand source, distinct combinations get distinct indices, and
everything else gets 0 (decoded in the kernel).  Host code only: compiled with g++ here."""
import os
import shutil
import subprocess
import tempfile

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "qinchworm.jl_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <map>
#include <tuple>
#include "qiw_dispatch.hpp"
using namespace qiw;
static int fails = 0;
#define CHECK(c) do { if (!(c)) { std::printf("fail line %d\n", __LINE__); ++fails; } } while (0)
int main() {
  const int dims[] = {1, 2, 3, 4, 8, 9};
  std::map<int, std::tuple<int, int, int, int, int, int>> seen;   // handler -> (op, r, k, c, coef, src)
  for (int op : {OP_LOADP, OP_LOADC, OP_PMUL, OP_PMULD, OP_OMUL, OP_AXPY, OP_LEAF, OP_LOADI, OP_PMAXPY})
    for (int r : dims) for (int k : dims) for (int c : dims)
      for (int w : {-1, 5}) for (int fl = 0; fl < 32; ++fl) for (int reg = 0; reg < 2; ++reg) {
        Instr I{};
        I.op = (uint8_t)op; I.rows = (uint8_t)r; I.inner = (uint8_t)k; I.cols = (uint8_t)c;
        I.flags = (uint8_t)fl; I.w = w;
        const int h = handler_of(I, reg != 0);
        CHECK(h >= 0 && h < kHandlers);
        const bool small = small_code(r) >= 0 && small_code(c) >= 0;
        const bool coef = w >= 0 || (fl & 1);
        const bool src_reg = reg && (fl & 4);
        int src = 0;
        switch (op) {
          case OP_PMUL:
            if (!small) { CHECK(h == 0); break; }
            CHECK(h == (reg && (fl & 8) ? kHPmulReg : kHPmul) + small_code(r) * 3 + small_code(c));
            src = reg && (fl & 8);
            break;
          case OP_PMULD:
            CHECK(h == (small ? kHPmulD + small_code(r) * 3 + small_code(c) : 0));
            break;
          case OP_OMUL: {
            if (!small || small_code(k) < 0) { CHECK(h == 0); break; }
            const int base = src_reg ? (coef ? kHOmulRegC : kHOmulReg1) : (coef ? kHOmulC : kHOmul1);
            CHECK(h == base + small_code(r) * 9 + small_code(k) * 3 + small_code(c));
            src = src_reg;
            break;
          }
          case OP_AXPY: {
            const int n = pow2_code(r * c);
            if (n < 0) { CHECK(h == 0); break; }
            CHECK(h == (src_reg ? kHAxpyReg : kHAxpy) + n);
            src = src_reg;
            break;
          }
          default:
            CHECK(h == 0);
        }
        if (h == 0) continue;
        // one index, one routine: opcode, shape, coefficient mode (OMUL) and source agree
        const int key_k = op == OP_OMUL ? k : 0, key_coef = op == OP_OMUL ? coef : 0;
        const int kr = op == OP_AXPY ? r * c : r, kc = op == OP_AXPY ? 0 : c;
        auto key = std::make_tuple(op, kr, key_k, kc, key_coef, src);
        auto it = seen.find(h);
        if (it == seen.end()) seen[h] = key; else CHECK(it->second == key);
      }
  CHECK((int)seen.size() == kHandlers - 1);   // every index of the table is reachable
  std::printf("%d handlers, %d failures\n", (int)seen.size(), fails);
  return fails != 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_dispatch_index_ranges_and_uniqueness():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "dispatch_check.cpp")
        exe = os.path.join(d, "dispatch_check")
        with open(src, "w") as f:
            f.write(PROGRAM)
        subprocess.run(["g++", "-std=c++17", "-O1", "-I", CSRC, src, "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "145 handlers, 0 failures" in r.stdout
