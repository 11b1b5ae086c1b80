// Learned change of variables on the qMC hypercube of a topology group.
//
// A warp w maps a Sobol point y in [0,1]^D to x = w(y) in [0,1]^D with a triangular
// (autoregressive) monotone map: in dimension d the density of x_d given x_<d is continuous
// and piecewise linear on K equal bins, q_d(x) = v_b + (v_{b+1} - v_b) t (t the position in
// bin b), with knot heights v = (1 - a) e^l / S + a normalised to unit integral (S) and mixed
// with the uniform density (a), logits l = l_d(x_<d) from a masked MLP (MADE: D inputs, 3
// hidden layers of 64 tanh units, D*(K+1) outputs; output d sees inputs < d only).  The CDF
// is quadratic per bin and is inverted in closed form.  q(x) = prod_d q_d, so the estimator
// (1/N) sum_i f(u(x_i)) J / q(x_i) is unbiased for every set of weights; because q is
// continuous the warped integrand stays continuous, which keeps quasi-Monte Carlo effective; the
// smooth activation keeps the conditioner l_d(x_<d) smooth as well (ReLU units would add kinks
// along oblique hyperplanes of x_<d, which qMC points resolve poorly).  Training
// minimises the |f|-weighted negative log-likelihood -sum_i w_i log q(x_i) of samples x_i
// produced by plain qMC (w_i = |f(x_i)|), i.e. fits q to |f|.  Weights are stored in BF16
// (FP32 master copy for Adam); all arithmetic accumulates in FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "qiw_ctx.hpp"

namespace qiw {
namespace {

constexpr int WH = 64;         // hidden width
constexpr int WK = 16;         // bins per dimension
constexpr int WKP = WK + 1;    // knot heights (outputs) per dimension
constexpr int WDMAX = 8;       // max dimensions (order <= 4)
constexpr int WTILE = 64;      // samples per training block
constexpr float WALPHA_DEFAULT = 0.3f;  // uniform mixing of the density (default)

// parameter layout: W1[H][D] b1[H] W2[H][H] b2[H] W3[H][H] b3[H] W4[DK][H] b4[DK]
struct Layout {
  int D, DK, oW1, ob1, oW2, ob2, oW3, ob3, oW4, ob4, n;
  __host__ __device__ explicit Layout(int d) : D(d), DK(d * WKP) {
    int o = 0;
    oW1 = o; o += WH * D; ob1 = o; o += WH;
    oW2 = o; o += WH * WH; ob2 = o; o += WH;
    oW3 = o; o += WH * WH; ob3 = o; o += WH;
    oW4 = o; o += DK * WH; ob4 = o; o += DK;
    n = o;
  }
};

__device__ __forceinline__ float act(float x) { return tanhf(x); }

// ---------------------------------------------------------------------------------------
// Tensor-core GEMM tiles (mma.sync m16n8k16, BF16 operands, FP32 accumulate).
//
// The weights are BF16 numbers, so a weight operand is exact in BF16.  Activations and
// gradients are FP32: they enter as a two-term BF16 split x = hi + lo (hi = bf16(x),
// lo = bf16(x - hi), about 16 significant bits), so a product with a weight operand is
// A_hi*W + A_lo*W and a product of two FP32 operands is A_hi*B_hi + A_hi*B_lo + A_lo*B_hi.
// Accumulation is FP32 throughout; every sum over samples runs in a fixed order.

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);   // .x (low half) = a
  return *reinterpret_cast<uint32_t *>(&h);
}

// (hi, lo) BF16 pairs of two FP32 values.
__device__ __forceinline__ void split_bf16(float a, float b, uint32_t &hi, uint32_t &lo) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
  hi = *reinterpret_cast<uint32_t *>(&h);
  lo = *reinterpret_cast<uint32_t *>(&l);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One warp: C[16][8*NT] += A[16][16*kt] * B[16*kt][8*NT] over k tiles kt = 0 .. KT-1.
// fa(r, k) gives A (FP32), fb(k, n) gives B; B_EXACT: B is BF16-exact (2 products per tile),
// otherwise it is split as well (3 products).  Fragment layouts of m16n8k16 (PTX ISA): lane
// l = 4g + t holds A rows g, g+8 at columns 2t, 2t+1, 2t+8, 2t+9; B columns n = g at rows 2t,
// 2t+1, 2t+8, 2t+9; C rows g, g+8 at columns 2t, 2t+1.
template <int NT, bool B_EXACT, typename FA, typename FB>
__device__ __forceinline__ void warp_gemm(float (&c)[NT][4], int KT, FA fa, FB fb) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll 1
  for (int kt = 0; kt < KT; ++kt) {
    const int k0 = 16 * kt + 2 * t;
    uint32_t ah[4], al[4];
    split_bf16(fa(g, k0), fa(g, k0 + 1), ah[0], al[0]);
    split_bf16(fa(g + 8, k0), fa(g + 8, k0 + 1), ah[1], al[1]);
    split_bf16(fa(g, k0 + 8), fa(g, k0 + 9), ah[2], al[2]);
    split_bf16(fa(g + 8, k0 + 8), fa(g + 8, k0 + 9), ah[3], al[3]);
#pragma unroll
    for (int j = 0; j < NT; ++j) {
      const int n = 8 * j + g;
      if (B_EXACT) {
        const uint32_t b0 = pack_bf16(fb(k0, n), fb(k0 + 1, n)), b1 = pack_bf16(fb(k0 + 8, n), fb(k0 + 9, n));
        mma_bf16(c[j], ah, b0, b1);
        mma_bf16(c[j], al, b0, b1);
      } else {
        uint32_t bh0, bl0, bh1, bl1;
        split_bf16(fb(k0, n), fb(k0 + 1, n), bh0, bl0);
        split_bf16(fb(k0 + 8, n), fb(k0 + 9, n), bh1, bl1);
        mma_bf16(c[j], ah, bh0, bh1);
        mma_bf16(c[j], ah, bl0, bl1);
        mma_bf16(c[j], al, bh0, bh1);
      }
    }
  }
}

template <int NT>
__device__ __forceinline__ void zero_acc(float (&c)[NT][4]) {
#pragma unroll
  for (int j = 0; j < NT; ++j) c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.f;
}

// Store C (rows r0 + g, r0 + g + 8; columns 8j + 2t, +1) through f(r, n, value).
template <int NT, typename F>
__device__ __forceinline__ void store_acc(const float (&c)[NT][4], F f) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    const int n = 8 * j + 2 * t;
    f(g, n, c[j][0]);
    f(g, n + 1, c[j][1]);
    f(g + 8, n, c[j][2]);
    f(g + 8, n + 1, c[j][3]);
  }
}

// Shared-memory image of the network for the tensor-core kernels: BF16 weights with the
// first layer's inputs padded to 16 and the output rows padded to a multiple of 16 (zeros),
// FP32 biases.
template <int D>
struct TcNet {
  static constexpr int DK = D * WKP;
  static constexpr int DKP = 16 * ((DK + 15) / 16);   // output rows, padded
  static constexpr int HS = WH + 4;                   // FP32 activation row stride (floats)
  static constexpr int DLS = DKP + 4;                 // FP32 logit row stride
  static constexpr int KIN = 16;                      // first-layer inputs, padded
  // bf16 offsets
  static constexpr int W1 = 0, W2 = W1 + WH * KIN, W3 = W2 + WH * WH, W4 = W3 + WH * WH, NW = W4 + DKP * WH;
  // float offsets of the biases
  static constexpr int B1 = 0, B2 = B1 + WH, B3 = B2 + WH, B4 = B3 + WH, NB = B4 + DKP;
};

template <int D>
__device__ void load_net(const __nv_bfloat16 *__restrict__ wq, __nv_bfloat16 *sw, float *sb) {
  using N = TcNet<D>;
  const Layout L(D);
  const __nv_bfloat16 z = __float2bfloat16(0.f);
  for (int i = threadIdx.x; i < WH * N::KIN; i += blockDim.x) {
    const int j = i / N::KIN, k = i % N::KIN;
    sw[N::W1 + i] = k < D ? wq[L.oW1 + j * D + k] : z;
  }
  for (int i = threadIdx.x; i < WH * WH; i += blockDim.x) {
    sw[N::W2 + i] = wq[L.oW2 + i];
    sw[N::W3 + i] = wq[L.oW3 + i];
  }
  for (int i = threadIdx.x; i < N::DKP * WH; i += blockDim.x) sw[N::W4 + i] = i < N::DK * WH ? wq[L.oW4 + i] : z;
  for (int i = threadIdx.x; i < WH; i += blockDim.x) {
    sb[N::B1 + i] = __bfloat162float(wq[L.ob1 + i]);
    sb[N::B2 + i] = __bfloat162float(wq[L.ob2 + i]);
    sb[N::B3 + i] = __bfloat162float(wq[L.ob3 + i]);
  }
  for (int i = threadIdx.x; i < N::DKP; i += blockDim.x) sb[N::B4 + i] = i < N::DK ? __bfloat162float(wq[L.ob4 + i]) : 0.f;
}

// One hidden layer for the 16 rows of this warp: out[r][j] = act(b[j] + sum_k W[j][k] in[r][k]).
template <int D>
__device__ __forceinline__ void hidden_layer(const __nv_bfloat16 *w, int kin, const float *bias, const float *in,
                                             int in_stride, float *out, int r0) {
  using N = TcNet<D>;
  float c[WH / 8][4];
  zero_acc(c);
  warp_gemm<WH / 8, true>(
      c, kin / 16, [&](int r, int k) { return in[(r0 + r) * in_stride + k]; },
      [&](int k, int n) { return __bfloat162float(w[n * kin + k]); });
  store_acc(c, [&](int r, int n, float v) { out[(r0 + r) * N::HS + n] = act(v + bias[n]); });
}

template <int D>
constexpr size_t tc_grad_smem() {
  using N = TcNet<D>;
  return sizeof(__nv_bfloat16) * N::NW + sizeof(float) * (N::NB + WTILE * N::KIN + 4 * WTILE * N::HS + WTILE * N::DLS);
}

// One block = WTILE (64) samples, 4 warps of 16 samples: forward, |f|-weighted negative
// log-likelihood, backward.  The block's gradient and loss go to its own row of gpart / lpart
// (summed over blocks in order by grad_reduce_kernel), so the result does not depend on
// scheduling.
template <int D>
__global__ void __launch_bounds__(128) made_grad_tc_kernel(const __nv_bfloat16 *__restrict__ wq, float WALPHA,
                                                           const float *__restrict__ X, const float *__restrict__ wt,
                                                           int n, float *__restrict__ gpart,
                                                           float *__restrict__ lpart) {
  using N = TcNet<D>;
  const Layout L(D);
  extern __shared__ __align__(16) unsigned char tc_smem[];
  __nv_bfloat16 *sw = reinterpret_cast<__nv_bfloat16 *>(tc_smem);
  float *sb = reinterpret_cast<float *>(sw + N::NW);
  float *x = sb + N::NB;                 // [WTILE][KIN]
  float *h1 = x + WTILE * N::KIN;        // [WTILE][HS]
  float *h2 = h1 + WTILE * N::HS;
  float *h3 = h2 + WTILE * N::HS;
  float *dB = h3 + WTILE * N::HS;
  float *dl = dB + WTILE * N::HS;        // [WTILE][DLS]
  __shared__ float red[4];
  const int s0 = blockIdx.x * WTILE;
  const int ns = min(WTILE, n - s0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r0 = 16 * warp;
  float *gp = gpart + (size_t)blockIdx.x * L.n;
  load_net<D>(wq, sw, sb);
  for (int i = threadIdx.x; i < WTILE * N::KIN; i += blockDim.x) {
    const int s = i / N::KIN, d = i % N::KIN;
    x[i] = (s < ns && d < D) ? 2.f * X[(size_t)(s0 + s) * D + d] - 1.f : 0.f;
  }
  __syncthreads();
  // forward (each warp its own 16 rows)
  hidden_layer<D>(sw + N::W1, N::KIN, sb + N::B1, x, N::KIN, h1, r0);
  __syncwarp();
  hidden_layer<D>(sw + N::W2, WH, sb + N::B2, h1, N::HS, h2, r0);
  __syncwarp();
  hidden_layer<D>(sw + N::W3, WH, sb + N::B3, h2, N::HS, h3, r0);
  __syncwarp();
  {
    float c[N::DKP / 8][4];
    zero_acc(c);
    warp_gemm<N::DKP / 8, true>(
        c, WH / 16, [&](int r, int k) { return h3[(r0 + r) * N::HS + k]; },
        [&](int k, int o) { return __bfloat162float(sw[N::W4 + o * WH + k]); });
    store_acc(c, [&](int r, int o, float v) { dl[(r0 + r) * N::DLS + o] = v + sb[N::B4 + o]; });
  }
  __syncthreads();
  // loss and d loss / d logits, one thread per (sample, dimension)
  float lsum = 0.f;
  for (int i = threadIdx.x; i < WTILE * D; i += blockDim.x) {
    const int s = i / D, d = i % D;
    float *lg = dl + s * N::DLS + d * WKP;
    if (s >= ns) {
      for (int c = 0; c < WKP; ++c) lg[c] = 0.f;
      continue;
    }
    float mx = lg[0];
    for (int c = 1; c < WKP; ++c) mx = fmaxf(mx, lg[c]);
    float a[WKP], S = 0.f;
    for (int c = 0; c < WKP; ++c) a[c] = __expf(lg[c] - mx);
    for (int c = 0; c < WK; ++c) S += a[c] + a[c + 1];
    S *= 0.5f / WK;
    const float xd = 0.5f * (x[s * N::KIN + d] + 1.f);
    int b = (int)floorf(xd * WK);
    b = b < 0 ? 0 : (b > WK - 1 ? WK - 1 : b);
    const float t = xd * WK - (float)b;
    const float mix = (1.f - t) * a[b] + t * a[b + 1];
    const float qv = (1.f - WALPHA) * mix / S + WALPHA;
    const float w = wt[s0 + s];
    lsum += -w * logf(qv);
    const float k1 = -w * (1.f - WALPHA) / (qv * S);
    const float k2 = mix / S * (0.5f / WK);
    for (int c = 0; c < WKP; ++c) {
      const float own = (c == b ? 1.f - t : 0.f) + (c == b + 1 ? t : 0.f);
      const float nc = (c == 0 || c == WK) ? 1.f : 2.f;
      lg[c] = k1 * a[c] * (own - k2 * nc);
    }
  }
  for (int i = threadIdx.x; i < WTILE * (N::DLS - N::DK); i += blockDim.x) {   // padded logit columns
    const int s = i / (N::DLS - N::DK), o = N::DK + i % (N::DLS - N::DK);
    dl[s * N::DLS + o] = 0.f;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
  if (lane == 0) red[warp] = lsum;
  __syncthreads();
  if (threadIdx.x == 0) lpart[blockIdx.x] = ((red[0] + red[1]) + red[2]) + red[3];
  // dW4[o][j] = sum_s dl[s][o] h3[s][j]: m tiles of outputs over the warps, K = samples
  for (int mt = warp; mt < N::DKP / 16; mt += 4) {
    float c[WH / 8][4];
    zero_acc(c);
    warp_gemm<WH / 8, false>(
        c, WTILE / 16, [&](int r, int k) { return dl[k * N::DLS + 16 * mt + r]; },
        [&](int k, int j) { return h3[k * N::HS + j]; });
    store_acc(c, [&](int r, int j, float v) {
      const int o = 16 * mt + r;
      if (o < N::DK) gp[L.oW4 + o * WH + j] = v;
    });
  }
  for (int o = threadIdx.x; o < N::DK; o += blockDim.x) {
    float g = 0.f;
    for (int s = 0; s < WTILE; ++s) g += dl[s * N::DLS + o];
    gp[L.ob4 + o] = g;
  }
  // dh3 = dl W4 (own rows), dB = dh3 (1 - h3^2)
  {
    float c[WH / 8][4];
    zero_acc(c);
    warp_gemm<WH / 8, true>(
        c, N::DKP / 16, [&](int r, int k) { return dl[(r0 + r) * N::DLS + k]; },
        [&](int k, int j) { return __bfloat162float(sw[N::W4 + k * WH + j]); });
    store_acc(c, [&](int r, int j, float v) {
      const float h = h3[(r0 + r) * N::HS + j];
      dB[(r0 + r) * N::HS + j] = v * (1.f - h * h);
    });
  }
  __syncthreads();
  // dW3 = dB^T h2, db3; then dh2 = dB W3 -> h3 (own rows), times (1 - h2^2)
  {
    float c[WH / 8][4];
    zero_acc(c);
    warp_gemm<WH / 8, false>(
        c, WTILE / 16, [&](int r, int k) { return dB[k * N::HS + r0 + r]; },
        [&](int k, int j) { return h2[k * N::HS + j]; });
    store_acc(c, [&](int r, int j, float v) { gp[L.oW3 + (r0 + r) * WH + j] = v; });
  }
  for (int j = threadIdx.x; j < WH; j += blockDim.x) {
    float g = 0.f;
    for (int s = 0; s < WTILE; ++s) g += dB[s * N::HS + j];
    gp[L.ob3 + j] = g;
  }
  {
    float c[WH / 8][4];
    zero_acc(c);
    warp_gemm<WH / 8, true>(
        c, WH / 16, [&](int r, int k) { return dB[(r0 + r) * N::HS + k]; },
        [&](int k, int j) { return __bfloat162float(sw[N::W3 + k * WH + j]); });
    store_acc(c, [&](int r, int j, float v) {
      const float h = h2[(r0 + r) * N::HS + j];
      h3[(r0 + r) * N::HS + j] = v * (1.f - h * h);
    });
  }
  __syncthreads();
  // dW2 = h3^T h1, db2; then dh1 = h3 W2 -> dB (own rows), times (1 - h1^2)
  {
    float c[WH / 8][4];
    zero_acc(c);
    warp_gemm<WH / 8, false>(
        c, WTILE / 16, [&](int r, int k) { return h3[k * N::HS + r0 + r]; },
        [&](int k, int j) { return h1[k * N::HS + j]; });
    store_acc(c, [&](int r, int j, float v) { gp[L.oW2 + (r0 + r) * WH + j] = v; });
  }
  for (int j = threadIdx.x; j < WH; j += blockDim.x) {
    float g = 0.f;
    for (int s = 0; s < WTILE; ++s) g += h3[s * N::HS + j];
    gp[L.ob2 + j] = g;
  }
  __syncthreads();   // every warp has read dB above before it is overwritten
  {
    float c[WH / 8][4];
    zero_acc(c);
    warp_gemm<WH / 8, true>(
        c, WH / 16, [&](int r, int k) { return h3[(r0 + r) * N::HS + k]; },
        [&](int k, int j) { return __bfloat162float(sw[N::W2 + k * WH + j]); });
    store_acc(c, [&](int r, int j, float v) {
      const float h = h1[(r0 + r) * N::HS + j];
      dB[(r0 + r) * N::HS + j] = v * (1.f - h * h);
    });
  }
  __syncthreads();
  // dW1 = dB^T x (inputs padded to 8 columns), db1
  {
    float c[1][4];
    zero_acc(c);
    warp_gemm<1, false>(
        c, WTILE / 16, [&](int r, int k) { return dB[k * N::HS + r0 + r]; },
        [&](int k, int d) { return x[k * N::KIN + d]; });
    store_acc(c, [&](int r, int d, float v) {
      if (d < D) gp[L.oW1 + (r0 + r) * D + d] = v;
    });
  }
  for (int j = threadIdx.x; j < WH; j += blockDim.x) {
    float g = 0.f;
    for (int s = 0; s < WTILE; ++s) g += dB[s * N::HS + j];
    gp[L.ob1 + j] = g;
  }
}

// grad[i] = sum over blocks b (in order) of gpart[b][i]; loss likewise.
__global__ void grad_reduce_kernel(const float *__restrict__ gpart, const float *__restrict__ lpart, int nb, int np,
                                   float *__restrict__ grad, float *__restrict__ loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < np) {
    float g = 0.f;
    for (int b = 0; b < nb; ++b) g += gpart[(size_t)b * np + i];
    grad[i] = g;
  }
  if (i == 0) {
    float l = 0.f;
    for (int b = 0; b < nb; ++b) l += lpart[b];
    *loss = l;
  }
}

// Adam on the FP32 master weights; masked entries stay zero; BF16 copy refreshed.
__global__ void adam_kernel(float *p, float *m, float *v, const float *g, const float *mask, __nv_bfloat16 *wq,
                            int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i] * mask[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = (p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps)) * mask[i];
    p[i] = pi;
    wq[i] = __float2bfloat16(pi);
  }
}

template <int D>
constexpr size_t tc_map_smem() {
  using N = TcNet<D>;
  return sizeof(__nv_bfloat16) * N::NW + sizeof(float) * (N::NB + WTILE * N::KIN + 2 * WTILE * N::HS + WTILE * 24);
}

// y (Sobol) -> x = w(y) and the importance weight 1/q(x).  A block maps WTILE (64) samples,
// 4 warps of 16; for each dimension d in turn a warp runs the network on its 16 samples (the
// inputs x_<d found so far, x_>=d still zero, which the masks ignore), keeps the 17 logits of
// dimension d and inverts that dimension's CDF, one lane per sample.
template <int D>
__global__ void __launch_bounds__(128) warp_map_tc_kernel(const __nv_bfloat16 *__restrict__ wq, float WALPHA,
                                                          const uint32_t *__restrict__ sm_m,
                                                          const uint32_t *__restrict__ sm_x0, uint64_t first,
                                                          uint64_t n, double *__restrict__ pts) {
  using N = TcNet<D>;
  extern __shared__ __align__(16) unsigned char tc_smem[];
  __nv_bfloat16 *sw = reinterpret_cast<__nv_bfloat16 *>(tc_smem);
  float *sb = reinterpret_cast<float *>(sw + N::NW);
  float *xin = sb + N::NB;               // [WTILE][KIN]
  float *ha = xin + WTILE * N::KIN;      // [WTILE][HS]
  float *hb = ha + WTILE * N::HS;
  float *lg = hb + WTILE * N::HS;        // [WTILE][24]
  load_net<D>(wq, sw, sb);
  for (int i = threadIdx.x; i < WTILE * N::KIN; i += blockDim.x) xin[i] = 0.f;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r0 = 16 * warp;
  const uint64_t base = (uint64_t)blockIdx.x * WTILE + r0;   // this warp's first sample
  const bool mine = lane < 16 && base + lane < n;             // lane r handles sample base + r
  float y[D];
  double wt = 1.0;
  if (mine) {
    const uint64_t idx = first + base + lane;
    const uint32_t gray = (uint32_t)(idx ^ (idx >> 1));
#pragma unroll
    for (int d = 0; d < D; ++d) {
      uint32_t v = sm_x0[d];
      for (int b = 0; b < 32; ++b)
        if ((gray >> b) & 1u) v ^= sm_m[d * 32 + b];
      y[d] = (float)ldexp((double)v, -32);
    }
  }
#pragma unroll 1
  for (int d = 0; d < D; ++d) {
    hidden_layer<D>(sw + N::W1, N::KIN, sb + N::B1, xin, N::KIN, ha, r0);
    __syncwarp();
    hidden_layer<D>(sw + N::W2, WH, sb + N::B2, ha, N::HS, hb, r0);
    __syncwarp();
    hidden_layer<D>(sw + N::W3, WH, sb + N::B3, hb, N::HS, ha, r0);
    __syncwarp();
    {
      float c[3][4];   // the 17 logits of dimension d (24 columns)
      zero_acc(c);
      const int o0 = d * WKP;
      warp_gemm<3, true>(
          c, WH / 16, [&](int r, int k) { return ha[(r0 + r) * N::HS + k]; },
          [&](int k, int o) { return __bfloat162float(sw[N::W4 + (o0 + o) * WH + k]); });
      store_acc(c, [&](int r, int o, float v) { lg[(r0 + r) * 24 + o] = v + sb[N::B4 + o0 + o]; });
    }
    __syncwarp();
    if (mine) {
      float v[WKP], mx = -1e30f;
      const float *l = lg + (r0 + lane) * 24;
      for (int c = 0; c < WKP; ++c) {
        v[c] = l[c];
        mx = fmaxf(mx, v[c]);
      }
      float S = 0.f;
      for (int c = 0; c < WKP; ++c) v[c] = __expf(v[c] - mx);
      for (int c = 0; c < WK; ++c) S += v[c] + v[c + 1];
      S *= 0.5f / WK;
      for (int c = 0; c < WKP; ++c) v[c] = (1.f - WALPHA) * v[c] / S + WALPHA;
      // invert the quadratic CDF: bin mass m_b = (v_b + v_{b+1}) / 2K
      float yd = 0.f;
#pragma unroll
      for (int e = 0; e < D; ++e)
        if (e == d) yd = y[e];
      float cum = 0.f;
      int b = WK - 1;
      for (int c = 0; c < WK; ++c) {
        const float mb = 0.5f * (v[c] + v[c + 1]) / WK;
        if (yd < cum + mb || c == WK - 1) { b = c; break; }
        cum += mb;
      }
      const float r = fmaxf(yd - cum, 0.f) * WK;
      const float dv = v[b + 1] - v[b];
      float t = 2.f * r / (v[b] + sqrtf(fmaxf(v[b] * v[b] + 2.f * dv * r, 0.f)));
      t = t < 0.f ? 0.f : (t >= 1.f ? 0.99999994f : t);
      const float xd = ((float)b + t) / (float)WK;
      xin[(r0 + lane) * N::KIN + d] = 2.f * xd - 1.f;
      pts[(base + lane) * (D + 1) + d] = (double)xd;
      wt /= (double)(v[b] + dv * t);
    }
    __syncwarp();
  }
  if (mine) pts[(base + lane) * (D + 1) + D] = wt;
}

}  // namespace

struct WarpRec {
  int D = 0;
  float alpha = WALPHA_DEFAULT;
  DevBuf<float> p, m, v, g, mask, loss;
  DevBuf<__nv_bfloat16> wq;
  DevBuf<float> X, w;
  DevBuf<float> gpart, lpart;   // per-block gradient and loss rows of made_grad_tc_kernel
  int64_t t = 0;
  std::vector<float> hmask;
};

void destroy_warps(qiw_ctx *c) {
  for (WarpRec *w : c->warps) {
    w->p.release(); w->m.release(); w->v.release(); w->g.release(); w->mask.release(); w->loss.release();
    w->wq.release(); w->X.release(); w->w.release(); w->gpart.release(); w->lpart.release();
    delete w;
  }
  c->warps.clear();
}

int warp_dim(qiw_ctx *c, int id) { return c->warps[id]->D; }

// Launch of a D-templated warp kernel for the runtime dimension (2 <= D <= WDMAX).
#define QIW_WARP_D_SWITCH(D, CALL) \
  switch (D) {                     \
    case 2: CALL(2); break;        \
    case 3: CALL(3); break;        \
    case 4: CALL(4); break;        \
    case 5: CALL(5); break;        \
    case 6: CALL(6); break;        \
    case 7: CALL(7); break;        \
    default: CALL(8); break;       \
  }

int aux_streams(qiw_ctx *c, int n) {
  int rc;
  for (int i = (int)c->aux.size(); i < n; ++i) {
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    if ((rc = c->cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "auxiliary streams"))) return rc;
    if ((rc = c->cuda(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "auxiliary streams"))) {
      cudaStreamDestroy(s);
      return rc;
    }
    c->aux.push_back(s);
    c->aux_ev.push_back(ev);
  }
  return QIW_OK;
}

int aux_fork(qiw_ctx *c, int n) {
  int rc;
  if ((rc = c->cuda(cudaEventRecord(c->aux_ev[0], c->stream), "auxiliary streams: fork"))) return rc;
  for (int i = 0; i < n; ++i)
    if ((rc = c->cuda(cudaStreamWaitEvent(c->aux[i], c->aux_ev[0], 0), "auxiliary streams: fork"))) return rc;
  return QIW_OK;
}

int aux_join(qiw_ctx *c, int n) {
  int rc = QIW_OK;
  for (int i = 0; i < n; ++i) {
    int r2;
    if ((r2 = c->cuda(cudaEventRecord(c->aux_ev[i], c->aux[i]), "auxiliary streams: join")) ||
        (r2 = c->cuda(cudaStreamWaitEvent(c->stream, c->aux_ev[i], 0), "auxiliary streams: join"))) {
      cudaStreamSynchronize(c->aux[i]);
      if (!rc) rc = r2;
    }
  }
  return rc;
}

int warp_map_device(qiw_ctx *c, int id, const uint32_t *m_dev, const uint32_t *x0_dev, uint64_t first, uint64_t n,
                    double *pts_dev, cudaStream_t st) {
  if (!st) st = c->stream;
  WarpRec *w = c->warps[id];
  const unsigned blocks = (unsigned)((n + WTILE - 1) / WTILE);
  if (blocks == 0) return QIW_OK;
  cudaError_t e = cudaSuccess;
#define QIW_MAP_CALL(DD)                                                                                   \
  {                                                                                                        \
    const size_t smem = tc_map_smem<DD>();                                                                 \
    e = cudaFuncSetAttribute(warp_map_tc_kernel<DD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (e == cudaSuccess)                                                                                  \
      warp_map_tc_kernel<DD><<<blocks, 128, smem, st>>>(w->wq.p, w->alpha, m_dev, x0_dev, first, n, pts_dev); \
  }
  QIW_WARP_D_SWITCH(w->D, QIW_MAP_CALL)
#undef QIW_MAP_CALL
  if (e != cudaSuccess) return c->cuda(e, "warp map kernel: shared memory");
  return c->cuda(cudaGetLastError(), "warp map kernel");
}

}  // namespace qiw

using namespace qiw;

extern "C" {

int qiw_warp_create(qiw_ctx *c, int32_t D, uint64_t seed, int32_t *warp_id) {
  if (!c || !warp_id) return QIW_ERR_ARG;
  if (D < 2 || D > WDMAX) return c->fail(QIW_ERR_UNSUPPORTED, "qiw_warp_create: dimension must lie in 2..8");
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_warp_create: cudaSetDevice");
  Layout L(D);
  WarpRec *w = new WarpRec();
  w->D = D;
  // MADE masks: input i has degree i+1, hidden unit j degree 1 + j mod (D-1), output d degree d+1
  std::vector<float> mask(L.n, 1.f), p(L.n, 0.f);
  auto hdeg = [&](int j) { return 1 + j % (D - 1); };
  for (int j = 0; j < WH; ++j)
    for (int k = 0; k < D; ++k) mask[L.oW1 + j * D + k] = (hdeg(j) >= k + 1) ? 1.f : 0.f;
  for (int j = 0; j < WH; ++j)
    for (int k = 0; k < WH; ++k) {
      mask[L.oW2 + j * WH + k] = (hdeg(j) >= hdeg(k)) ? 1.f : 0.f;
      mask[L.oW3 + j * WH + k] = (hdeg(j) >= hdeg(k)) ? 1.f : 0.f;
    }
  for (int o = 0; o < L.DK; ++o)
    for (int k = 0; k < WH; ++k) mask[L.oW4 + o * WH + k] = (o / WKP + 1 > hdeg(k)) ? 1.f : 0.f;
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  auto init = [&](int off, int rows, int cols) {
    const float sc = std::sqrt(1.f / (float)cols);
    for (int i = 0; i < rows * cols; ++i) p[off + i] = nd(rng) * sc * mask[off + i];
  };
  init(L.oW1, WH, D);
  init(L.oW2, WH, WH);
  init(L.oW3, WH, WH);
  for (int i = 0; i < L.DK * WH; ++i) p[L.oW4 + i] = 0.f;  // start at the uniform density
  std::vector<__nv_bfloat16> q(L.n);
  for (int i = 0; i < L.n; ++i) q[i] = __float2bfloat16(p[i]);
  std::vector<float> zero(L.n, 0.f);
  int rc;
  if ((rc = c->cuda(w->p.upload(p.data(), L.n, c->stream), "warp upload")) ||
      (rc = c->cuda(w->m.upload(zero.data(), L.n, c->stream), "warp upload")) ||
      (rc = c->cuda(w->v.upload(zero.data(), L.n, c->stream), "warp upload")) ||
      (rc = c->cuda(w->g.reserve(L.n), "warp alloc")) ||
      (rc = c->cuda(w->mask.upload(mask.data(), L.n, c->stream), "warp upload")) ||
      (rc = c->cuda(w->wq.upload(q.data(), L.n, c->stream), "warp upload")) ||
      (rc = c->cuda(w->loss.reserve(1), "warp alloc")) || (rc = c->cuda(cudaStreamSynchronize(c->stream), "warp"))) {
    delete w;
    return rc;
  }
  w->hmask = mask;
  c->warps.push_back(w);
  *warp_id = (int32_t)c->warps.size() - 1;
  return QIW_OK;
}

int qiw_warp_set_mix(qiw_ctx *c, int32_t id, double uniform_mix) {
  if (!c || id < 0 || id >= (int)c->warps.size() || !(uniform_mix > 0.0) || !(uniform_mix <= 1.0))
    return QIW_ERR_ARG;
  c->warps[id]->alpha = (float)uniform_mix;
  return QIW_OK;
}

int qiw_warp_n_params(qiw_ctx *c, int32_t id, int64_t *n) {
  if (!c || !n || id < 0 || id >= (int)c->warps.size()) return QIW_ERR_ARG;
  *n = Layout(c->warps[id]->D).n;
  return QIW_OK;
}

int qiw_warp_get_params(qiw_ctx *c, int32_t id, double *out) {
  if (!c || !out || id < 0 || id >= (int)c->warps.size()) return QIW_ERR_ARG;
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_warp_get_params: cudaSetDevice");
  WarpRec *w = c->warps[id];
  const int n = Layout(w->D).n;
  std::vector<float> p(n);
  int rc = c->cuda(cudaMemcpy(p.data(), w->p.p, sizeof(float) * n, cudaMemcpyDeviceToHost), "warp params");
  if (rc) return rc;
  for (int i = 0; i < n; ++i) out[i] = p[i];
  return QIW_OK;
}

int qiw_warp_set_params(qiw_ctx *c, int32_t id, const double *in) {
  if (!c || !in || id < 0 || id >= (int)c->warps.size()) return QIW_ERR_ARG;
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_warp_set_params: cudaSetDevice");
  WarpRec *w = c->warps[id];
  const int n = Layout(w->D).n;
  std::vector<float> p(n);
  std::vector<__nv_bfloat16> q(n);
  for (int i = 0; i < n; ++i) {
    p[i] = (float)in[i] * w->hmask[i];
    q[i] = __float2bfloat16(p[i]);
  }
  int rc;
  if ((rc = c->cuda(w->p.upload(p.data(), n, c->stream), "warp params")) ||
      (rc = c->cuda(w->wq.upload(q.data(), n, c->stream), "warp params")) ||
      (rc = c->cuda(cudaStreamSynchronize(c->stream), "warp params")))
    return rc;
  return QIW_OK;
}

static int upload_batch(qiw_ctx *c, WarpRec *w, const double *x, const double *wt, int64_t n) {
  std::vector<float> xf((size_t)n * w->D), wf(n);
  double tot = 0.0;
  for (int64_t i = 0; i < n; ++i) tot += wt[i];
  if (!(tot > 0.0)) return c->fail(QIW_ERR_ARG, "qiw_warp: training weights must have a positive sum");
  for (int64_t i = 0; i < (int64_t)n * w->D; ++i) xf[i] = (float)x[i];
  for (int64_t i = 0; i < n; ++i) wf[i] = (float)(wt[i] / tot);
  int rc;
  if ((rc = c->cuda(w->X.upload(xf.data(), xf.size(), c->stream), "warp data")) ||
      (rc = c->cuda(w->w.upload(wf.data(), wf.size(), c->stream), "warp data")))
    return rc;
  return QIW_OK;
}

// Gradient and loss of n samples into w->g and w->loss: one made_grad_tc_kernel block per 64
// samples writes its own row, grad_reduce_kernel sums the rows in block order.
static int run_grad(qiw_ctx *c, WarpRec *w, const float *X, const float *wt, int64_t n, cudaStream_t st) {
  const int Lw = Layout(w->D).n;
  const unsigned blocks = (unsigned)((n + WTILE - 1) / WTILE);
  int rc;
  if ((rc = c->cuda(w->gpart.reserve((size_t)blocks * Lw), "warp grad partials")) ||
      (rc = c->cuda(w->lpart.reserve(blocks), "warp grad partials")))
    return rc;
  cudaError_t e = cudaSuccess;
#define QIW_GRAD_CALL(DD)                                                                                    \
  {                                                                                                          \
    const size_t smem = tc_grad_smem<DD>();                                                                  \
    e = cudaFuncSetAttribute(made_grad_tc_kernel<DD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (e == cudaSuccess)                                                                                    \
      made_grad_tc_kernel<DD><<<blocks, 128, smem, st>>>(w->wq.p, w->alpha, X, wt, (int)n, w->gpart.p, w->lpart.p); \
  }
  QIW_WARP_D_SWITCH(w->D, QIW_GRAD_CALL)
#undef QIW_GRAD_CALL
  if (e != cudaSuccess) return c->cuda(e, "warp grad kernel: shared memory");
  if ((rc = c->cuda(cudaGetLastError(), "warp grad kernel"))) return rc;
  grad_reduce_kernel<<<(Lw + 255) / 256, 256, 0, st>>>(w->gpart.p, w->lpart.p, (int)blocks, Lw, w->g.p, w->loss.p);
  return c->cuda(cudaGetLastError(), "warp grad reduce kernel");
}

int qiw_warp_grad(qiw_ctx *c, int32_t id, const double *x, const double *wt, int64_t n, double *grad_out,
                  double *loss_out) {
  if (!c || !x || !wt || !grad_out || id < 0 || id >= (int)c->warps.size() || n <= 0) return QIW_ERR_ARG;
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_warp_grad: cudaSetDevice");
  WarpRec *w = c->warps[id];
  int rc = upload_batch(c, w, x, wt, n);
  if (rc || (rc = run_grad(c, w, w->X.p, w->w.p, n, c->stream))) return rc;
  const int Lw = Layout(w->D).n;
  std::vector<float> g(Lw);
  float loss = 0.f;
  if ((rc = c->cuda(cudaMemcpyAsync(g.data(), w->g.p, sizeof(float) * Lw, cudaMemcpyDeviceToHost, c->stream), "warp")) ||
      (rc = c->cuda(cudaMemcpyAsync(&loss, w->loss.p, sizeof(float), cudaMemcpyDeviceToHost, c->stream), "warp")) ||
      (rc = c->cuda(cudaStreamSynchronize(c->stream), "warp")))
    return rc;
  for (int i = 0; i < Lw; ++i) grad_out[i] = g[i];
  if (loss_out) *loss_out = loss;
  return QIW_OK;
}

int qiw_warp_train(qiw_ctx *c, int32_t id, const double *x, const double *wt, int64_t n, int32_t steps,
                   int32_t batch, double lr, double *final_loss) {
  if (!c || !x || !wt || id < 0 || id >= (int)c->warps.size() || n <= 0 || steps < 0 || batch <= 0)
    return QIW_ERR_ARG;
  return qiw_warp_train_batch(c, 1, &id, &x, &wt, &n, steps, batch, lr, final_loss);
}

int qiw_warp_train_batch(qiw_ctx *c, int32_t n_warps, const int32_t *ids, const double *const *x,
                         const double *const *wt, const int64_t *n, int32_t steps, int32_t batch, double lr,
                         double *final_loss) {
  if (!c || n_warps < 0 || (n_warps > 0 && (!ids || !x || !wt || !n)) || steps < 0 || batch <= 0) return QIW_ERR_ARG;
  for (int k = 0; k < n_warps; ++k) {
    if (ids[k] < 0 || ids[k] >= (int)c->warps.size() || !x[k] || !wt[k] || n[k] <= 0) return QIW_ERR_ARG;
    for (int j = 0; j < k; ++j)
      if (ids[j] == ids[k]) return c->fail(QIW_ERR_ARG, "qiw_warp_train_batch: a warp appears twice");
  }
  if (n_warps == 0) return QIW_OK;
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_warp_train: cudaSetDevice");
  // Uploads (whole-set normalisation) and every buffer a step uses, reserved before any step
  // runs: minibatch b of warp k covers its samples [b*batch, (b+1)*batch) cyclically.
  int rc;
  for (int k = 0; k < n_warps; ++k) {
    WarpRec *w = c->warps[ids[k]];
    const size_t blocks = (size_t)((n[k] + WTILE - 1) / WTILE);
    if ((rc = upload_batch(c, w, x[k], wt[k], n[k])) ||
        (rc = c->cuda(w->gpart.reserve(blocks * Layout(w->D).n), "warp grad partials")) ||
        (rc = c->cuda(w->lpart.reserve(blocks), "warp grad partials")))
      return rc;
  }
  // One warp trains on the context stream; several train concurrently, warp k on auxiliary
  // stream k mod kAuxStreams (its steps stay in order there), forked from and joined back into
  // the context stream.  Each warp owns its parameters, moments and gradient rows, so the
  // results are those of training the warps one after another.
  const int n_st = n_warps == 1 ? 0 : std::min(n_warps, kAuxStreams);
  if (n_st > 0 && ((rc = aux_streams(c, n_st)) || (rc = aux_fork(c, n_st)))) return rc;
  auto stream_of = [&](int k) { return n_st == 0 ? c->stream : c->aux[k % n_st]; };
  auto enqueue = [&]() -> int {
    const float b1 = 0.9f, b2 = 0.999f;
    int r;
    for (int s = 0; s < steps; ++s) {
      for (int k = 0; k < n_warps; ++k) {
        WarpRec *w = c->warps[ids[k]];
        cudaStream_t st = stream_of(k);
        const int64_t nb = std::max<int64_t>(1, n[k] / batch);
        const int64_t lo = (s % nb) * batch, cnt = std::min<int64_t>(batch, n[k] - lo);
        if ((r = run_grad(c, w, w->X.p + lo * w->D, w->w.p + lo, cnt, st))) return r;
        w->t += 1;
        const float c1 = 1.f - std::pow(b1, (float)w->t), c2 = 1.f - std::pow(b2, (float)w->t);
        adam_kernel<<<64, 256, 0, st>>>(w->p.p, w->m.p, w->v.p, w->g.p, w->mask.p, w->wq.p, Layout(w->D).n,
                                        (float)lr, b1, b2, 1e-8f, c1, c2);
        if ((r = c->cuda(cudaGetLastError(), "adam kernel"))) return r;
      }
    }
    if (final_loss)
      for (int k = 0; k < n_warps; ++k) {
        WarpRec *w = c->warps[ids[k]];
        if ((r = run_grad(c, w, w->X.p, w->w.p, n[k], stream_of(k)))) return r;
      }
    return QIW_OK;
  };
  rc = enqueue();
  // join the auxiliary streams back into the context stream, also after a failed launch, so
  // later work on the context stream is ordered after everything enqueued here
  const int rj = aux_join(c, n_st);
  if (rc || (rc = rj)) return rc;
  if (final_loss) {
    std::vector<float> loss(n_warps, 0.f);
    for (int k = 0; k < n_warps; ++k)
      if ((rc = c->cuda(cudaMemcpyAsync(&loss[k], c->warps[ids[k]]->loss.p, sizeof(float), cudaMemcpyDeviceToHost,
                                        c->stream), "warp")))
        return rc;
    if ((rc = c->cuda(cudaStreamSynchronize(c->stream), "warp train"))) return rc;
    for (int k = 0; k < n_warps; ++k) final_loss[k] = loss[k];
    return QIW_OK;
  }
  return c->cuda(cudaStreamSynchronize(c->stream), "warp train");
}

int qiw_warp_map(qiw_ctx *c, int32_t id, const uint32_t *m, const uint32_t *x0, uint64_t first, uint64_t n,
                 double *pts_out) {
  if (!c || !m || !x0 || !pts_out || id < 0 || id >= (int)c->warps.size()) return QIW_ERR_ARG;
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_warp_map: cudaSetDevice");
  WarpRec *w = c->warps[id];
  DevBuf<uint32_t> dm;
  DevBuf<double> dp;
  int rc;
  std::vector<uint32_t> tab(m, m + 32 * w->D);
  tab.insert(tab.end(), x0, x0 + w->D);
  if ((rc = c->cuda(dm.upload(tab.data(), tab.size(), c->stream), "warp map")) ||
      (rc = c->cuda(dp.reserve((size_t)n * (w->D + 1)), "warp map")) ||
      (rc = warp_map_device(c, id, dm.p, dm.p + 32 * w->D, first, n, dp.p)) ||
      (rc = c->cuda(cudaMemcpyAsync(pts_out, dp.p, sizeof(double) * n * (w->D + 1), cudaMemcpyDeviceToHost, c->stream),
                    "warp map")) ||
      (rc = c->cuda(cudaStreamSynchronize(c->stream), "warp map"))) {
    dm.release();
    dp.release();
    return rc;
  }
  dm.release();
  dp.release();
  return QIW_OK;
}

}  // extern "C"
