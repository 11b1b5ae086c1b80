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

// Weights (BF16 on the device) -> FP32 in shared memory.
__device__ void load_weights(const __nv_bfloat16 *wq, float *sw, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) sw[i] = __bfloat162float(wq[i]);
}

// One block = WTILE samples: forward, weighted NLL, backward, per-block gradient sums
// (one atomicAdd per parameter per block).
__global__ void made_grad_kernel(const __nv_bfloat16 *__restrict__ wq, int D, float WALPHA,
                                 const float *__restrict__ X, const float *__restrict__ wt, int n,
                                 float *__restrict__ grad, float *__restrict__ loss) {
  extern __shared__ float sm[];
  const Layout L(D);
  float *W = sm;                       // L.n
  float *x = W + L.n;                  // [WTILE][WDMAX]
  float *h1 = x + WTILE * WDMAX;       // [WTILE][WH]
  float *h2 = h1 + WTILE * WH;
  float *h3 = h2 + WTILE * WH;
  float *dl = h3 + WTILE * WH;         // [WTILE][DK]
  float *dB = dl + WTILE * L.DK;       // [WTILE][WH]
  const int s0 = blockIdx.x * WTILE;
  const int ns = min(WTILE, n - s0);
  load_weights(wq, W, L.n);
  for (int i = threadIdx.x; i < WTILE * WDMAX; i += blockDim.x) {
    const int s = i / WDMAX, d = i % WDMAX;
    x[i] = (s < ns && d < D) ? 2.f * X[(size_t)(s0 + s) * D + d] - 1.f : 0.f;
  }
  __syncthreads();
  // forward
  for (int i = threadIdx.x; i < WTILE * WH; i += blockDim.x) {
    const int s = i / WH, j = i % WH;
    float a = W[L.ob1 + j];
    for (int k = 0; k < D; ++k) a = fmaf(W[L.oW1 + j * D + k], x[s * WDMAX + k], a);
    h1[i] = act(a);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < WTILE * WH; i += blockDim.x) {
    const int s = i / WH, j = i % WH;
    float a = W[L.ob2 + j];
    for (int k = 0; k < WH; ++k) a = fmaf(W[L.oW2 + j * WH + k], h1[s * WH + k], a);
    h2[i] = act(a);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < WTILE * WH; i += blockDim.x) {
    const int s = i / WH, j = i % WH;
    float a = W[L.ob3 + j];
    for (int k = 0; k < WH; ++k) a = fmaf(W[L.oW3 + j * WH + k], h2[s * WH + k], a);
    h3[i] = act(a);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < WTILE * L.DK; i += blockDim.x) {
    const int s = i / L.DK, o = i % L.DK;
    float a = W[L.ob4 + o];
    for (int k = 0; k < WH; ++k) a = fmaf(W[L.oW4 + o * WH + k], h3[s * WH + k], a);
    dl[i] = a;
  }
  __syncthreads();
  // loss and d loss / d logits, one thread per (sample, dimension)
  float lsum = 0.f;
  for (int i = threadIdx.x; i < WTILE * D; i += blockDim.x) {
    const int s = i / D, d = i % D;
    float *lg = dl + s * L.DK + d * WKP;
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
    const float xd = 0.5f * (x[s * WDMAX + d] + 1.f);
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
  atomicAdd(loss, lsum);
  __syncthreads();
  // backward: W4, b4, dh3
  for (int i = threadIdx.x; i < L.DK * WH; i += blockDim.x) {
    const int o = i / WH, j = i % WH;
    float g = 0.f;
    for (int s = 0; s < ns; ++s) g = fmaf(dl[s * L.DK + o], h3[s * WH + j], g);
    atomicAdd(grad + L.oW4 + i, g);
  }
  for (int o = threadIdx.x; o < L.DK; o += blockDim.x) {
    float g = 0.f;
    for (int s = 0; s < ns; ++s) g += dl[s * L.DK + o];
    atomicAdd(grad + L.ob4 + o, g);
  }
  for (int i = threadIdx.x; i < WTILE * WH; i += blockDim.x) {
    const int s = i / WH, j = i % WH;
    float a = 0.f;
    for (int o = 0; o < L.DK; ++o) a = fmaf(W[L.oW4 + o * WH + j], dl[s * L.DK + o], a);
    dB[i] = a * (1.f - h3[i] * h3[i]);
  }
  __syncthreads();
  // W3, b3, dh2 (into h3)
  for (int i = threadIdx.x; i < WH * WH; i += blockDim.x) {
    const int jo = i / WH, ji = i % WH;
    float g = 0.f;
    for (int s = 0; s < ns; ++s) g = fmaf(dB[s * WH + jo], h2[s * WH + ji], g);
    atomicAdd(grad + L.oW3 + i, g);
  }
  for (int j = threadIdx.x; j < WH; j += blockDim.x) {
    float g = 0.f;
    for (int s = 0; s < ns; ++s) g += dB[s * WH + j];
    atomicAdd(grad + L.ob3 + j, g);
  }
  for (int i = threadIdx.x; i < WTILE * WH; i += blockDim.x) {
    const int s = i / WH, j = i % WH;
    float a = 0.f;
    for (int o = 0; o < WH; ++o) a = fmaf(W[L.oW3 + o * WH + j], dB[s * WH + o], a);
    h3[i] = a * (1.f - h2[i] * h2[i]);
  }
  __syncthreads();
  // W2, b2, dh1 (into dB)
  for (int i = threadIdx.x; i < WH * WH; i += blockDim.x) {
    const int jo = i / WH, ji = i % WH;
    float g = 0.f;
    for (int s = 0; s < ns; ++s) g = fmaf(h3[s * WH + jo], h1[s * WH + ji], g);
    atomicAdd(grad + L.oW2 + i, g);
  }
  for (int j = threadIdx.x; j < WH; j += blockDim.x) {
    float g = 0.f;
    for (int s = 0; s < ns; ++s) g += h3[s * WH + j];
    atomicAdd(grad + L.ob2 + j, g);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < WTILE * WH; i += blockDim.x) {
    const int s = i / WH, j = i % WH;
    float a = 0.f;
    for (int o = 0; o < WH; ++o) a = fmaf(W[L.oW2 + o * WH + j], h3[s * WH + o], a);
    dB[i] = a * (1.f - h1[i] * h1[i]);
  }
  __syncthreads();
  // W1, b1
  for (int i = threadIdx.x; i < WH * D; i += blockDim.x) {
    const int jo = i / D, k = i % D;
    float g = 0.f;
    for (int s = 0; s < ns; ++s) g = fmaf(dB[s * WH + jo], x[s * WDMAX + k], g);
    atomicAdd(grad + L.oW1 + i, g);
  }
  for (int j = threadIdx.x; j < WH; j += blockDim.x) {
    float g = 0.f;
    for (int s = 0; s < ns; ++s) g += dB[s * WH + j];
    atomicAdd(grad + L.ob1 + j, g);
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

// y (Sobol) -> x = w(y) and the importance weight 1/q(x); one thread per sample.
__global__ void warp_map_kernel(const __nv_bfloat16 *__restrict__ wq, int D, float WALPHA,
                                const uint32_t *__restrict__ sm_m,
                                const uint32_t *__restrict__ sm_x0, uint64_t first, uint64_t n,
                                double *__restrict__ pts) {
  extern __shared__ float sw[];
  const Layout L(D);
  load_weights(wq, sw, L.n);
  __syncthreads();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t idx = first + i;
  const uint32_t gray = (uint32_t)(idx ^ (idx >> 1));
  float y[WDMAX], xin[WDMAX];
  for (int d = 0; d < D; ++d) {
    uint32_t v = sm_x0[d];
    for (int b = 0; b < 32; ++b)
      if ((gray >> b) & 1u) v ^= sm_m[d * 32 + b];
    y[d] = (float)ldexp((double)v, -32);
    xin[d] = 0.f;
  }
  double wt = 1.0;
  float h1[WH], h2[WH], h3[WH];
  for (int d = 0; d < D; ++d) {
    for (int j = 0; j < WH; ++j) {
      float a = sw[L.ob1 + j];
      for (int k = 0; k < D; ++k) a = fmaf(sw[L.oW1 + j * D + k], xin[k], a);
      h1[j] = act(a);
    }
    for (int j = 0; j < WH; ++j) {
      float a = sw[L.ob2 + j];
      for (int k = 0; k < WH; ++k) a = fmaf(sw[L.oW2 + j * WH + k], h1[k], a);
      h2[j] = act(a);
    }
    for (int j = 0; j < WH; ++j) {
      float a = sw[L.ob3 + j];
      for (int k = 0; k < WH; ++k) a = fmaf(sw[L.oW3 + j * WH + k], h2[k], a);
      h3[j] = act(a);
    }
    float v[WKP], mx = -1e30f;
    for (int c = 0; c < WKP; ++c) {
      const int o = d * WKP + c;
      float a = sw[L.ob4 + o];
      for (int k = 0; k < WH; ++k) a = fmaf(sw[L.oW4 + o * WH + k], h3[k], a);
      v[c] = a;
      mx = fmaxf(mx, a);
    }
    float S = 0.f;
    for (int c = 0; c < WKP; ++c) v[c] = __expf(v[c] - mx);
    for (int c = 0; c < WK; ++c) S += v[c] + v[c + 1];
    S *= 0.5f / WK;
    for (int c = 0; c < WKP; ++c) v[c] = (1.f - WALPHA) * v[c] / S + WALPHA;
    // invert the quadratic CDF: bin mass m_b = (v_b + v_{b+1}) / 2K
    float cum = 0.f;
    int b = WK - 1;
    for (int c = 0; c < WK; ++c) {
      const float mb = 0.5f * (v[c] + v[c + 1]) / WK;
      if (y[d] < cum + mb || c == WK - 1) { b = c; break; }
      cum += mb;
    }
    const float r = fmaxf(y[d] - cum, 0.f) * WK;
    const float dv = v[b + 1] - v[b];
    float t = 2.f * r / (v[b] + sqrtf(fmaxf(v[b] * v[b] + 2.f * dv * r, 0.f)));
    t = t < 0.f ? 0.f : (t >= 1.f ? 0.99999994f : t);
    const float xd = ((float)b + t) / (float)WK;
    xin[d] = 2.f * xd - 1.f;
    pts[i * (D + 1) + d] = (double)xd;
    wt /= (double)(v[b] + dv * t);
  }
  pts[i * (D + 1) + D] = wt;
}

}  // namespace

struct WarpRec {
  int D = 0;
  float alpha = WALPHA_DEFAULT;
  DevBuf<float> p, m, v, g, mask, loss;
  DevBuf<__nv_bfloat16> wq;
  DevBuf<float> X, w;
  int64_t t = 0;
  std::vector<float> hmask;
};

void destroy_warps(qiw_ctx *c) {
  for (WarpRec *w : c->warps) {
    w->p.release(); w->m.release(); w->v.release(); w->g.release(); w->mask.release(); w->loss.release();
    w->wq.release(); w->X.release(); w->w.release();
    delete w;
  }
  c->warps.clear();
}

int warp_dim(qiw_ctx *c, int id) { return c->warps[id]->D; }

static size_t train_smem(int D) {
  Layout L(D);
  return sizeof(float) * ((size_t)L.n + WTILE * WDMAX + 4 * WTILE * WH + (size_t)WTILE * L.DK);
}

int warp_map_device(qiw_ctx *c, int id, const uint32_t *m_dev, const uint32_t *x0_dev, uint64_t first, uint64_t n,
                    double *pts_dev) {
  WarpRec *w = c->warps[id];
  const size_t smem = sizeof(float) * Layout(w->D).n;
  cudaFuncSetAttribute(warp_map_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int threads = 128;
  const unsigned blocks = (unsigned)((n + threads - 1) / threads);
  if (blocks == 0) return QIW_OK;
  warp_map_kernel<<<blocks, threads, smem, c->stream>>>(w->wq.p, w->D, w->alpha, m_dev, x0_dev, first, n, pts_dev);
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

static int run_grad(qiw_ctx *c, WarpRec *w, const float *X, const float *wt, int64_t n) {
  const int Lw = Layout(w->D).n;
  const size_t smem = train_smem(w->D);
  cudaFuncSetAttribute(made_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int rc;
  if ((rc = c->cuda(cudaMemsetAsync(w->g.p, 0, sizeof(float) * Lw, c->stream), "warp grad")) ||
      (rc = c->cuda(cudaMemsetAsync(w->loss.p, 0, sizeof(float), c->stream), "warp grad")))
    return rc;
  const unsigned blocks = (unsigned)((n + WTILE - 1) / WTILE);
  made_grad_kernel<<<blocks, 128, smem, c->stream>>>(w->wq.p, w->D, w->alpha, X, wt, (int)n, w->g.p, w->loss.p);
  return c->cuda(cudaGetLastError(), "warp grad kernel");
}

int qiw_warp_grad(qiw_ctx *c, int32_t id, const double *x, const double *wt, int64_t n, double *grad_out,
                  double *loss_out) {
  if (!c || !x || !wt || !grad_out || id < 0 || id >= (int)c->warps.size() || n <= 0) return QIW_ERR_ARG;
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_warp_grad: cudaSetDevice");
  WarpRec *w = c->warps[id];
  int rc = upload_batch(c, w, x, wt, n);
  if (rc || (rc = run_grad(c, w, w->X.p, w->w.p, n))) return rc;
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
  qiw::DeviceScope dev_scope(c->device);
  if (dev_scope.status != cudaSuccess) return c->cuda(dev_scope.status, "qiw_warp_fit: cudaSetDevice");
  WarpRec *w = c->warps[id];
  // whole-set normalisation; minibatch b covers samples [b*batch, (b+1)*batch) cyclically
  int rc = upload_batch(c, w, x, wt, n);
  if (rc) return rc;
  const int Lw = Layout(w->D).n;
  const int64_t nb = std::max<int64_t>(1, n / batch);
  float loss = 0.f;
  for (int s = 0; s < steps; ++s) {
    const int64_t b = s % nb;
    const int64_t lo = b * batch, cnt = std::min<int64_t>(batch, n - lo);
    if ((rc = run_grad(c, w, w->X.p + lo * w->D, w->w.p + lo, cnt))) return rc;
    w->t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)w->t), c2 = 1.f - std::pow(b2, (float)w->t);
    // the minibatch gradient is scaled by n/cnt so its size does not depend on the batch
    const float scale_lr = (float)lr;
    adam_kernel<<<64, 256, 0, c->stream>>>(w->p.p, w->m.p, w->v.p, w->g.p, w->mask.p, w->wq.p, Lw, scale_lr, b1, b2,
                                           1e-8f, c1, c2);
    if ((rc = c->cuda(cudaGetLastError(), "adam kernel"))) return rc;
  }
  if (final_loss) {
    if ((rc = run_grad(c, w, w->X.p, w->w.p, n)) ||
        (rc = c->cuda(cudaMemcpyAsync(&loss, w->loss.p, sizeof(float), cudaMemcpyDeviceToHost, c->stream), "warp")) ||
        (rc = c->cuda(cudaStreamSynchronize(c->stream), "warp")))
      return rc;
    *final_loss = loss;
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
