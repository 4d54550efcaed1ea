// Integrand surrogate: a multilayer perceptron with hand-written training and
// inference kernels.
//
// Layers: in -> H -> H -> H -> out, GELU after every hidden layer. The forward
// pass reads BF16 copies of the weights and accumulates in FP32; training keeps
// FP32 master weights and Adam moments and refreshes the BF16 copies after every
// step. All products go through one tiled shared-memory kernel
//   C[m, n] = sum_k A(m, k) B(n, k)   (A, B with arbitrary strides, B in BF16 or FP32)
// used for the forward product, the data gradient and the weight gradient.
//
// Parameter layout (flattened FP32): W1 (H x in), b1 (H), W2 (H x H), b2,
// W3 (H x H), b3, W4 (out x H), b4; W row-major (row = output unit).
#include <cuda_bf16.h>

#include <cmath>
#include <random>

#include "gc_internal.cuh"

struct gc_mlp {
  int in = 0, hid = 0, out = 0;
  int nlayer = 4;
  size_t nparam = 0;
  size_t woff[4], boff[4];
  int din[4], dout[4];
  gc::DevBuf<float> master, grad, m1, m2;
  gc::DevBuf<__nv_bfloat16> wbf;  // BF16 copy of the whole parameter vector
  gc::DevBuf<float> act;           // activations / pre-activations for the largest batch seen
  int act_batch = 0;
  long long step = 0;
};

namespace {

constexpr int T = 16;  // tile edge of the product kernel

__device__ __forceinline__ float load_el(const float *p, long long i) { return p[i]; }
__device__ __forceinline__ float load_el(const __nv_bfloat16 *p, long long i) {
  return __bfloat162float(p[i]);
}

// C[m*ldc + n] (+)= sum_k A[m*sam + k*sak] * B[n*sbn + k*sbk] (+ bias[n]);
// act 1: also writes GELU(C) to H[m*ldc + n] (C keeps the pre-activation).
template <typename TB>
__global__ void k_prod(int M, int N, int K, const float *__restrict__ A, long long sam,
                       long long sak, const TB *__restrict__ B, long long sbn, long long sbk,
                       float *__restrict__ C, long long ldc, const float *__restrict__ bias,
                       int accumulate, int act, float *__restrict__ H) {
  __shared__ float as[T][T + 1], bs[T][T + 1];
  int tx = threadIdx.x, ty = threadIdx.y;
  int m = blockIdx.y * T + ty, n = blockIdx.x * T + tx;
  float acc = 0.f;
  for (int k0 = 0; k0 < K; k0 += T) {
    int ka = k0 + tx;
    as[ty][tx] = (m < M && ka < K) ? A[(long long)m * sam + (long long)ka * sak] : 0.f;
    int nb = blockIdx.x * T + ty;
    bs[ty][tx] = (nb < N && ka < K) ? load_el(B, (long long)nb * sbn + (long long)ka * sbk) : 0.f;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < T; ++k) acc += as[ty][k] * bs[tx][k];
    __syncthreads();
  }
  if (m < M && n < N) {
    long long o = (long long)m * ldc + n;
    float v = acc + (bias ? bias[n] : 0.f);
    if (accumulate) v += C[o];
    C[o] = v;
    if (act) H[o] = 0.5f * v * (1.f + erff(v * 0.70710678118654752f));
  }
}

// dZ = dH * GELU'(Z)
__global__ void k_gelu_bwd(long long total, const float *__restrict__ Z, const float *__restrict__ dH,
                           float *__restrict__ dZ) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    float z = Z[t];
    float g = 0.5f * (1.f + erff(z * 0.70710678118654752f)) +
              z * 0.3989422804014327f * expf(-0.5f * z * z);
    dZ[t] = dH[t] * g;
  }
}

// db[n] = sum_m dZ[m, n]
__global__ void k_colsum(int M, int N, const float *__restrict__ dZ, float *__restrict__ db) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; ++m) s += dZ[(long long)m * N + n];
  db[n] = s;
}

// MSE: loss partials and dY = 2 (Y - T) / (M N)
__global__ void k_mse(long long total, float inv, const float *__restrict__ Y,
                      const float *__restrict__ Tt, float *__restrict__ dY, float *__restrict__ part) {
  __shared__ float red[256];
  float s = 0.f;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    float d = Y[t] - Tt[t];
    s += d * d;
    dY[t] = 2.f * d * inv;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_adam(long long n, float lr, float b1, float b2, float eps, float c1, float c2,
                       float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, __nv_bfloat16 *__restrict__ wbf) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    float gt = g[t];
    float mt = b1 * m[t] + (1.f - b1) * gt;
    float vt = b2 * v[t] + (1.f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    float wt = w[t] - lr * (mt / c1) / (sqrtf(vt / c2) + eps);
    w[t] = wt;
    wbf[t] = __float2bfloat16(wt);
  }
}

__global__ void k_to_bf16(long long n, const float *__restrict__ w, __nv_bfloat16 *__restrict__ o) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    o[t] = __float2bfloat16(w[t]);
}

template <typename TB>
int prod(gc_context *ctx, int M, int N, int K, const float *A, long long sam, long long sak,
         const TB *B, long long sbn, long long sbk, float *C, long long ldc, const float *bias,
         int accumulate, int act, float *H) {
  dim3 grid(gc::ceil_div(N, T), gc::ceil_div(M, T));
  k_prod<TB><<<grid, dim3(T, T), 0, ctx->stream>>>(M, N, K, A, sam, sak, B, sbn, sbk, C, ldc, bias,
                                                   accumulate, act, H);
  GC_LAUNCHED(ctx);
  return GC_OK;
}

// activation workspace: per layer l: Z_l (B x dout), H_l (B x dout); plus dA, dB (B x max)
size_t layer_floats(const gc_mlp *m, int batch) {
  size_t s = 0;
  for (int l = 0; l < m->nlayer; ++l) s += 2 * (size_t)batch * m->dout[l];
  return s;
}

int max_width(const gc_mlp *m) { return std::max(std::max(m->in, m->hid), m->out); }

int ensure_act(gc_context *ctx, gc_mlp *m, int batch) {
  if (batch <= m->act_batch) return GC_OK;
  GC_TRY(m->act.alloc(ctx, layer_floats(m, batch) + 2 * (size_t)batch * max_width(m)));
  m->act_batch = batch;
  return GC_OK;
}

// Forward through all layers; Z_l and H_l (H of the last layer = output) kept in act.
int forward(gc_context *ctx, gc_mlp *m, int B, const float *x, float **Z, float **H) {
  GC_TRY(ensure_act(ctx, m, B));
  float *p = m->act.p;
  const int stride = m->act_batch;
  for (int l = 0; l < m->nlayer; ++l) {
    Z[l] = p;
    p += (size_t)stride * m->dout[l];
    H[l] = p;
    p += (size_t)stride * m->dout[l];
  }
  const float *in = x;
  for (int l = 0; l < m->nlayer; ++l) {
    const bool last = l == m->nlayer - 1;
    GC_TRY(prod(ctx, B, m->dout[l], m->din[l], in, m->din[l], 1, m->wbf.p + m->woff[l],
                (long long)m->din[l], 1, last ? H[l] : Z[l], m->dout[l], m->master.p + m->boff[l],
                0, last ? 0 : 1, H[l]));
    in = H[l];
  }
  return GC_OK;
}

// Loss and gradient of the FP32 master parameters for one batch.
int loss_grad(gc_context *ctx, gc_mlp *m, int B, const float *x, const float *t, float *loss) {
  float *Z[4], *H[4];
  GC_TRY(forward(ctx, m, B, x, Z, H));
  float *dA = m->act.p + layer_floats(m, m->act_batch);
  float *dB = dA + (size_t)m->act_batch * max_width(m);
  const long long nout = (long long)B * m->out;
  const int nb = 64;
  gc::DevBuf<float> part;
  GC_TRY(part.alloc(ctx, nb));
  k_mse<<<nb, 256, 0, ctx->stream>>>(nout, 1.f / (float)nout, H[m->nlayer - 1], t, dA, part.p);
  GC_LAUNCHED(ctx);
  // dA holds dL/dZ of the current layer (the last layer has no activation)
  for (int l = m->nlayer - 1; l >= 0; --l) {
    const float *inp = l == 0 ? x : H[l - 1];
    // dW_l[o, i] = sum_b dZ[b, o] inp[b, i]
    GC_TRY(prod(ctx, m->dout[l], m->din[l], B, dA, 1, m->dout[l], inp, 1, m->din[l],
                m->grad.p + m->woff[l], m->din[l], nullptr, 0, 0, nullptr));
    k_colsum<<<gc::ceil_div(m->dout[l], 128), 128, 0, ctx->stream>>>(B, m->dout[l], dA,
                                                                      m->grad.p + m->boff[l]);
    GC_LAUNCHED(ctx);
    if (l == 0) break;
    // dH_{l-1}[b, i] = sum_o dZ[b, o] W_l[o, i]
    GC_TRY(prod(ctx, B, m->din[l], m->dout[l], dA, m->dout[l], 1, m->wbf.p + m->woff[l], 1,
                m->din[l], dB, m->din[l], nullptr, 0, 0, nullptr));
    long long tot = (long long)B * m->din[l];
    k_gelu_bwd<<<std::min<unsigned>(gc::ceil_div(tot, 256), 4096u), 256, 0, ctx->stream>>>(
        tot, Z[l - 1], dB, dA);
    GC_LAUNCHED(ctx);
  }
  if (loss) {
    float hp[nb];
    GC_CUDA(ctx, cudaMemcpyAsync(hp, part.p, sizeof hp, cudaMemcpyDeviceToHost, ctx->stream));
    GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double s = 0;
    for (int i = 0; i < nb; ++i) s += hp[i];
    *loss = (float)(s / (double)nout);
  }
  return GC_OK;
}

}  // namespace

extern "C" {

int gc_mlp_create(gc_context *ctx, int in_dim, int hidden, int out_dim, unsigned long long seed,
                  gc_mlp **out) {
  if (!ctx || !out || in_dim <= 0 || hidden <= 0 || out_dim <= 0) return GC_EINVAL;
  gc_mlp *m = new gc_mlp();
  m->in = in_dim;
  m->hid = hidden;
  m->out = out_dim;
  int dims[5] = {in_dim, hidden, hidden, hidden, out_dim};
  size_t off = 0;
  for (int l = 0; l < 4; ++l) {
    m->din[l] = dims[l];
    m->dout[l] = dims[l + 1];
    m->woff[l] = off;
    off += (size_t)dims[l] * dims[l + 1];
    m->boff[l] = off;
    off += dims[l + 1];
  }
  m->nparam = off;
  std::vector<float> h(off, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < 4; ++l) {
    std::normal_distribution<float> nd(0.f, 1.f / std::sqrt((float)m->din[l]));
    for (size_t i = 0; i < (size_t)m->din[l] * m->dout[l]; ++i) h[m->woff[l] + i] = nd(rng);
  }
  int r;
  if ((r = m->master.upload(ctx, h.data(), off)) != GC_OK || (r = m->grad.alloc(ctx, off)) != GC_OK ||
      (r = m->m1.alloc(ctx, off)) != GC_OK || (r = m->m2.alloc(ctx, off)) != GC_OK ||
      (r = m->wbf.alloc(ctx, off)) != GC_OK) {
    delete m;
    return r;
  }
  cudaMemsetAsync(m->m1.p, 0, off * 4, ctx->stream);
  cudaMemsetAsync(m->m2.p, 0, off * 4, ctx->stream);
  k_to_bf16<<<gc::ceil_div(off, 256), 256, 0, ctx->stream>>>(off, m->master.p, m->wbf.p);
  ctx->launches++;
  *out = m;
  return GC_OK;
}

int gc_mlp_destroy(gc_mlp *m) {
  delete m;
  return GC_OK;
}

long long gc_mlp_num_params(const gc_mlp *m) { return m ? (long long)m->nparam : 0; }

int gc_mlp_set_params(gc_context *ctx, gc_mlp *m, const float *params_dev) {
  if (!ctx || !m || !params_dev) return GC_EINVAL;
  GC_CUDA(ctx, cudaMemcpyAsync(m->master.p, params_dev, m->nparam * 4, cudaMemcpyDeviceToDevice,
                               ctx->stream));
  k_to_bf16<<<gc::ceil_div(m->nparam, 256), 256, 0, ctx->stream>>>(m->nparam, m->master.p, m->wbf.p);
  GC_LAUNCHED(ctx);
  return GC_OK;
}

int gc_mlp_get_params(gc_context *ctx, gc_mlp *m, float *params_dev) {
  if (!ctx || !m || !params_dev) return GC_EINVAL;
  GC_CUDA(ctx, cudaMemcpyAsync(params_dev, m->master.p, m->nparam * 4, cudaMemcpyDeviceToDevice,
                               ctx->stream));
  return GC_OK;
}

int gc_mlp_forward(gc_context *ctx, gc_mlp *m, int batch, const float *x_dev, float *y_dev) {
  if (!ctx || !m || batch <= 0 || !x_dev || !y_dev) return GC_EINVAL;
  float *Z[4], *H[4];
  GC_TRY(forward(ctx, m, batch, x_dev, Z, H));
  GC_CUDA(ctx, cudaMemcpyAsync(y_dev, H[3], (size_t)batch * m->out * 4, cudaMemcpyDeviceToDevice,
                               ctx->stream));
  return GC_OK;
}

int gc_mlp_gradients(gc_context *ctx, gc_mlp *m, int batch, const float *x_dev, const float *t_dev,
                     float *grad_dev, float *loss_host) {
  if (!ctx || !m || batch <= 0 || !x_dev || !t_dev) return GC_EINVAL;
  GC_TRY(loss_grad(ctx, m, batch, x_dev, t_dev, loss_host));
  if (grad_dev)
    GC_CUDA(ctx, cudaMemcpyAsync(grad_dev, m->grad.p, m->nparam * 4, cudaMemcpyDeviceToDevice,
                                 ctx->stream));
  return GC_OK;
}

int gc_mlp_train_step(gc_context *ctx, gc_mlp *m, int batch, const float *x_dev, const float *t_dev,
                      float lr, float *loss_host) {
  if (!ctx || !m || batch <= 0 || !x_dev || !t_dev || !(lr > 0.f)) return GC_EINVAL;
  GC_TRY(loss_grad(ctx, m, batch, x_dev, t_dev, loss_host));
  m->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
  k_adam<<<std::min<unsigned>(gc::ceil_div(m->nparam, 256), 4096u), 256, 0, ctx->stream>>>(
      m->nparam, lr, b1, b2, 1e-8f, c1, c2, m->master.p, m->grad.p, m->m1.p, m->m2.p, m->wbf.p);
  GC_LAUNCHED(ctx);
  return GC_OK;
}

}  // extern "C"
