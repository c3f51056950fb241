// Learned bandwidth warm start: summary features and a small MLP
// (32 -> 128 -> 128 -> 3, ReLU) trained and run by this library's own
// kernels. Weights are used in BF16 by the forward and backward passes with
// FP32 accumulation; FP32 master weights and Adam moments are updated on the
// device. The network maps the 32 features of an instance to
// r_j = log(h_amise_j / h0_j) per dimension, which warm-starts the AMISE
// bandwidth search (ENT_HEST_AMISE_WARM).
//
// Feature layout (32 floats per instance of dimension d <= 3):
//   [0..17]  per dimension j (slots j >= d are zero): mean, sd, skewness,
//            excess kurtosis, mean and sd of the 1-D distance to the 8th
//            nearest neighbour divided by sd                 (6 x 3)
//   [18..26] quantiles 0.1 .. 0.9 of dimension 0, standardised (9)
//   [27]     log(n)
//   [28]     d
//   [29..31] validity mask of dimensions 0..2
//
// The GEMMs here are at most 128 x 128 x B; they run on the CUDA cores
// (a few MFLOP per step) -- negligible beside the pair kernels.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/entropical_gb300.h"
#include "api_internal.h"
#include "engine.h"

using namespace ent;

namespace {

constexpr int NI = 32, NH = 128, NO = 3;
constexpr float FEAT_CLIP = 6.f;
constexpr size_t OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NI, OFF_W2 = OFF_B1 + NH,
                 OFF_B2 = OFF_W2 + NH * NH, OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NO * NH,
                 N_PARAMS = OFF_B3 + NO;  // 21,123

// ------------------------------------------------------------- features
struct FeatDim {
  const float* x;       // instance dimension (device)
  const uint32_t* ord;  // value order of x (device)
  uint32_t n;
  uint32_t inst, dim, d;
};

__global__ void __launch_bounds__(256) k_features(const FeatDim* __restrict__ dims,
                                                  float* __restrict__ feat) {
  const FeatDim F = dims[blockIdx.x];
  __shared__ double red[8][6];
  const uint32_t n = F.n;
  // pass 1: mean
  double s1 = 0.0;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) s1 += F.x[i];
  for (int o = 16; o; o >>= 1) s1 += __shfl_xor_sync(0xffffffffu, s1, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][0] = s1;
  __syncthreads();
  double mean = 0.0;
  for (int w = 0; w < 8; ++w) mean += red[w][0];
  mean /= (double)n;
  __syncthreads();
  // pass 2: central moments and the 8-NN distance along the sorted order
  double m2 = 0, m3 = 0, m4 = 0, k1 = 0, k2 = 0;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double dv = (double)F.x[i] - mean;
    const double d2 = dv * dv;
    m2 += d2;
    m3 += d2 * dv;
    m4 += d2 * d2;
    // k = 8 nearest neighbours among the sorted neighbours on both sides
    const float xi = F.x[F.ord[i]];
    int l = (int)i - 1, r = (int)i + 1;
    float dk = 0.f;
    for (int k = 0; k < 8 && (l >= 0 || r < (int)n); ++k) {
      const float dl = l >= 0 ? xi - F.x[F.ord[l]] : INFINITY;
      const float dr = r < (int)n ? F.x[F.ord[r]] - xi : INFINITY;
      if (dl <= dr) {
        dk = dl;
        --l;
      } else {
        dk = dr;
        ++r;
      }
    }
    k1 += dk;
    k2 += (double)dk * dk;
  }
  double v[5] = {m2, m3, m4, k1, k2};
  for (int q = 0; q < 5; ++q)
    for (int o = 16; o; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
  if ((threadIdx.x & 31) == 0)
    for (int q = 0; q < 5; ++q) red[threadIdx.x >> 5][q] = v[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[5] = {0, 0, 0, 0, 0};
    for (int w = 0; w < 8; ++w)
      for (int q = 0; q < 5; ++q) t[q] += red[w][q];
    const double var = t[0] / n, sd = sqrt(fmax(var, 1e-300));
    float* f = feat + (size_t)F.inst * NI;
    f[6 * F.dim + 0] = (float)mean;
    f[6 * F.dim + 1] = (float)sd;
    f[6 * F.dim + 2] = (float)(t[1] / n / (sd * sd * sd));
    f[6 * F.dim + 3] = (float)(t[2] / n / (var * var) - 3.0);
    const double km = t[3] / n;
    f[6 * F.dim + 4] = (float)(km / sd);
    f[6 * F.dim + 5] = (float)(sqrt(fmax(t[4] / n - km * km, 0.0)) / sd);
    if (F.dim == 0) {
      for (int q = 1; q <= 9; ++q) {
        const uint32_t k = (uint32_t)(((uint64_t)q * (n - 1)) / 10);
        f[18 + q - 1] = (float)(((double)F.x[F.ord[k]] - mean) / sd);
      }
      f[27] = (float)log((double)n);
      f[28] = (float)F.d;
      for (int j = 0; j < 3; ++j) f[29 + j] = j < (int)F.d ? 1.f : 0.f;
    }
  }
}

// ------------------------------------------------------------------ GEMM
// C[M x N] = op(A) op(B) (+ bias[N]) with optional ReLU; FP32 accumulate.
// A is FP32 (activations), B is BF16 (weights) or FP32 (activations).
template <typename TB, bool TA, bool TB_>
__global__ void __launch_bounds__(256)
    k_gemm(int M, int N, int K, const float* __restrict__ A, int lda,
           const TB* __restrict__ B, int ldb, float* __restrict__ C, int ldc,
           const float* __restrict__ bias, int relu) {
  __shared__ float sa[16][17], sb[16][17];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int row = blockIdx.y * 16 + ty, col = blockIdx.x * 16 + tx;
  float acc = 0.f;
  for (int k0 = 0; k0 < K; k0 += 16) {
    {  // A tile: rows blockIdx.y*16 + ty, k = k0 + tx
      const int r = blockIdx.y * 16 + ty, k = k0 + tx;
      float v = 0.f;
      if (r < M && k < K) v = TA ? A[(size_t)k * lda + r] : A[(size_t)r * lda + k];
      sa[ty][tx] = v;
    }
    {  // B tile: k = k0 + ty, col
      const int k = k0 + ty, cc = blockIdx.x * 16 + tx;
      float v = 0.f;
      if (k < K && cc < N) {
        const TB b = TB_ ? B[(size_t)cc * ldb + k] : B[(size_t)k * ldb + cc];
        v = (float)b;
      }
      sb[ty][tx] = v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) acc = fmaf(sa[ty][k], sb[k][tx], acc);
    __syncthreads();
  }
  if (row < M && col < N) {
    if (bias) acc += bias[col];
    if (relu) acc = fmaxf(acc, 0.f);
    C[(size_t)row * ldc + col] = acc;
  }
}

template <typename TB, bool TA, bool TB_>
void gemm(cudaStream_t s, int M, int N, int K, const float* A, int lda, const TB* B, int ldb,
          float* C, int ldc, const float* bias, int relu) {
  dim3 g((N + 15) / 16, (M + 15) / 16);
  k_gemm<TB, TA, TB_><<<g, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, relu);
}

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ q, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    q[i] = __float2bfloat16_rn(p[i]);
}

// dY = 2 mask (Y - T) / sum(mask); loss = sum(mask (Y - T)^2) / sum(mask)
__global__ void k_loss_grad(const float* __restrict__ Y, const float* __restrict__ T,
                            const float* __restrict__ Mk, int B, float* __restrict__ dY,
                            float* __restrict__ loss) {
  __shared__ double s_l[8], s_m[8];
  double l = 0.0, m = 0.0;
  for (int i = threadIdx.x; i < B * NO; i += blockDim.x) {
    m += Mk[i];
    const double e = (double)Y[i] - T[i];
    l += Mk[i] * e * e;
  }
  for (int o = 16; o; o >>= 1) {
    l += __shfl_xor_sync(0xffffffffu, l, o);
    m += __shfl_xor_sync(0xffffffffu, m, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_l[threadIdx.x >> 5] = l;
    s_m[threadIdx.x >> 5] = m;
  }
  __syncthreads();
  double lt = 0, mt = 0;
  for (int w = 0; w < 8; ++w) {
    lt += s_l[w];
    mt += s_m[w];
  }
  mt = fmax(mt, 1.0);
  for (int i = threadIdx.x; i < B * NO; i += blockDim.x)
    dY[i] = (float)(2.0 * Mk[i] * ((double)Y[i] - T[i]) / mt);
  if (threadIdx.x == 0) *loss = (float)(lt / mt);
}

// dH *= [H > 0] (ReLU derivative from the post-activation)
__global__ void k_relu_back(float* __restrict__ dH, const float* __restrict__ H, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (!(H[i] > 0.f)) dH[i] = 0.f;
}

// bias gradient: column sums of dH [B x N]
__global__ void k_colsum(const float* __restrict__ dH, int B, int N, float* __restrict__ g) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  float a = 0.f;
  for (int b = 0; b < B; ++b) a += dH[(size_t)b * N + c];
  g[c] = a;
}

__global__ void k_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, int n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_normalize(float* __restrict__ X, const float* __restrict__ mu,
                            const float* __restrict__ sd, int B) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B * NI; i += gridDim.x * blockDim.x) {
    const int f = i % NI;
    // standardised and clipped: heavy-tailed features (kurtosis of narrow
    // mixtures) must not dominate the first layer
    X[i] = fminf(fmaxf((X[i] - mu[f]) / sd[f], -FEAT_CLIP), FEAT_CLIP);
  }
}

}  // namespace

// A network on the device: FP32 masters, BF16 working copy, Adam state,
// feature normalisation.
struct ent_mlp {
  int device = 0;
  float* p = nullptr;           // N_PARAMS FP32 masters
  __nv_bfloat16* pb = nullptr;  // BF16 copy used by the passes
  float* m = nullptr;
  float* v = nullptr;
  float* g = nullptr;
  float* mu = nullptr;  // feature normalisation (32 + 32)
  float* sd = nullptr;
  int step = 0;
  // scratch for a batch
  float *X = nullptr, *H1 = nullptr, *H2 = nullptr, *Y = nullptr, *T = nullptr, *Mk = nullptr,
        *dY = nullptr, *dH1 = nullptr, *dH2 = nullptr, *loss = nullptr;
  size_t cap = 0;
};

namespace {

int mlp_reserve(Ctx& c, ent_mlp* n, size_t B) {
  if (B <= n->cap) return ENT_OK;
  float** bufs[] = {&n->X, &n->H1, &n->H2, &n->Y, &n->T, &n->Mk, &n->dY, &n->dH1, &n->dH2};
  for (float** b : bufs)
    if (*b) cudaFree(*b);
  const size_t sz[] = {NI, NH, NH, NO, NO, NO, NO, NH, NH};
  for (int i = 0; i < 9; ++i)
    if (cudaMalloc(bufs[i], sizeof(float) * B * sz[i]) != cudaSuccess) {
      cudaGetLastError();
      n->cap = 0;
      return c.fail(ENT_ERR_CUDA, "out of device memory (mlp)");
    }
  n->cap = B;
  return ENT_OK;
}

void sync_bf16(cudaStream_t s, ent_mlp* n) {
  k_to_bf16<<<64, 256, 0, s>>>(n->p, n->pb, (int)N_PARAMS);
}

// forward of B normalised rows already in n->X
void forward(cudaStream_t s, ent_mlp* n, int B) {
  const __nv_bfloat16* w = n->pb;
  gemm<__nv_bfloat16, false, true>(s, B, NH, NI, n->X, NI, w + OFF_W1, NI, n->H1, NH,
                                   n->p + OFF_B1, 1);
  gemm<__nv_bfloat16, false, true>(s, B, NH, NH, n->H1, NH, w + OFF_W2, NH, n->H2, NH,
                                   n->p + OFF_B2, 1);
  gemm<__nv_bfloat16, false, true>(s, B, NO, NH, n->H2, NH, w + OFF_W3, NH, n->Y, NO,
                                   n->p + OFF_B3, 0);
}

// gradients of the masked MSE into n->g
void backward(cudaStream_t s, ent_mlp* n, int B) {
  const __nv_bfloat16* w = n->pb;
  k_loss_grad<<<1, 256, 0, s>>>(n->Y, n->T, n->Mk, B, n->dY, n->loss);
  // layer 3
  gemm<float, true, false>(s, NO, NH, B, n->dY, NO, n->H2, NH, n->g + OFF_W3, NH, nullptr, 0);
  k_colsum<<<1, 32, 0, s>>>(n->dY, B, NO, n->g + OFF_B3);
  gemm<__nv_bfloat16, false, false>(s, B, NH, NO, n->dY, NO, w + OFF_W3, NH, n->dH2, NH,
                                    nullptr, 0);
  k_relu_back<<<64, 256, 0, s>>>(n->dH2, n->H2, B * NH);
  // layer 2
  gemm<float, true, false>(s, NH, NH, B, n->dH2, NH, n->H1, NH, n->g + OFF_W2, NH, nullptr, 0);
  k_colsum<<<1, 128, 0, s>>>(n->dH2, B, NH, n->g + OFF_B2);
  gemm<__nv_bfloat16, false, false>(s, B, NH, NH, n->dH2, NH, w + OFF_W2, NH, n->dH1, NH,
                                    nullptr, 0);
  k_relu_back<<<64, 256, 0, s>>>(n->dH1, n->H1, B * NH);
  // layer 1
  gemm<float, true, false>(s, NH, NI, B, n->dH1, NH, n->X, NI, n->g + OFF_W1, NI, nullptr, 0);
  k_colsum<<<1, 128, 0, s>>>(n->dH1, B, NH, n->g + OFF_B1);
}

int upload_batch(Ctx& c, ent_mlp* n, const float* X, const float* T, const float* Mk, size_t B) {
  int s = mlp_reserve(c, n, B);
  if (s) return s;
  cudaError_t e = cudaMemcpyAsync(n->X, X, sizeof(float) * B * NI, cudaMemcpyHostToDevice,
                                  c.stream);
  if (e == cudaSuccess && T)
    e = cudaMemcpyAsync(n->T, T, sizeof(float) * B * NO, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess && Mk)
    e = cudaMemcpyAsync(n->Mk, Mk, sizeof(float) * B * NO, cudaMemcpyHostToDevice, c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload batch");
  k_normalize<<<64, 256, 0, c.stream>>>(n->X, n->mu, n->sd, (int)B);
  return ENT_OK;
}

}  // namespace

// Features of a batch of device instances (used by the learned hestimate).
int mlp_features_device(Ctx& c, const std::vector<const float*>& base,
                        const std::vector<uint32_t>& n, const std::vector<uint32_t>& d,
                        float* d_feat) {
  std::vector<ViewSpec> views;
  std::vector<FeatDim> fd;
  for (size_t q = 0; q < base.size(); ++q)
    for (uint32_t j = 0; j < d[q]; ++j) {
      views.push_back({base[q] + (size_t)j * n[q], n[q]});
      FeatDim f;
      f.x = base[q] + (size_t)j * n[q];
      f.ord = nullptr;
      f.n = n[q];
      f.inst = (uint32_t)q;
      f.dim = j;
      f.d = d[q];
      fd.push_back(f);
    }
  SortedViews sv;
  int s = sort_views(c, views, &sv);
  if (s) return s;
  for (size_t k = 0; k < fd.size(); ++k) fd[k].ord = sv.perm + sv.off[k];
  FeatDim* dfd = static_cast<FeatDim*>(c.arena.alloc(sizeof(FeatDim) * fd.size()));
  if (!dfd) return c.fail(ENT_ERR_CUDA, "out of device memory");
  cudaError_t e = cudaMemcpyAsync(dfd, fd.data(), sizeof(FeatDim) * fd.size(),
                                  cudaMemcpyHostToDevice, c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload feature jobs");
  cudaMemsetAsync(d_feat, 0, sizeof(float) * NI * base.size(), c.stream);
  k_features<<<(unsigned)fd.size(), 256, 0, c.stream>>>(dfd, d_feat);
  c.stats.kernel_launches += 1;
  if ((e = cudaGetLastError()) != cudaSuccess) return c.cuda_fail(e, "features");
  return ENT_OK;
}

// Forward pass on device features (normalised in place).
int mlp_forward_device(Ctx& c, ent_mlp* n, float* d_feat, size_t B, float* d_out) {
  int s = mlp_reserve(c, n, B);
  if (s) return s;
  cudaMemcpyAsync(n->X, d_feat, sizeof(float) * B * NI, cudaMemcpyDeviceToDevice, c.stream);
  k_normalize<<<64, 256, 0, c.stream>>>(n->X, n->mu, n->sd, (int)B);
  forward(c.stream, n, (int)B);
  cudaMemcpyAsync(d_out, n->Y, sizeof(float) * B * NO, cudaMemcpyDeviceToDevice, c.stream);
  c.stats.kernel_launches += 4;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ENT_OK : c.cuda_fail(e, "mlp forward");
}

extern "C" {

size_t ent_mlp_param_count(void) { return N_PARAMS; }

int ent_mlp_create(ent_ctx* ctx, uint64_t seed, ent_mlp** out) {
  if (!ctx || !out) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  cudaSetDevice(c.device);
  ent_mlp* n = new ent_mlp();
  n->device = c.device;
  if (cudaMalloc(&n->p, 4 * N_PARAMS) != cudaSuccess ||
      cudaMalloc(&n->pb, 2 * N_PARAMS) != cudaSuccess ||
      cudaMalloc(&n->m, 4 * N_PARAMS) != cudaSuccess ||
      cudaMalloc(&n->v, 4 * N_PARAMS) != cudaSuccess ||
      cudaMalloc(&n->g, 4 * N_PARAMS) != cudaSuccess || cudaMalloc(&n->mu, 4 * NI) != cudaSuccess ||
      cudaMalloc(&n->sd, 4 * NI) != cudaSuccess || cudaMalloc(&n->loss, 16) != cudaSuccess) {
    cudaGetLastError();
    delete n;
    return ENT_ERR_CUDA;
  }
  // He initialisation for the ReLU layers, zero biases
  std::vector<float> p(N_PARAMS, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  for (size_t i = 0; i < (size_t)NH * NI; ++i) p[OFF_W1 + i] = nd(rng) * std::sqrt(2.f / NI);
  for (size_t i = 0; i < (size_t)NH * NH; ++i) p[OFF_W2 + i] = nd(rng) * std::sqrt(2.f / NH);
  // the output layer starts at zero: the network begins as the constant
  // predictor b3 and opens its feature paths only where they reduce the loss
  for (size_t i = 0; i < (size_t)NO * NH; ++i) p[OFF_W3 + i] = 0.f;
  std::vector<float> mu(NI, 0.f), sd(NI, 1.f);
  cudaMemcpy(n->p, p.data(), 4 * N_PARAMS, cudaMemcpyHostToDevice);
  cudaMemset(n->m, 0, 4 * N_PARAMS);
  cudaMemset(n->v, 0, 4 * N_PARAMS);
  cudaMemcpy(n->mu, mu.data(), 4 * NI, cudaMemcpyHostToDevice);
  cudaMemcpy(n->sd, sd.data(), 4 * NI, cudaMemcpyHostToDevice);
  sync_bf16(nullptr, n);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    cudaGetLastError();
    return ENT_ERR_CUDA;
  }
  *out = n;
  return ENT_OK;
}

void ent_mlp_destroy(ent_mlp* n) {
  if (!n) return;
  cudaSetDevice(n->device);
  float* bufs[] = {n->p, n->m, n->v, n->g, n->mu, n->sd, n->loss, n->X, n->H1, n->H2,
                   n->Y, n->T, n->Mk, n->dY, n->dH1, n->dH2};
  for (float* b : bufs)
    if (b) cudaFree(b);
  if (n->pb) cudaFree(n->pb);
  delete n;
}

int ent_mlp_set_params(ent_mlp* n, const float* params, const float* feat_mu,
                       const float* feat_sd) {
  if (!n) return ENT_ERR_ARG;
  cudaSetDevice(n->device);
  if (params) cudaMemcpy(n->p, params, 4 * N_PARAMS, cudaMemcpyHostToDevice);
  if (feat_mu) cudaMemcpy(n->mu, feat_mu, 4 * NI, cudaMemcpyHostToDevice);
  if (feat_sd) cudaMemcpy(n->sd, feat_sd, 4 * NI, cudaMemcpyHostToDevice);
  cudaMemset(n->m, 0, 4 * N_PARAMS);
  cudaMemset(n->v, 0, 4 * N_PARAMS);
  n->step = 0;
  sync_bf16(nullptr, n);
  return cudaDeviceSynchronize() == cudaSuccess ? ENT_OK : ENT_ERR_CUDA;
}

int ent_mlp_get_params(const ent_mlp* n, float* params, float* feat_mu, float* feat_sd) {
  if (!n) return ENT_ERR_ARG;
  cudaSetDevice(n->device);
  if (params) cudaMemcpy(params, n->p, 4 * N_PARAMS, cudaMemcpyDeviceToHost);
  if (feat_mu) cudaMemcpy(feat_mu, n->mu, 4 * NI, cudaMemcpyDeviceToHost);
  if (feat_sd) cudaMemcpy(feat_sd, n->sd, 4 * NI, cudaMemcpyDeviceToHost);
  return cudaDeviceSynchronize() == cudaSuccess ? ENT_OK : ENT_ERR_CUDA;
}

int ent_mlp_forward(ent_ctx* ctx, ent_mlp* n, const float* X, size_t B, float* Y) {
  if (!ctx || !n || !X || !Y) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  s = upload_batch(c, n, X, nullptr, nullptr, B);
  if (s) return s;
  forward(c.stream, n, (int)B);
  cudaError_t e = cudaMemcpyAsync(Y, n->Y, sizeof(float) * B * NO, cudaMemcpyDeviceToHost,
                                  c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "mlp forward");
  return c.end_call();
}

int ent_mlp_gradients(ent_ctx* ctx, ent_mlp* n, const float* X, const float* T,
                      const float* mask, size_t B, float* grads, float* loss) {
  if (!ctx || !n || !X || !T || !mask) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  s = upload_batch(c, n, X, T, mask, B);
  if (s) return s;
  forward(c.stream, n, (int)B);
  backward(c.stream, n, (int)B);
  if (grads) cudaMemcpyAsync(grads, n->g, 4 * N_PARAMS, cudaMemcpyDeviceToHost, c.stream);
  if (loss) cudaMemcpyAsync(loss, n->loss, 4, cudaMemcpyDeviceToHost, c.stream);
  return c.end_call();
}

int ent_mlp_train_step(ent_ctx* ctx, ent_mlp* n, const float* X, const float* T,
                       const float* mask, size_t B, float lr, float* loss) {
  if (!ctx || !n || !X || !T || !mask || B == 0) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  s = upload_batch(c, n, X, T, mask, B);
  if (s) return s;
  forward(c.stream, n, (int)B);
  backward(c.stream, n, (int)B);
  n->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)n->step), c2 = 1.f - std::pow(b2, (float)n->step);
  k_adam<<<128, 256, 0, c.stream>>>(n->p, n->m, n->v, n->g, (int)N_PARAMS, lr, b1, b2, 1e-8f, c1,
                                   c2);
  sync_bf16(c.stream, n);
  if (loss) cudaMemcpyAsync(loss, n->loss, 4, cudaMemcpyDeviceToHost, c.stream);
  return c.end_call();
}

int ent_features(ent_ctx* ctx, const ent_instance* inst, size_t n_inst, float* feat) {
  if (!ctx || !inst || !feat) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  std::vector<const float*> base(n_inst);
  std::vector<uint32_t> nn(n_inst), dd(n_inst);
  for (size_t q = 0; q < n_inst; ++q) {
    if (inst[q].d < 1 || inst[q].d > 3) return c.fail(ENT_ERR_DIM, ent_status_string(ENT_ERR_DIM));
    if (inst[q].n < 2 || inst[q].n > 0xffffff00ull) return c.fail(ENT_ERR_ARG, "bad size");
    float* p = static_cast<float*>(c.arena.alloc(4 * inst[q].n * inst[q].d));
    if (!p) return c.fail(ENT_ERR_CUDA, "out of device memory");
    cudaError_t e = cudaMemcpyAsync(p, inst[q].coords, 4 * inst[q].n * inst[q].d,
                                    cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) return c.cuda_fail(e, "copy coordinates");
    base[q] = p;
    nn[q] = (uint32_t)inst[q].n;
    dd[q] = inst[q].d;
  }
  float* df = static_cast<float*>(c.arena.alloc(4 * NI * n_inst));
  if (!df) return c.fail(ENT_ERR_CUDA, "out of device memory");
  s = mlp_features_device(c, base, nn, dd, df);
  if (s) return s;
  cudaError_t e = cudaMemcpyAsync(feat, df, 4 * NI * n_inst, cudaMemcpyDeviceToHost, c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "copy features");
  return c.end_call();
}

}  // extern "C"
