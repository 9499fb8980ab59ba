// Learned warm start for the EM imputation: a small MLP, trained on the GPU by
// the kernels of this file, that predicts the centred genotype of a missing
// entry.  Its predictions replace the first EM fill (the mean-imputed start of
// src/Halko.cpp:290-320 and src/Data.cpp:318-348); EM then iterates as usual,
// so plain EM remains the reference the warm start must agree with.
//
// Network (all layers dense, ReLU between them):
//   x[64] -> 256 -> 256 -> 1,  out = centred dosage d/2 - f (clamped like EM)
// Weights are kept in FP32 (Adam state, updates) and rounded to BF16 for the
// forward pass; every product accumulates in FP32.  The gradient is taken with
// respect to the BF16-rounded weights the forward pass used.
//
// Input features of entry (position p, sample i), SNP s = perm[p]:
//   [0, 32)   centred dosages d/2 - f of sample i at the 16 SNPs before and
//             the 16 after s in file order (missing or outside -> 0)
//   [32, 32+q) sqrt(N) * U[i][0..q)   the sample's top-q scores
//   [32+q, 32+2q) sqrt(M) * V[p][0..q) the SNP's top-q loadings
//   [32+2q]   2 f_s - 1
//   [33+2q]   the sample's fraction of missing genotypes
//   [34+2q]   the SNP's fraction of missing genotypes
// with q = min(k, 14); the rest is zero.  The two missing fractions let the
// network undo the shrinkage that mean imputation gives the scores of samples
// (and loadings of SNPs) with many missing genotypes.
//
// Parameter vector layout (FP32, kParams entries):
//   W1 [64 x 256] (row = input), b1 [256], W2 [256 x 256], b2 [256],
//   w3 [256], b3 [1]
#include <cuda_bf16.h>

#include <cmath>
#include <vector>

#include "internal.cuh"
#include "mlp.cuh"

namespace pcaone {
namespace mlp {

namespace {

constexpr int kTile = 64, kTileK = 16;

__device__ __forceinline__ float ld_f(const float* p) { return *p; }
__device__ __forceinline__ float ld_f(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// C[M x N] (ldc) = op(A) op(B) (+ bias[n]) (ReLU) (* (mask > 0)), FP32
// accumulation.  op(A)(m,k) = TA ? A[k*lda + m] : A[m*lda + k]; op(B)(k,n) =
// TB ? B[n*ldb + k] : B[k*ldb + n].  64 x 64 tiles, 256 threads, 4 x 4 outputs
// per thread.
template <typename TA_t, typename TB_t, bool TA, bool TB>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const TA_t* __restrict__ A, int lda,
                                              const TB_t* __restrict__ B, int ldb, float* __restrict__ C, int ldc,
                                              const float* __restrict__ bias, int relu,
                                              const float* __restrict__ mask) {
  __shared__ float As[kTileK][kTile + 4];
  __shared__ float Bs[kTileK][kTile + 4];
  const int tid = threadIdx.x;
  const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
  const int tm = (tid >> 4) * 4, tn = (tid & 15) * 4;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kTileK) {
    for (int e = tid; e < kTile * kTileK; e += 256) {
      // A tile: row m (0..63), column k (0..15)
      const int mm = TA ? (e % kTile) : (e / kTileK), kk = TA ? (e / kTile) : (e % kTileK);
      const int gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < K) v = ld_f(TA ? A + (size_t)gk * lda + gm : A + (size_t)gm * lda + gk);
      As[kk][mm] = v;
      const int nn = TB ? (e / kTileK) : (e % kTile), kb = TB ? (e % kTileK) : (e / kTile);
      const int gn = n0 + nn, gkb = k0 + kb;
      float w = 0.f;
      if (gn < N && gkb < K) w = ld_f(TB ? B + (size_t)gn * ldb + gkb : B + (size_t)gkb * ldb + gn);
      Bs[kb][nn] = w;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTileK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tm + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tn + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + tm + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tn + j;
      if (n >= N) continue;
      float v = acc[i][j];
      if (bias) v += bias[n];
      if (relu) v = fmaxf(v, 0.f);
      if (mask && !(mask[(size_t)m * ldc + n] > 0.f)) v = 0.f;
      C[(size_t)m * ldc + n] = v;
    }
  }
}

template <typename TA_t, typename TB_t, bool TA, bool TB>
void gemm(int M, int N, int K, const TA_t* A, int lda, const TB_t* B, int ldb, float* C, int ldc, const float* bias,
          bool relu, const float* mask, cudaStream_t s) {
  dim3 grid(ceil_div(N, kTile), ceil_div(M, kTile));
  k_gemm<TA_t, TB_t, TA, TB><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, relu ? 1 : 0, mask);
  PCAONE_LAUNCH_CHECK();
}

// out[n] = sum over rows of A[rows x N] (column sums; one thread per column
// and row block, then a second pass over the blocks keeps the order fixed)
__global__ void k_colsum(const float* __restrict__ A, int rows, int N, float* __restrict__ out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += A[(size_t)r * N + n];
  out[n] = s;
}

// d_out = 2 (out - y) / B; per-row squared errors for the loss
__global__ void k_mse_grad(const float* __restrict__ out, const float* __restrict__ y, int B, float* __restrict__ dout,
                           float* __restrict__ sq) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= B) return;
  const float e = out[r] - y[r];
  dout[r] = 2.f * e / (float)B;
  sq[r] = e * e;
}

// dZ2 = (d_out outer w3) * (Z2 > 0)
__global__ void k_outer_mask(const float* __restrict__ dout, const __nv_bfloat16* __restrict__ w3, const float* __restrict__ z,
                             int B, int H, float* __restrict__ dz) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)B * H) return;
  const int r = (int)(idx / H), h = (int)(idx % H);
  dz[idx] = z[idx] > 0.f ? dout[r] * __bfloat162float(w3[h]) : 0.f;
}

__global__ void k_sum(const float* __restrict__ a, int n, float* __restrict__ out) {
  __shared__ float red[256];
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += 256) s += a[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// Adam (Kingma & Ba 2015) on the FP32 parameters, then their BF16 copies
__global__ void k_adam(float* __restrict__ theta, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  theta[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_to_bf16(const float* __restrict__ a, __nv_bfloat16* __restrict__ b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = __float2bfloat16_rn(a[i]);
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

__device__ __forceinline__ uint32_t code_at(const uint8_t* bed, int64_t stride, int64_t row, int i) {
  return (bed[row * stride + (i >> 2)] >> (2 * (i & 3))) & 3u;
}

// Draws `count` observed entries (code != 01) at random: candidate t of draw r
// is (position, sample) from a hash of (seed, r, t); the first observed one of
// up to 16 candidates is taken (entries are (-1, -1) if none was observed).
__global__ void k_draw_observed(const uint8_t* __restrict__ bed, int64_t stride, int64_t nsnps, int nsamples,
                                const int32_t* __restrict__ perm, uint64_t seed, int count, int32_t* __restrict__ pos,
                                int32_t* __restrict__ sample) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= count) return;
  int32_t bp = -1, bs = -1;
  for (int t = 0; t < 16; ++t) {
    const uint64_t h = mix64(seed ^ mix64(((uint64_t)r << 4) | (uint64_t)t));
    const int64_t p = (int64_t)(h % (uint64_t)nsnps);
    const int i = (int)((h >> 32) % (uint64_t)nsamples);
    const int64_t snp = perm ? (int64_t)perm[p] : p;
    if (code_at(bed, stride, snp, i) != 1u) {
      bp = (int32_t)p;
      bs = i;
      break;
    }
  }
  pos[r] = bp;
  sample[r] = bs;
}

// BED2GENO on the centred scale: d/2 - f (missing -> 0)
__device__ __forceinline__ float centred(uint32_t code, double f) {
  if (code == 1u) return 0.f;
  const double g = code == 0u ? 1.0 : (code == 2u ? 0.5 : 0.0);
  return (float)(g - f);
}

__global__ void k_features(FeatureArgs a, const int32_t* __restrict__ pos, const int32_t* __restrict__ sample,
                           int count, float* __restrict__ X, float* __restrict__ y) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)count * kIn) return;
  const int r = (int)(idx / kIn), c = (int)(idx % kIn);
  const int64_t p = pos[r];
  const int i = sample[r];
  float v = 0.f;
  if (p >= 0) {
    const int64_t s = a.perm ? (int64_t)a.perm[p] : p;
    if (c < 32) {
      const int64_t s2 = s + (c < 16 ? c - 16 : c - 15);
      if (s2 >= 0 && s2 < a.nsnps) v = centred(code_at(a.bed, a.stride, s2, i), a.F[s2]);
    } else if (c < 32 + a.q) {
      v = (float)(a.U[(size_t)i * a.k + (c - 32)] * a.sqrt_n);
    } else if (c < 32 + 2 * a.q) {
      v = (float)(a.V[(size_t)p * a.k + (c - 32 - a.q)] * a.sqrt_m);
    } else if (c == 32 + 2 * a.q) {
      v = (float)(2.0 * a.F[s] - 1.0);
    } else if (c == 33 + 2 * a.q) {
      v = a.smiss[i];
    } else if (c == 34 + 2 * a.q) {
      v = (float)a.counts[s * 4 + 1] / (float)a.nsamples;
    }
    if (y && c == 0) y[r] = centred(code_at(a.bed, a.stride, s, i), a.F[s]);
  } else if (y && c == 0) {
    y[r] = 0.f;
  }
  X[idx] = v;
}

__global__ void k_sample_missing(const int64_t* __restrict__ ptr, int nwin, int nsamples, int64_t nsnps,
                                 float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsamples) return;
  int64_t n = 0;
  for (int w = 0; w < nwin; ++w) n += ptr[(int64_t)w * nsamples + i + 1] - ptr[(int64_t)w * nsamples + i];
  out[i] = (float)((double)n / (double)nsnps);
}

// fill values of missing entries: the prediction clamped to [-f, 1 - f] (the
// EM fill's range, src/Data.cpp:328)
__global__ void k_fill(const float* __restrict__ out, const int32_t* __restrict__ pos, const int32_t* __restrict__ perm,
                       const double* __restrict__ F, int count, double* __restrict__ value) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= count) return;
  const int64_t p = pos[r];
  const double f = F[perm ? (int64_t)perm[p] : p];
  value[r] = fmin(fmax((double)out[r], -f), 1.0 - f);
}

}  // namespace

Net::Net(cudaStream_t s) : s_(s) {}

Net::~Net() { release(); }

void Net::release() {
  for (void* p : {(void*)theta_, (void*)grad_, (void*)m_, (void*)v_, (void*)wh_, (void*)X_, (void*)y_, (void*)z1_,
                  (void*)z2_, (void*)out_, (void*)dout_, (void*)dz1_, (void*)dz2_, (void*)sq_, (void*)loss_})
    if (p) cudaFree(p);
  theta_ = grad_ = m_ = v_ = X_ = y_ = z1_ = z2_ = out_ = dout_ = dz1_ = dz2_ = sq_ = loss_ = nullptr;
  wh_ = nullptr;
  cap_ = 0;
}

void Net::ensure_batch(int B) {
  if (!theta_) {
    PCAONE_CUDA(cudaMalloc(&theta_, kParams * sizeof(float)));
    PCAONE_CUDA(cudaMalloc(&grad_, kParams * sizeof(float)));
    PCAONE_CUDA(cudaMalloc(&m_, kParams * sizeof(float)));
    PCAONE_CUDA(cudaMalloc(&v_, kParams * sizeof(float)));
    PCAONE_CUDA(cudaMalloc(&wh_, kParams * sizeof(__nv_bfloat16)));
    PCAONE_CUDA(cudaMalloc(&loss_, sizeof(float)));
  }
  if (B <= cap_) return;
  for (void* p : {(void*)X_, (void*)y_, (void*)z1_, (void*)z2_, (void*)out_, (void*)dout_, (void*)dz1_, (void*)dz2_,
                  (void*)sq_})
    if (p) cudaFree(p);
  PCAONE_CUDA(cudaMalloc(&X_, (size_t)B * kIn * sizeof(float)));
  PCAONE_CUDA(cudaMalloc(&y_, (size_t)B * sizeof(float)));
  PCAONE_CUDA(cudaMalloc(&z1_, (size_t)B * kH * sizeof(float)));
  PCAONE_CUDA(cudaMalloc(&z2_, (size_t)B * kH * sizeof(float)));
  PCAONE_CUDA(cudaMalloc(&out_, (size_t)B * sizeof(float)));
  PCAONE_CUDA(cudaMalloc(&dout_, (size_t)B * sizeof(float)));
  PCAONE_CUDA(cudaMalloc(&dz1_, (size_t)B * kH * sizeof(float)));
  PCAONE_CUDA(cudaMalloc(&dz2_, (size_t)B * kH * sizeof(float)));
  PCAONE_CUDA(cudaMalloc(&sq_, (size_t)B * sizeof(float)));
  cap_ = B;
}

void Net::init(uint64_t seed) {
  // He-uniform weights from a host generator (the draw order is the layout
  // order), zero biases
  std::vector<float> h(kParams, 0.f);
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
  auto uni = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return (double)(st >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  };
  const double a1 = std::sqrt(6.0 / kIn), a2 = std::sqrt(6.0 / kH), a3 = std::sqrt(3.0 / kH);
  for (int i = 0; i < kIn * kH; ++i) h[kOffW1 + i] = (float)(a1 * uni());
  for (int i = 0; i < kH * kH; ++i) h[kOffW2 + i] = (float)(a2 * uni());
  for (int i = 0; i < kH; ++i) h[kOffW3 + i] = (float)(a3 * uni());
  set_params(h.data());
  PCAONE_CUDA(cudaMemsetAsync(m_, 0, kParams * sizeof(float), s_));
  PCAONE_CUDA(cudaMemsetAsync(v_, 0, kParams * sizeof(float), s_));
  step_ = 0;
}

void Net::set_params(const float* host) {
  ensure_batch(0);
  PCAONE_CUDA(cudaMemcpyAsync(theta_, host, kParams * sizeof(float), cudaMemcpyHostToDevice, s_));
  refresh_bf16();
}

void Net::refresh_bf16() {
  k_to_bf16<<<ceil_div(kParams, 256), 256, 0, s_>>>(theta_, wh_, kParams);
  PCAONE_LAUNCH_CHECK();
}

void Net::forward(const float* X, int B, bool keep) {
  ensure_batch(B);
  // Z1 = X W1 + b1, A1 = relu(Z1) (the ReLU output is what the next layer and
  // the backward mask read); Z2 likewise; out = A2 w3 + b3
  gemm<float, __nv_bfloat16, false, false>(B, kH, kIn, X, kIn, wh_ + kOffW1, kH, z1_, kH, theta_ + kOffB1, true,
                                           nullptr, s_);
  gemm<float, __nv_bfloat16, false, false>(B, kH, kH, z1_, kH, wh_ + kOffW2, kH, z2_, kH, theta_ + kOffB2, true,
                                           nullptr, s_);
  gemm<float, __nv_bfloat16, false, false>(B, 1, kH, z2_, kH, wh_ + kOffW3, 1, out_, 1, theta_ + kOffB3, false,
                                           nullptr, s_);
  (void)keep;
}

void Net::backward(const float* X, const float* y, int B) {
  k_mse_grad<<<ceil_div(B, 256), 256, 0, s_>>>(out_, y, B, dout_, sq_);
  PCAONE_LAUNCH_CHECK();
  // output layer: g_w3 = A2^T d_out, g_b3 = sum d_out
  gemm<float, float, true, false>(kH, 1, B, z2_, kH, dout_, 1, grad_ + kOffW3, 1, nullptr, false, nullptr, s_);
  k_colsum<<<1, 32, 0, s_>>>(dout_, B, 1, grad_ + kOffB3);
  PCAONE_LAUNCH_CHECK();
  // dZ2 = (d_out w3^T) * (A2 > 0)
  k_outer_mask<<<ceil_div((int64_t)B * kH, 256), 256, 0, s_>>>(dout_, wh_ + kOffW3, z2_, B, kH, dz2_);
  PCAONE_LAUNCH_CHECK();
  // g_W2 = A1^T dZ2, g_b2 = column sums of dZ2
  gemm<float, float, true, false>(kH, kH, B, z1_, kH, dz2_, kH, grad_ + kOffW2, kH, nullptr, false, nullptr, s_);
  k_colsum<<<ceil_div(kH, 128), 128, 0, s_>>>(dz2_, B, kH, grad_ + kOffB2);
  PCAONE_LAUNCH_CHECK();
  // dZ1 = (dZ2 W2^T) * (A1 > 0)
  gemm<float, __nv_bfloat16, false, true>(B, kH, kH, dz2_, kH, wh_ + kOffW2, kH, dz1_, kH, nullptr, false, z1_, s_);
  // g_W1 = X^T dZ1, g_b1 = column sums of dZ1
  gemm<float, float, true, false>(kIn, kH, B, X, kIn, dz1_, kH, grad_ + kOffW1, kH, nullptr, false, nullptr, s_);
  k_colsum<<<ceil_div(kH, 128), 128, 0, s_>>>(dz1_, B, kH, grad_ + kOffB1);
  PCAONE_LAUNCH_CHECK();
  k_sum<<<1, 256, 0, s_>>>(sq_, B, loss_);
  PCAONE_LAUNCH_CHECK();
}

void Net::adam(float lr) {
  ++step_;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)step_), c2 = 1.f - std::pow(b2, (float)step_);
  k_adam<<<ceil_div(kParams, 256), 256, 0, s_>>>(theta_, grad_, m_, v_, kParams, lr, b1, b2, 1e-8f, c1, c2);
  PCAONE_LAUNCH_CHECK();
  refresh_bf16();
}

float Net::loss_host() {
  float l = 0.f;
  PCAONE_CUDA(cudaMemcpyAsync(&l, loss_, sizeof(float), cudaMemcpyDeviceToHost, s_));
  PCAONE_CUDA(cudaStreamSynchronize(s_));
  return l;
}

void draw_observed(const BedView& v, const int32_t* perm, uint64_t seed, int count, int32_t* pos, int32_t* sample,
                   cudaStream_t s) {
  if (count <= 0) return;
  k_draw_observed<<<ceil_div(count, 256), 256, 0, s>>>(v.bed, v.stride, v.nsnps, v.nsamples, perm, seed, count, pos,
                                                       sample);
  PCAONE_LAUNCH_CHECK();
}

void features(const FeatureArgs& a, const int32_t* pos, const int32_t* sample, int count, float* X, float* y,
              cudaStream_t s) {
  if (count <= 0) return;
  k_features<<<ceil_div((int64_t)count * kIn, 256), 256, 0, s>>>(a, pos, sample, count, X, y);
  PCAONE_LAUNCH_CHECK();
}

void sample_missing(const int64_t* bk_ptr, int nwin, int nsamples, int64_t nsnps, float* out, cudaStream_t s) {
  k_sample_missing<<<ceil_div(nsamples, 256), 256, 0, s>>>(bk_ptr, nwin, nsamples, nsnps, out);
  PCAONE_LAUNCH_CHECK();
}

void fill(const float* out, const int32_t* pos, const int32_t* perm, const double* F, int count, double* value,
          cudaStream_t s) {
  if (count <= 0) return;
  k_fill<<<ceil_div(count, 256), 256, 0, s>>>(out, pos, perm, F, count, value);
  PCAONE_LAUNCH_CHECK();
}

}  // namespace mlp
}  // namespace pcaone
