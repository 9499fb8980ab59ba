// Learned warm start for the EM imputation (mlp.cu): network, features and
// the training / inference steps.
#pragma once

#include <cuda_bf16.h>

#include "internal.cuh"

namespace pcaone {
namespace mlp {

constexpr int kIn = 64;   // input features (zero padded)
constexpr int kH = 256;   // width of both hidden layers
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kIn * kH;
constexpr int kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH;
constexpr int kOffW3 = kOffB2 + kH;
constexpr int kOffB3 = kOffW3 + kH;
constexpr int kParams = kOffB3 + 1;  // 82,689

// What the feature kernel reads for entry (position p, sample i).
struct FeatureArgs {
  const uint8_t* bed;    // packed genotypes in file order
  int64_t stride;
  int64_t nsnps;
  int nsamples;
  const int32_t* perm;   // position -> SNP (nullptr: identity)
  const double* F;       // allele frequencies (file order)
  const double* U;       // N x k scores (row-major)
  const double* V;       // M x k loadings by position (row-major)
  const float* smiss;    // per sample fraction of missing genotypes
  const int32_t* counts; // per SNP (n00, n01, n10, n11), file order
  int k, q;              // q = min(k, 14) components used
  double sqrt_n, sqrt_m;
};

// The network's parameters, Adam state and activations for batches of up to
// the largest size requested so far.  All work runs on the stream given.
class Net {
 public:
  explicit Net(cudaStream_t s);
  ~Net();
  Net(const Net&) = delete;
  Net& operator=(const Net&) = delete;
  void init(uint64_t seed);
  void set_params(const float* host);            // kParams FP32 values
  void forward(const float* X, int B, bool keep);  // -> out()
  void backward(const float* X, const float* y, int B);  // after forward: grad(), loss
  void adam(float lr);
  float loss_host();                             // sum of squared errors of the last backward
  void ensure_batch(int B);
  float* X() { return X_; }
  float* y() { return y_; }
  const float* out() const { return out_; }
  const float* grad() const { return grad_; }
  const float* params() const { return theta_; }

 private:
  void release();
  void refresh_bf16();
  cudaStream_t s_;
  float *theta_ = nullptr, *grad_ = nullptr, *m_ = nullptr, *v_ = nullptr;
  __nv_bfloat16* wh_ = nullptr;
  float *X_ = nullptr, *y_ = nullptr, *z1_ = nullptr, *z2_ = nullptr, *out_ = nullptr, *dout_ = nullptr;
  float *dz1_ = nullptr, *dz2_ = nullptr, *sq_ = nullptr, *loss_ = nullptr;
  int cap_ = 0;
  int step_ = 0;
};

// `count` random observed entries (position, sample); -1 where none was found
void draw_observed(const BedView& v, const int32_t* perm, uint64_t seed, int count, int32_t* pos, int32_t* sample,
                   cudaStream_t s);
// X[count x 64] features of the entries and, if y, their centred dosages
void features(const FeatureArgs& a, const int32_t* pos, const int32_t* sample, int count, float* X, float* y,
              cudaStream_t s);
// per sample fraction of missing genotypes from the (window, sample) buckets
void sample_missing(const int64_t* bk_ptr, int nwin, int nsamples, int64_t nsnps, float* out, cudaStream_t s);
// value[r] = out[r] clamped to [-f, 1 - f] of the entry's SNP
void fill(const float* out, const int32_t* pos, const int32_t* perm, const double* F, int count, double* value,
          cudaStream_t s);

}  // namespace mlp
}  // namespace pcaone
