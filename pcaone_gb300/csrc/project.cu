// Projection of new samples onto a fit (run_projection, src/Projection.cpp:
// 236-247): the loaded genotypes are decoded, centred and standardised with
// the fit's allele frequencies (a per-SNP FP64 table, as the reference reads F
// from the .mbim, src/Data.cpp:17-32), then
//   mode 1: U = X B with B = V S^-1 (missing genotypes at the mean, 0), and
//   mode 2: per sample the least-squares solution of (V S) x = g over its
//           observed SNPs (solve_projection_scores, src/Projection.cpp:
//           159-178), through the normal equations
//           (B^T B - sum_{j missing} B_j B_j^T) x = (X B)_i,  B = V S,
//           since X is 0 at missing genotypes.
// FP64 throughout: projection is a single pass, off the RSVD hot path.
#include "internal.cuh"

namespace pcaone {

namespace {

constexpr int kProjMaxK = 32;
constexpr int kTileSnps = 32;

// part[s][i][q] = sum over SNPs of split s of x_ij B[j][q]; one thread per
// sample (128 per CTA), SNP tiles of 32 staged in shared memory with their
// decode tables
__global__ void __launch_bounds__(128) k_project_rhs(BedView v, const double* __restrict__ lut64,
                                                     const double* __restrict__ B, int k, int64_t per,
                                                     double* __restrict__ part, int npad) {
  __shared__ double Bs[kTileSnps][kProjMaxK];
  __shared__ double Ls[kTileSnps][4];
  const int i = blockIdx.x * 128 + threadIdx.x;
  const int64_t j0 = (int64_t)blockIdx.y * per;
  const int64_t j1 = j0 + per < v.nsnps ? j0 + per : v.nsnps;
  double acc[kProjMaxK];
#pragma unroll
  for (int q = 0; q < kProjMaxK; ++q) acc[q] = 0.0;
  for (int64_t jt = j0; jt < j1; jt += kTileSnps) {
    const int nt = (int)(j1 - jt < kTileSnps ? j1 - jt : kTileSnps);
    __syncthreads();
    for (int e = threadIdx.x; e < kTileSnps * kProjMaxK; e += 128) {
      const int jj = e / kProjMaxK, q = e % kProjMaxK;
      Bs[jj][q] = (jj < nt && q < k) ? B[(jt + jj) * k + q] : 0.0;
    }
    for (int e = threadIdx.x; e < kTileSnps * 4; e += 128) {
      const int jj = e / 4;
      Ls[jj][e % 4] = jj < nt ? lut64[(jt + jj) * 4 + (e % 4)] : 0.0;
    }
    __syncthreads();
    if (i < v.nsamples) {
      for (int jj = 0; jj < nt; ++jj) {
        const uint32_t code = (v.bed[(jt + jj) * v.stride + (i >> 2)] >> (2 * (i & 3))) & 3u;
        const double x = Ls[jj][code];
#pragma unroll
        for (int q = 0; q < kProjMaxK; ++q)
          if (q < k) acc[q] = fma(x, Bs[jj][q], acc[q]);
      }
    }
  }
  if (i >= v.nsamples) return;
  double* dst = part + ((size_t)blockIdx.y * npad + i) * k;
#pragma unroll
  for (int q = 0; q < kProjMaxK; ++q)
    if (q < k) dst[q] = acc[q];
}

__global__ void k_project_reduce(const double* __restrict__ part, int nsplit, int N, int npad, int k,
                                 double* __restrict__ R) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)N * k) return;
  const int64_t i = idx / k;
  const int q = (int)(idx % k);
  double s = 0.0;
  for (int t = 0; t < nsplit; ++t) s += part[((size_t)t * npad + i) * k + q];
  R[idx] = s;
}

// One warp per sample: K_i = K - sum over its missing SNPs of B_j B_j^T
// (k x k in shared memory), Cholesky K_i = L L^T (columns in turn, rows
// across the lanes), then L y = r and L^T x = y.  A sample whose K_i is not
// positive definite gets NaN scores.
__global__ void k_project_solve(const double* __restrict__ K, const double* __restrict__ B, int k,
                                const int64_t* __restrict__ ptr, const int32_t* __restrict__ pos,
                                const double* __restrict__ R, int N, double* __restrict__ X) {
  extern __shared__ double sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + warp;
  double* Ki = sm + (size_t)warp * (k * k + k);
  double* y = Ki + k * k;
  if (i >= N) return;
  for (int e = lane; e < k * k; e += 32) Ki[e] = K[e];
  __syncwarp();
  for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e) {
    const double* b = B + (int64_t)pos[e] * k;
    for (int t = lane; t < k * k; t += 32) Ki[t] -= b[t / k] * b[t % k];
  }
  __syncwarp();
  bool ok = true;
  for (int c = 0; c < k; ++c) {
    double d = Ki[c * k + c];
    ok = ok && d > 0.0;
    d = sqrt(fmax(d, 1e-300));
    __syncwarp();
    if (lane == 0) Ki[c * k + c] = d;
    for (int r = c + 1 + lane; r < k; r += 32) Ki[r * k + c] /= d;
    __syncwarp();
    for (int r = c + 1 + lane; r < k; r += 32)
      for (int t = c + 1; t <= r; ++t) Ki[r * k + t] -= Ki[r * k + c] * Ki[t * k + c];
    __syncwarp();
  }
  if (lane == 0) {
    for (int r = 0; r < k; ++r) {
      double s = R[(int64_t)i * k + r];
      for (int t = 0; t < r; ++t) s -= Ki[r * k + t] * y[t];
      y[r] = s / Ki[r * k + r];
    }
    for (int r = k - 1; r >= 0; --r) {
      double s = y[r];
      for (int t = r + 1; t < k; ++t) s -= Ki[t * k + r] * y[t];
      y[r] = s / Ki[r * k + r];
    }
    for (int r = 0; r < k; ++r) X[(int64_t)i * k + r] = ok ? y[r] : __longlong_as_double(0x7ff8000000000000ll);
  }
}

}  // namespace

int project_max_k() { return kProjMaxK; }

void launch_project_rhs(const BedView& v, const double* lut64, const double* B, int k, int npad, double* part,
                        int nsplit, double* R, cudaStream_t s) {
  const int64_t per = (v.nsnps + nsplit - 1) / nsplit;
  dim3 grid(npad / 128, nsplit);
  k_project_rhs<<<grid, 128, 0, s>>>(v, lut64, B, k, per, part, npad);
  PCAONE_LAUNCH_CHECK();
  k_project_reduce<<<ceil_div((int64_t)v.nsamples * k, 256), 256, 0, s>>>(part, nsplit, v.nsamples, npad, k, R);
  PCAONE_LAUNCH_CHECK();
}

void launch_project_solve(const double* K, const double* B, int k, const int64_t* ptr, const int32_t* pos,
                          const double* R, int N, double* X, cudaStream_t s) {
  const int warps = 4;
  const size_t smem = (size_t)warps * (k * k + k) * sizeof(double);
  k_project_solve<<<ceil_div(N, warps), warps * 32, smem, s>>>(K, B, k, ptr, pos, R, N, X);
  PCAONE_LAUNCH_CHECK();
}

}  // namespace pcaone
