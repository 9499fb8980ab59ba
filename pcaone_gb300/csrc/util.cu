// Small utility kernels: the missing-genotype list for the EM fill, the sign
// convention flip_UV, and the row-major -> column-major copy of outputs.
#include "internal.cuh"

namespace pcaone {

namespace {

// One warp per position p: missing lanes (code 01) of SNP perm[p], written in
// sample order at rowptr[p] ...
__global__ void k_missing_list(BedView v, const int32_t* __restrict__ perm, const int64_t* __restrict__ rowptr,
                               int32_t* __restrict__ epos, int32_t* __restrict__ sample) {
  const int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (p >= v.nsnps) return;
  const int64_t snp = perm ? (int64_t)perm[p] : p;
  const uint32_t* row = reinterpret_cast<const uint32_t*>(v.bed + snp * v.stride);
  const int nwords = (int)(v.stride >> 2);
  int64_t base = rowptr[p];
  for (int w0 = 0; w0 < nwords; w0 += 32) {
    const int w = w0 + lane;
    const uint32_t word = w < nwords ? row[w] : 0u;
    const uint32_t lo = word & 0x55555555u, hi = (word >> 1) & 0x55555555u;
    uint32_t miss = lo & ~hi;
    const int cnt = __popc(miss);
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    int64_t idx = base + (incl - cnt);
    while (miss) {
      const int b = __ffs(miss) - 1;
      const int i = w * 16 + (b >> 1);
      if (i < v.nsamples) {
        epos[idx] = (int32_t)p;
        sample[idx] = i;
        ++idx;
      }
      miss &= miss - 1u;
    }
    base += __shfl_sync(0xffffffffu, incl, 31);
  }
}

// flip_UV with ubase = false (src/Utils.cpp:118-154): for column c, the entry
// of largest |V| (first on ties) decides; if negative, U[:,c] and V[:,c] flip.
__global__ void k_flip_uv_sign(const double* __restrict__ V, int64_t rows, int k, int* __restrict__ flag) {
  const int c = blockIdx.x;
  __shared__ double bv[256];
  __shared__ int64_t bi[256];
  double best = -1.0;
  int64_t bidx = 0;
  for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) {
    const double a = fabs(V[r * k + c]);
    if (a > best) {
      best = a;
      bidx = r;
    }
  }
  bv[threadIdx.x] = best;
  bi[threadIdx.x] = bidx;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double o = bv[threadIdx.x + s];
      const int64_t oi = bi[threadIdx.x + s];
      if (o > bv[threadIdx.x] || (o == bv[threadIdx.x] && oi < bi[threadIdx.x])) {
        bv[threadIdx.x] = o;
        bi[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) flag[c] = V[bi[0] * k + c] < 0.0 ? -1 : 1;
}

__global__ void k_apply_flag(double* __restrict__ A, int64_t rows, int k, const int* __restrict__ flag) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= rows * k) return;
  if (flag[idx % k] < 0) A[idx] = -A[idx];
}

__global__ void k_transpose_out(const double* __restrict__ A, int64_t rows, int lda, int cols,
                                double* __restrict__ out) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= rows * cols) return;
  const int64_t c = idx / rows, r = idx - c * rows;
  out[idx] = A[r * lda + c];
}

}  // namespace

void launch_missing_list(const BedView& v, const int32_t* perm, const int64_t* rowptr, int32_t* epos,
                         int32_t* sample, cudaStream_t s) {
  if (v.nsnps == 0) return;
  k_missing_list<<<ceil_div(v.nsnps * 32, 256), 256, 0, s>>>(v, perm, rowptr, epos, sample);
  PCAONE_LAUNCH_CHECK();
}

void launch_flip_uv(double* U, int64_t nrows_u, double* V, int64_t nrows_v, int k, int* flag, cudaStream_t s) {
  k_flip_uv_sign<<<k, 256, 0, s>>>(V, nrows_v, k, flag);
  PCAONE_LAUNCH_CHECK();
  k_apply_flag<<<ceil_div(nrows_u * k, 256), 256, 0, s>>>(U, nrows_u, k, flag);
  PCAONE_LAUNCH_CHECK();
  k_apply_flag<<<ceil_div(nrows_v * k, 256), 256, 0, s>>>(V, nrows_v, k, flag);
  PCAONE_LAUNCH_CHECK();
}

void launch_transpose_out(const double* A, int64_t rows, int lda, int cols, double* out, cudaStream_t s) {
  if (rows * cols == 0) return;
  k_transpose_out<<<ceil_div(rows * cols, 256), 256, 0, s>>>(A, rows, lda, cols, out);
  PCAONE_LAUNCH_CHECK();
}

}  // namespace pcaone
