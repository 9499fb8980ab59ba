// Arnoldi matvec y = X X^T x that allocates no device memory.
//
// Some callers cannot allocate device memory themselves: hosts whose own
// allocator or memory arena owns every byte of the device, and latency-bound
// loops that cannot afford the device-wide synchronisation cudaMalloc and
// cudaFree may imply.  For them this file provides a variant of the matvec of
// dense64.cu that runs on the caller's own device buffers and keeps its
// intermediates, t = X^T x (one double per SNP) and the per-split partial sums
// of y, in the file-scope array below.  That array is part of the module:
// every GPU that loads the library holds its 16 MiB from module load until
// process exit.
//
// The array is shared by every call on a device and keeps the last call's
// contents; the first kernel overwrites every entry it uses, so nothing has to
// be cleared between calls.  Calls whose work overlaps on the GPU (for example
// from two streams at once) race on the array and must be serialised by the
// caller.
#include <algorithm>
#include <mutex>

#include "../../include/pcaone_gpu.h"
#include "internal.cuh"

namespace pcaone {
namespace noalloc {

constexpr int64_t kMaxSnps = int64_t(1) << 21;  // 2,097,152 SNPs -> 16 MiB of scratch

static __device__ __align__(256) double g_snp_scratch[kMaxSnps];

constexpr int kMaxDevices = 64;
static std::mutex g_mutex;
static double* g_scratch_addr[kMaxDevices];

// Device address of g_snp_scratch on `device` (the current device), resolved
// once per device.  In host code the array's name is only a host-side stand-in,
// never a device address, so kernels get the resolved pointer.
static cudaError_t scratch_on(int device, double** out) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_snp_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[device];
  return cudaSuccess;
}

__device__ __forceinline__ double geno_half(uint32_t code) {
  // BED2GENO on the g/2 scale: 00 -> 1, 10 -> 0.5, 11 -> 0 (01, missing, is skipped)
  return code == 0u ? 1.0 : (code == 2u ? 0.5 : 0.0);
}

__device__ __forceinline__ double snp_scale(double f, int standardize) {
  double s = 1.0;
  if (standardize) {
    const double sd = sqrt(f * (1.0 - f));
    if (sd > 1e-9) s = sqrt(2.0) / sd;
  }
  return s;
}

// t[j] = s_j^2 * sum_i (g_ij - f_j) x_i over the observed samples of SNP j
// (one warp per SNP), so that y_i = sum_j (g_ij - f_j) t[j].
__global__ void k_static_t(const uint8_t* __restrict__ bed, uint64_t pitch, int64_t nsnps, int nsamples,
                           const double* __restrict__ F, int standardize, const double* __restrict__ x,
                           double* __restrict__ t) {
  const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= nsnps) return;
  const double f = F[j];
  const uint8_t* row = bed + j * pitch;
  const int nbytes = (nsamples + 3) >> 2;
  double acc = 0.0;
  for (int b = lane; b < nbytes; b += 32) {
    const uint32_t w = row[b];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = b * 4 + q;
      const uint32_t c = (w >> (2 * q)) & 3u;
      if (i < nsamples && c != 1u) acc = fma(geno_half(c) - f, x[i], acc);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    const double s = snp_scale(f, standardize);
    t[j] = s * s * acc;
  }
}

// y_i = sum_j (g_ij - f_j) t[j] over the SNPs where sample i is observed: one
// thread per sample and SNP range (blockIdx.y of nsplit ranges;
// neighbouring threads read neighbouring bytes of a row), written to y
// directly with one range, else to part[split][i] for k_static_reduce.
__global__ void k_static_y(const uint8_t* __restrict__ bed, uint64_t pitch, int64_t nsnps, int nsamples,
                           const double* __restrict__ F, const double* __restrict__ t, int nsplit,
                           double* __restrict__ part, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsamples) return;
  const int64_t per = (nsnps + nsplit - 1) / nsplit;
  const int64_t j0 = (int64_t)blockIdx.y * per;
  const int64_t j1 = j0 + per < nsnps ? j0 + per : nsnps;
  const int64_t byte = i >> 2;
  const int sh = 2 * (i & 3);
  double acc = 0.0;
  for (int64_t j = j0; j < j1; ++j) {
    const uint32_t c = (bed[j * pitch + byte] >> sh) & 3u;
    if (c != 1u) acc = fma(geno_half(c) - F[j], t[j], acc);
  }
  if (nsplit == 1)
    y[i] = acc;
  else
    part[(size_t)blockIdx.y * nsamples + i] = acc;
}

// y_i = sum over the ranges of part[s][i], in range order (deterministic)
__global__ void k_static_reduce(const double* __restrict__ part, int nsplit, int nsamples, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsamples) return;
  double acc = 0.0;
  for (int s = 0; s < nsplit; ++s) acc += part[(size_t)s * nsamples + i];
  y[i] = acc;
}

}  // namespace noalloc
}  // namespace pcaone

extern "C" int pcaone_gpu_matvec_static(const uint8_t* d_packed, uint64_t row_pitch, uint64_t nsnps,
                                        uint32_t nsamples, const double* d_F, int standardize, const double* d_x,
                                        double* d_y, void* stream) {
  using namespace pcaone::noalloc;
  if (!d_packed || !d_F || !d_x || !d_y || nsnps == 0 || nsamples == 0) return PCAONE_E_ARG;
  if (row_pitch < ((uint64_t)nsamples + 3) / 4) return PCAONE_E_ARG;
  if (nsnps > (uint64_t)kMaxSnps) return PCAONE_E_LIMIT;  // the scratch holds kMaxSnps doubles
  if (nsamples > 0x7fffff00u) return PCAONE_E_LIMIT;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) return PCAONE_E_CUDA;
  double* t = nullptr;
  if (scratch_on(device, &t) != cudaSuccess) return PCAONE_E_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t M = (int64_t)nsnps;
  const int N = (int)nsamples;
  k_static_t<<<(unsigned)((M * 32 + 255) / 256), 256, 0, s>>>(d_packed, row_pitch, M, N, d_F, standardize, d_x, t);
  if (cudaGetLastError() != cudaSuccess) return PCAONE_E_CUDA;
  // SNP ranges for the y pass: enough thread blocks to fill the GPU (about
  // 1216), ranges of at least 32 SNPs, partial sums in the scratch behind t
  const int xblocks = (N + 127) / 128;
  const int64_t room = (kMaxSnps - M) / N;  // partial rows that fit behind t
  int64_t nsplit = std::max<int64_t>(1, (1216 + xblocks - 1) / xblocks);
  nsplit = std::min<int64_t>(nsplit, std::max<int64_t>(1, (M + 31) / 32));
  nsplit = std::min<int64_t>(nsplit, std::max<int64_t>(1, std::min<int64_t>(room, 65535)));
  double* part = t + M;
  k_static_y<<<dim3((unsigned)xblocks, (unsigned)nsplit), 128, 0, s>>>(d_packed, row_pitch, M, N, d_F, t, (int)nsplit,
                                                                       part, d_y);
  if (cudaGetLastError() != cudaSuccess) return PCAONE_E_CUDA;
  if (nsplit > 1) {
    k_static_reduce<<<(unsigned)xblocks, 128, 0, s>>>(part, (int)nsplit, N, d_y);
    if (cudaGetLastError() != cudaSuccess) return PCAONE_E_CUDA;
  }
  return PCAONE_OK;
}
