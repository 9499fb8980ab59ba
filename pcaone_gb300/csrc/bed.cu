// PLINK 2-bit genotype kernels: padding sanitation, integer counts and allele
// frequency, per-SNP decode tables, and the synthetic-genotype generator; and
// the conversion of dense (FileBinary) rows to FP16 with their means.
//
// Code map (reference src/Common.hpp:50-59, BED2GENO = {1, -9, 0.5, 0} on the
// g/2 scale):  00 two copies of A1, 01 missing, 10 one copy, 11 no copy.
#include <cuda_fp16.h>

#include "../../include/pcaone_gpu.h"
#include "internal.cuh"

namespace pcaone {

namespace {

// Keeps the low 2*(N%4) bits of each SNP's last data byte (lanes past the last
// sample read as code 00); bytes past (N+3)/4 are zeroed at load time.
__global__ void k_sanitize(uint8_t* bed, int64_t stride, int64_t nsnps, int nsamples) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= nsnps) return;
  const int rem = nsamples & 3;
  if (rem == 0) return;
  uint8_t* p = bed + j * stride + (nsamples >> 2);
  *p = (uint8_t)(*p & ((1u << (2 * rem)) - 1u));
}

// Rows of `bps` bytes from a packed source (pitch src_pitch) into rows of
// dst_pitch bytes; one block per row, 16-, 4- or 1-byte moves as the pitches
// and bases allow.
template <class T>
__global__ void k_repitch(const uint8_t* __restrict__ src, int64_t src_pitch, uint8_t* __restrict__ dst,
                          int64_t dst_pitch, int64_t bps) {
  const int64_t r = blockIdx.x;
  const T* s = reinterpret_cast<const T*>(src + r * src_pitch);
  T* d = reinterpret_cast<T*>(dst + r * dst_pitch);
  const int64_t n = bps / (int64_t)sizeof(T);
  for (int64_t q = threadIdx.x; q < n; q += blockDim.x) d[q] = s[q];
}

// One warp per SNP row.  Per 32-bit word of 16 lanes: lo = bit 0 of each lane,
// hi = bit 1.  n11 = popc(lo & hi), n01 = popc(lo & ~hi), n10 = popc(hi & ~lo);
// n00 = N - the rest (padding lanes are code 00 and drop out).
__global__ void __launch_bounds__(256) k_counts(BedView v, int32_t* __restrict__ counts, double* __restrict__ F) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t j = (int64_t)blockIdx.x * 8 + warp;
  if (j >= v.nsnps) return;
  const uint4* row = reinterpret_cast<const uint4*>(v.bed + j * v.stride);
  const int nvec = (int)(v.stride >> 4);
  int n01 = 0, n10 = 0, n11 = 0;
  for (int q = lane; q < nvec; q += 32) {
    const uint4 w4 = __ldg(row + q);
    const uint32_t ws[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const uint32_t lo = ws[t] & 0x55555555u;
      const uint32_t hi = (ws[t] >> 1) & 0x55555555u;
      n11 += __popc(lo & hi);
      n01 += __popc(lo & ~hi);
      n10 += __popc(hi & ~lo);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    n01 += __shfl_xor_sync(0xffffffffu, n01, o);
    n10 += __shfl_xor_sync(0xffffffffu, n10, o);
    n11 += __shfl_xor_sync(0xffffffffu, n11, o);
  }
  if (lane == 0) {
    const int n00 = v.nsamples - n01 - n10 - n11;
    if (counts) {
      counts[j * 4 + 0] = n00;
      counts[j * 4 + 1] = n01;
      counts[j * 4 + 2] = n10;
      counts[j * 4 + 3] = n11;
    }
    // F = (sum of BED2GENO over observed) / n_observed (FilePlink.cpp:37-55);
    // n00 + 0.5*n10 is exact, so the quotient equals the reference's.
    const int c = n00 + n10 + n11;
    F[j] = c == 0 ? 0.0 : ((double)n00 + 0.5 * (double)n10) / (double)c;
  }
}

__global__ void k_lut(const double* __restrict__ F, int64_t nsnps, int standardize, int ploidy,
                      float4* __restrict__ lut32, double* __restrict__ lut64, double* __restrict__ scale) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= nsnps) return;
  const double f = F[j];
  double s = 1.0;
  if (standardize) {  // Data::standardize_E, src/Data.cpp:351-362
    const double sd = sqrt(f * (1.0 - f));
    if (sd > 1e-9) s = sqrt((double)ploidy) / sd;
  }
  const double x00 = (1.0 - f) * s, x10 = (0.5 - f) * s, x11 = (0.0 - f) * s;
  if (lut32) lut32[j] = make_float4((float)x00, 0.f, (float)x10, (float)x11);
  if (lut64) {
    lut64[j * 4 + 0] = x00;
    lut64[j * 4 + 1] = 0.0;
    lut64[j * 4 + 2] = x10;
    lut64[j * 4 + 3] = x11;
  }
  if (scale) scale[j] = s;
}

// SplitMix64 output function (Steele, Lea & Flood 2014).
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double u01(uint64_t counter, uint64_t stream) {
  return (double)(mix64(counter ^ stream) >> 11) * (1.0 / 9007199254740992.0);
}

// One thread per output byte (4 samples of one SNP).  Arithmetic uses
// explicit round-to-nearest operations (no contraction) to match the numpy
// generator bit for bit.
__global__ void k_synth(uint8_t* __restrict__ bed, int64_t stride, int64_t snp0, int64_t nsnps, int nsamples,
                        int npop, const double* __restrict__ freq, const double* __restrict__ weights,
                        const double* __restrict__ miss_sample, const double* __restrict__ miss_snp,
                        uint64_t sa, uint64_t sb, uint64_t sm) {
  const int64_t nbytes = stride;
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= nsnps * nbytes) return;
  const int64_t jl = idx / nbytes;
  const int q = (int)(idx - jl * nbytes);
  const int64_t j = snp0 + jl;
  uint32_t byte = 0;
  const double bj = miss_snp[jl];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int i = q * 4 + t;
    if (i >= nsamples) break;
    double p = 0.0;
    for (int k = 0; k < npop; ++k) p = __dadd_rn(p, __dmul_rn(weights[(int64_t)i * npop + k], freq[jl * npop + k]));
    const double r = __dsub_rn(1.0, __dmul_rn(__dsub_rn(1.0, miss_sample[i]), __dsub_rn(1.0, bj)));
    const uint64_t ctr = ((uint64_t)j << 32) | (uint64_t)i;
    uint32_t code;
    if (u01(ctr, sm) < r) {
      code = 1u;
    } else {
      const int d = (u01(ctr, sa) < p) + (u01(ctr, sb) < p);
      code = d == 2 ? 0u : (d == 1 ? 2u : 3u);
    }
    byte |= code << (2 * t);
  }
  bed[jl * stride + q] = (uint8_t)byte;
}

// PLINK 2 hard calls (2-bit ALT allele counts, 3 = missing) to PLINK 1 codes
// with A1 = ALT, in place over a byte range: with a = b1 b0 the code is
// (NOT b1, NOT (b1 XOR b0)): 2 -> 00, 1 -> 10, 0 -> 11, 3 -> 01.  Four bytes
// per thread; padding lanes of the last byte of a row are cleared afterwards
// by the sanitation pass.
__global__ void k_genovec_to_bed(uint8_t* __restrict__ bytes, int64_t nbytes) {
  const int64_t i0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * 4;
  if (i0 >= nbytes) return;
  const int cnt = nbytes - i0 < 4 ? (int)(nbytes - i0) : 4;
  uint32_t w = 0;
  for (int k = 0; k < cnt; ++k) w |= (uint32_t)bytes[i0 + k] << (8 * k);
  const uint32_t lo = w & 0x55555555u, hi = (w >> 1) & 0x55555555u;
  w = ((~hi & 0x55555555u) << 1) | (~(hi ^ lo) & 0x55555555u);
  for (int k = 0; k < cnt; ++k) bytes[i0 + k] = (uint8_t)(w >> (8 * k));
}

// Rows perm[0 .. nrows) of src into consecutive rows of dst (stride bytes
// each, a multiple of 16), for sources across the host link (pinned host
// memory mapped into the device address space), whose latency wants many
// loads in flight: the rows' 16-byte chunks are strided over the grid, and
// every thread issues kGatherDepth loads before it stores them.  Consecutive
// threads take consecutive chunks of a row (coalesced).
constexpr int kGatherDepth = 8;
__global__ void __launch_bounds__(256) k_gather_rows_deep(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                                                          int64_t stride, const int32_t* __restrict__ perm,
                                                          int64_t nrows) {
  const int64_t cpr = stride >> 4;
  const int64_t total = nrows * cpr;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q0 < total; q0 += step * kGatherDepth) {
    uint4 v[kGatherDepth];
    int64_t d[kGatherDepth];
#pragma unroll
    for (int u = 0; u < kGatherDepth; ++u) {
      const int64_t q = q0 + u * step;
      d[u] = -1;
      if (q < total) {
        const int64_t r = q / cpr, c = q - r * cpr;
        const int64_t srow = perm ? (int64_t)perm[r] : r;
        v[u] = *reinterpret_cast<const uint4*>(src + srow * stride + (c << 4));
        d[u] = r * stride + (c << 4);
      }
    }
#pragma unroll
    for (int u = 0; u < kGatherDepth; ++u)
      if (d[u] >= 0) *reinterpret_cast<uint4*>(dst + d[u]) = v[u];
  }
}

}  // namespace

void launch_gather_rows_deep(const uint8_t* src, uint8_t* dst, int64_t stride, const int32_t* perm, int64_t nrows,
                             int ctas, cudaStream_t s) {
  if (nrows <= 0) return;
  if ((stride & 15) != 0 || ((uintptr_t)src & 15u) != 0 || ((uintptr_t)dst & 15u) != 0)
    throw Error(PCAONE_E_ARG, "internal: row gather needs 16-byte aligned rows");
  k_gather_rows_deep<<<ctas, 256, 0, s>>>(src, dst, stride, perm, nrows);
  PCAONE_LAUNCH_CHECK();
}

void launch_genovec_to_bed(uint8_t* bytes, int64_t nbytes, cudaStream_t s) {
  if (nbytes <= 0) return;
  k_genovec_to_bed<<<ceil_div(ceil_div(nbytes, 4), 256), 256, 0, s>>>(bytes, nbytes);
  PCAONE_LAUNCH_CHECK();
}

void launch_repitch(const uint8_t* src, int64_t src_pitch, uint8_t* dst, int64_t dst_pitch, int64_t nrows, int64_t bps,
                    cudaStream_t s) {
  if (nrows <= 0) return;
  const uintptr_t al = (uintptr_t)src | (uintptr_t)dst | (uintptr_t)src_pitch | (uintptr_t)dst_pitch | (uintptr_t)bps;
  if ((al & 15u) == 0)
    k_repitch<uint4><<<(unsigned)nrows, 256, 0, s>>>(src, src_pitch, dst, dst_pitch, bps);
  else if ((al & 3u) == 0)
    k_repitch<uint32_t><<<(unsigned)nrows, 256, 0, s>>>(src, src_pitch, dst, dst_pitch, bps);
  else
    k_repitch<uint8_t><<<(unsigned)nrows, 256, 0, s>>>(src, src_pitch, dst, dst_pitch, bps);
  PCAONE_LAUNCH_CHECK();
}

void launch_sanitize_padding(uint8_t* bed, int64_t stride, int64_t nsnps, int nsamples, cudaStream_t s) {
  if ((nsamples & 3) == 0 || nsnps == 0) return;
  k_sanitize<<<ceil_div(nsnps, 256), 256, 0, s>>>(bed, stride, nsnps, nsamples);
  PCAONE_LAUNCH_CHECK();
}

void launch_counts(const BedView& v, int32_t* counts, double* F, cudaStream_t s) {
  if (v.nsnps == 0) return;
  k_counts<<<ceil_div(v.nsnps, 8), 256, 0, s>>>(v, counts, F);
  PCAONE_LAUNCH_CHECK();
}

void launch_lut(const double* F, int64_t nsnps, int standardize, int ploidy, float4* lut32, double* lut64,
                double* scale, cudaStream_t s) {
  if (nsnps == 0) return;
  k_lut<<<ceil_div(nsnps, 256), 256, 0, s>>>(F, nsnps, standardize, ploidy, lut32, lut64, scale);
  PCAONE_LAUNCH_CHECK();
}

void launch_synth(uint8_t* bed, int64_t stride, int64_t snp0, int64_t nsnps, int nsamples, int npop,
                  const double* freq, const double* weights, const double* miss_sample, const double* miss_snp,
                  uint64_t seed, cudaStream_t s) {
  // stream keys as in pcaone_gb300/synthetic.py (KEY_ALLELE_A, KEY_ALLELE_B, KEY_MISSING)
  auto host_mix = [](uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  const uint64_t base = seed * 0x2545F4914F6CDD1Dull;
  const uint64_t sa = host_mix(base + 0x243F6A8885A308D3ull);
  const uint64_t sb = host_mix(base + 0x13198A2E03707344ull);
  const uint64_t sm = host_mix(base + 0xA4093822299F31D0ull);
  const int64_t total = nsnps * stride;
  if (total == 0) return;
  k_synth<<<ceil_div(total, 256), 256, 0, s>>>(bed, stride, snp0, nsnps, nsamples, npop, freq, weights,
                                                 miss_sample, miss_snp, sa, sb, sm);
  PCAONE_LAUNCH_CHECK();
}

namespace {

// One warp per row: float32 values -> FP16 (round to nearest) in a row of
// npad values (zeros past N), and the row's mean of the FP16 values, exact up
// to the final division: every FP16 value is an integer multiple of 2^-24, so
// the row sum is an exact int64 of units 2^-24 (rows of |values| <= 65504 and
// N <= 2^23).
__global__ void k_dense_rows(const float* __restrict__ src, int64_t nrows, int N, int npad,
                             __half* __restrict__ dst, double* __restrict__ mean) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nrows) return;
  const float* row = src + r * N;
  __half* out = dst + r * npad;
  long long sum = 0;
  for (int i = lane; i < npad; i += 32) {
    const __half h = i < N ? __float2half_rn(row[i]) : __float2half_rn(0.f);
    out[i] = h;
    sum += (long long)llrint((double)__half2float(h) * 16777216.0);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) mean[r] = (double)sum / 16777216.0 / (double)N;
}

}  // namespace

namespace {

// Continuous dosages of the synthetic model (pcaone_gb300/synthetic.py
// sample_dosages): allele count from the two allele draws plus sd times a
// Box-Muller normal from two further hashed uniforms, clipped to [0, 2].  The
// allele draws match the numpy generator bit for bit; the noise uses the
// device log/cos, so a value can land on the other side of an FP16 rounding
// boundary than numpy's in rare cases.
__global__ void k_synth_dense(float* __restrict__ out, int64_t snp0, int64_t nsnps, int nsamples, int npop,
                              const double* __restrict__ freq, const double* __restrict__ weights, double sd,
                              uint64_t sa, uint64_t sb, uint64_t s1, uint64_t s2) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= nsnps * nsamples) return;
  const int64_t jl = idx / nsamples;
  const int i = (int)(idx - jl * nsamples);
  const int64_t j = snp0 + jl;
  double p = 0.0;
  for (int k = 0; k < npop; ++k) p = __dadd_rn(p, __dmul_rn(weights[(int64_t)i * npop + k], freq[jl * npop + k]));
  const uint64_t ctr = ((uint64_t)j << 32) | (uint64_t)i;
  const double d = (double)((u01(ctr, sa) < p) + (u01(ctr, sb) < p));
  const double z = sqrt(-2.0 * log(fmax(u01(ctr, s1), 1e-300))) * cos(6.283185307179586 * u01(ctr, s2));
  out[idx] = (float)fmin(fmax(d + sd * z, 0.0), 2.0);
}

}  // namespace

void launch_synth_dense(float* out, int64_t snp0, int64_t nsnps, int nsamples, int npop, const double* freq,
                        const double* weights, double sd, uint64_t seed, cudaStream_t s) {
  auto host_mix = [](uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  // stream keys as in pcaone_gb300/synthetic.py (KEY_ALLELE_A, KEY_ALLELE_B, KEY_DOSAGE_NOISE, +1)
  const uint64_t base = seed * 0x2545F4914F6CDD1Dull;
  const uint64_t sa = host_mix(base + 0x243F6A8885A308D3ull);
  const uint64_t sb = host_mix(base + 0x13198A2E03707344ull);
  const uint64_t s1 = host_mix(base + 0xD05Eull);
  const uint64_t s2 = host_mix(base + 0xD05Full);
  const int64_t total = nsnps * nsamples;
  if (total == 0) return;
  k_synth_dense<<<ceil_div(total, 256), 256, 0, s>>>(out, snp0, nsnps, nsamples, npop, freq, weights, sd, sa, sb,
                                                     s1, s2);
  PCAONE_LAUNCH_CHECK();
}

void launch_dense_rows(const float* src, int64_t nrows, int N, int npad, uint8_t* dst, double* mean, cudaStream_t s) {
  if (nrows == 0) return;
  k_dense_rows<<<ceil_div(nrows * 32, 256), 256, 0, s>>>(src, nrows, N, npad, reinterpret_cast<__half*>(dst), mean);
  PCAONE_LAUNCH_CHECK();
}

}  // namespace pcaone
