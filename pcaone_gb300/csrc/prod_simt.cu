// Window block products of the winSVD / sSVD schedule, FP32 SIMT form.
//
// For the SNP window [pos0, pos0+nsnp) of the working order (positions map to
// .bed rows through `perm`), with x(i,j) the decoded, centred and scaled
// genotype of sample i at SNP j (per-SNP 4-entry table, missing -> 0):
//   G[pos0+j][:] = sum_i x(i,j) * Omega[i][:]      (reference: G_b = X_b^T Omega,
//                                                  src/Halko.cpp:195-196)
//   Hx[i][:]    += sum_j x(i,j) * G[pos0+j][:]     (H1/H2 += X_b G_b, :198-203)
// FP32 products; sums longer than one chunk/split are combined in FP64.
#include <algorithm>

#include "internal.cuh"

namespace pcaone {

namespace {

__device__ __forceinline__ float lut_pick(const float4& t, uint32_t code) {
  // code: 0 -> x00, 1 -> missing (0), 2 -> x10, 3 -> x11
  const float a = (code & 1u) ? t.y : t.x;
  const float b = (code & 1u) ? t.w : t.z;
  return (code & 2u) ? b : a;
}

constexpr int kGTileSnps = 128;   // SNPs per CTA in the G product
constexpr int kGStep = 32;        // samples per shared-memory step
constexpr int kHTileSamples = 128;
constexpr int kHStep = 32;        // SNPs per shared-memory step

// G partial product.  CTA: 128 SNPs x one sample chunk; thread: 4 SNPs x LP/8
// columns (column c*8 + cg).
template <int LP>
__global__ void __launch_bounds__(256) k_window_g(BedView v, const int32_t* __restrict__ perm,
                                                  const float4* __restrict__ lut, int64_t pos0, int nsnp,
                                                  int chunk, int npad, const float* __restrict__ omg32,
                                                  float* __restrict__ part) {
  constexpr int TC = LP / 8;
  __shared__ __align__(16) float xs[kGStep][kGTileSnps + 4];
  __shared__ __align__(16) float os[kGStep][LP];
  __shared__ const uint8_t* rowp[kGTileSnps];
  __shared__ float4 lt[kGTileSnps];
  const int tid = threadIdx.x;
  const int snp_base = blockIdx.x * kGTileSnps;
  const int s_begin = blockIdx.y * chunk;
  const int s_end = min(s_begin + chunk, npad);
  if (tid < kGTileSnps) {
    const int j = snp_base + tid;
    if (j < nsnp) {
      const int64_t pos = pos0 + j;
      const int64_t snp = perm ? (int64_t)perm[pos] : pos;
      rowp[tid] = v.bed + snp * v.stride;
      lt[tid] = lut[snp];
    } else {
      rowp[tid] = nullptr;
      lt[tid] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  __syncthreads();
  const int sg = tid >> 3;
  const int cg = tid & 7;
  float acc[4][TC];
#pragma unroll
  for (int t = 0; t < 4; ++t)
#pragma unroll
    for (int c = 0; c < TC; ++c) acc[t][c] = 0.f;

  for (int s0 = s_begin; s0 < s_end; s0 += kGStep) {
    for (int e = tid; e < kGStep * (LP / 4); e += 256) {
      const int r = e / (LP / 4), c4 = e % (LP / 4);
      reinterpret_cast<float4*>(&os[r][0])[c4] = reinterpret_cast<const float4*>(omg32 + (size_t)(s0 + r) * LP)[c4];
    }
    {
      // thread -> SNP tid/2, 16 samples (4 bytes) of the 32-sample step
      const int js = tid >> 1, half = tid & 1;
      const uint8_t* rp = rowp[js];
      uint32_t w = 0u;
      if (rp) w = *reinterpret_cast<const uint32_t*>(rp + (s0 >> 2) + half * 4);
      const float4 t4 = lt[js];
      const int sb = half * 16;
#pragma unroll
      for (int q = 0; q < 16; ++q) xs[sb + q][js] = lut_pick(t4, (w >> (2 * q)) & 3u);
    }
    __syncthreads();
#pragma unroll 4
    for (int r = 0; r < kGStep; ++r) {
      const float4 x = *reinterpret_cast<const float4*>(&xs[r][sg * 4]);
      float o[TC];
#pragma unroll
      for (int c = 0; c < TC; ++c) o[c] = os[r][c * 8 + cg];
#pragma unroll
      for (int c = 0; c < TC; ++c) {
        acc[0][c] = fmaf(x.x, o[c], acc[0][c]);
        acc[1][c] = fmaf(x.y, o[c], acc[1][c]);
        acc[2][c] = fmaf(x.z, o[c], acc[2][c]);
        acc[3][c] = fmaf(x.w, o[c], acc[3][c]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int j = snp_base + sg * 4 + t;
    if (j < nsnp) {
      float* dst = part + ((size_t)blockIdx.y * nsnp + j) * LP;
#pragma unroll
      for (int c = 0; c < TC; ++c) dst[c * 8 + cg] = acc[t][c];
    }
  }
}

// H partial product.  CTA: 128 samples x one SNP split; thread: 4 samples x
// LP/8 columns.
template <int LP>
__global__ void __launch_bounds__(256) k_window_h(BedView v, const int32_t* __restrict__ perm,
                                                  const float4* __restrict__ lut, int64_t pos0, int nsnp,
                                                  int per_split, int npad, const float* __restrict__ g32,
                                                  float* __restrict__ hpart) {
  constexpr int TC = LP / 8;
  __shared__ __align__(16) float xs[kHStep][kHTileSamples + 4];
  __shared__ __align__(16) float gs[kHStep][LP];
  const int tid = threadIdx.x;
  const int samp_base = blockIdx.x * kHTileSamples;
  const int jb = blockIdx.y * per_split;
  const int je = min(jb + per_split, nsnp);
  const int sg = tid >> 3;
  const int cg = tid & 7;
  float acc[4][TC];
#pragma unroll
  for (int t = 0; t < 4; ++t)
#pragma unroll
    for (int c = 0; c < TC; ++c) acc[t][c] = 0.f;

  for (int j0 = jb; j0 < je; j0 += kHStep) {
    for (int e = tid; e < kHStep * (LP / 4); e += 256) {
      const int r = e / (LP / 4), c4 = e % (LP / 4);
      float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
      if (j0 + r < je) val = reinterpret_cast<const float4*>(g32 + (size_t)(j0 + r) * LP)[c4];
      reinterpret_cast<float4*>(&gs[r][0])[c4] = val;
    }
    {
      const int r = tid >> 3, q = tid & 7;
      float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a, c = a, d = a;
      if (j0 + r < je) {
        const int64_t pos = pos0 + j0 + r;
        const int64_t snp = perm ? (int64_t)perm[pos] : pos;
        const uint32_t w = *reinterpret_cast<const uint32_t*>(v.bed + snp * v.stride + (samp_base >> 2) + q * 4);
        const float4 t4 = lut[snp];
        a = make_float4(lut_pick(t4, w & 3u), lut_pick(t4, (w >> 2) & 3u), lut_pick(t4, (w >> 4) & 3u),
                        lut_pick(t4, (w >> 6) & 3u));
        b = make_float4(lut_pick(t4, (w >> 8) & 3u), lut_pick(t4, (w >> 10) & 3u), lut_pick(t4, (w >> 12) & 3u),
                        lut_pick(t4, (w >> 14) & 3u));
        c = make_float4(lut_pick(t4, (w >> 16) & 3u), lut_pick(t4, (w >> 18) & 3u), lut_pick(t4, (w >> 20) & 3u),
                        lut_pick(t4, (w >> 22) & 3u));
        d = make_float4(lut_pick(t4, (w >> 24) & 3u), lut_pick(t4, (w >> 26) & 3u), lut_pick(t4, (w >> 28) & 3u),
                        lut_pick(t4, (w >> 30) & 3u));
      }
      float4* dst = reinterpret_cast<float4*>(&xs[r][q * 16]);
      dst[0] = a;
      dst[1] = b;
      dst[2] = c;
      dst[3] = d;
    }
    __syncthreads();
#pragma unroll 4
    for (int r = 0; r < kHStep; ++r) {
      const float4 x = *reinterpret_cast<const float4*>(&xs[r][sg * 4]);
      float g[TC];
#pragma unroll
      for (int c = 0; c < TC; ++c) g[c] = gs[r][c * 8 + cg];
#pragma unroll
      for (int c = 0; c < TC; ++c) {
        acc[0][c] = fmaf(x.x, g[c], acc[0][c]);
        acc[1][c] = fmaf(x.y, g[c], acc[1][c]);
        acc[2][c] = fmaf(x.z, g[c], acc[2][c]);
        acc[3][c] = fmaf(x.w, g[c], acc[3][c]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int i = samp_base + sg * 4 + t;
    float* dst = hpart + ((size_t)blockIdx.y * npad + i) * LP;
#pragma unroll
    for (int c = 0; c < TC; ++c) dst[c * 8 + cg] = acc[t][c];
  }
}

// G rows of the window: FP64 sum of the chunk partials plus the sparse
// missing-value term scale_j * sum_e value_e * Omega[sample_e][:], and the FP32
// copy used by the H product.  One warp per SNP row, lanes over columns.
__global__ void k_window_g_finish(int64_t pos0, int nsnp, int LP, const float* __restrict__ part, int nchunks,
                                  SparseRows sp, const double* __restrict__ omg, double* __restrict__ G,
                                  float* __restrict__ g32) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= nsnp) return;
  const int64_t pos = pos0 + warp;
  for (int l = lane; l < LP; l += 32) {
    double acc = 0.0;
    for (int c = 0; c < nchunks; ++c) acc += (double)part[((size_t)c * nsnp + warp) * LP + l];
    if (sp.active) {
      const int64_t snp = sp.perm ? (int64_t)sp.perm[pos] : pos;
      const double sc = sp.scale[snp];
      double sacc = 0.0;
      for (int64_t e = sp.rowptr[pos]; e < sp.rowptr[pos + 1]; ++e)
        sacc += sp.value[e] * omg[(size_t)sp.sample[e] * LP + l];
      acc += sc * sacc;
    }
    G[pos * LP + l] = acc;
    g32[(size_t)warp * LP + l] = (float)acc;
  }
}

__global__ void k_window_h_finish(int nsamples, int npad, int LP, const float* __restrict__ hpart, int nsplit,
                                  double* __restrict__ Hx) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nsamples * LP) return;
  const int64_t i = idx / LP;
  const int l = (int)(idx - i * LP);
  double acc = 0.0;
  for (int c = 0; c < nsplit; ++c) acc += (double)hpart[((size_t)c * npad + i) * LP + l];
  Hx[idx] += acc;
}

template <int LP>
void launch_g_t(const WindowArgs& a, const float* omg32, float* part, int nchunks, cudaStream_t s) {
  const int chunk = round_up(ceil_div(a.npad, nchunks), kGStep);
  dim3 grid(ceil_div(a.nsnp, kGTileSnps), nchunks);
  k_window_g<LP><<<grid, 256, 0, s>>>(a.v, a.perm, a.lut, a.pos0, a.nsnp, chunk, a.npad, omg32, part);
}

template <int LP>
void launch_h_t(const WindowArgs& a, const float* g32, float* hpart, int nsplit, cudaStream_t s) {
  const int per = round_up(ceil_div(a.nsnp, nsplit), kHStep);
  dim3 grid(a.npad / kHTileSamples, nsplit);
  k_window_h<LP><<<grid, 256, 0, s>>>(a.v, a.perm, a.lut, a.pos0, a.nsnp, per, a.npad, g32, hpart);
}

}  // namespace

int window_g_chunks(const WindowArgs& a) {
  // enough CTAs for ~4 waves on 152 SMs, FP32 runs of at most 2048 samples
  const int xt = ceil_div(a.nsnp, kGTileSnps);
  int ch = std::max(1, 608 / std::max(1, xt));
  ch = std::max(ch, ceil_div(a.npad, 2048));
  ch = std::min(ch, a.npad / kGStep);
  // the chunk length is rounded up to kGStep; drop chunks that would be empty
  const int chunk = round_up(ceil_div(a.npad, ch), kGStep);
  return ceil_div(a.npad, chunk);
}

int window_h_splits(const WindowArgs& a) {
  const int xt = a.npad / kHTileSamples;
  int sp = std::max(1, 608 / std::max(1, xt));
  sp = std::max(sp, ceil_div(a.nsnp, 2048));
  sp = std::min(sp, std::max(1, ceil_div(a.nsnp, kHStep)));
  const int per = round_up(ceil_div(a.nsnp, sp), kHStep);
  return std::max(1, ceil_div(a.nsnp, per));
}

#define PCAONE_LP_SWITCH(LPV, FN, ...)                              \
  switch (LPV) {                                                  \
    case 8: FN<8>(__VA_ARGS__); break;                            \
    case 16: FN<16>(__VA_ARGS__); break;                          \
    case 24: FN<24>(__VA_ARGS__); break;                          \
    case 32: FN<32>(__VA_ARGS__); break;                          \
    case 40: FN<40>(__VA_ARGS__); break;                          \
    case 48: FN<48>(__VA_ARGS__); break;                          \
    case 56: FN<56>(__VA_ARGS__); break;                          \
    case 64: FN<64>(__VA_ARGS__); break;                          \
    case 72: FN<72>(__VA_ARGS__); break;                          \
    case 80: FN<80>(__VA_ARGS__); break;                          \
    case 88: FN<88>(__VA_ARGS__); break;                          \
    case 96: FN<96>(__VA_ARGS__); break;                          \
    case 104: FN<104>(__VA_ARGS__); break;                        \
    case 112: FN<112>(__VA_ARGS__); break;                        \
    default: throw Error(-6, "unsupported padded sketch width");  \
  }

void launch_window_g(const WindowArgs& a, const float* omg32, float* part, int nchunks, cudaStream_t s) {
  PCAONE_LP_SWITCH(a.LP, launch_g_t, a, omg32, part, nchunks, s);
  PCAONE_LAUNCH_CHECK();
}

void launch_window_h(const WindowArgs& a, const float* g32, float* hpart, int nsplit, cudaStream_t s) {
  PCAONE_LP_SWITCH(a.LP, launch_h_t, a, g32, hpart, nsplit, s);
  PCAONE_LAUNCH_CHECK();
}

void launch_window_g_finish(const WindowArgs& a, const float* part, int nchunks, const SparseRows& sp,
                            const double* omg, double* G, float* g32, cudaStream_t s) {
  const int threads = 256;
  k_window_g_finish<<<ceil_div((int64_t)a.nsnp * 32, threads), threads, 0, s>>>(a.pos0, a.nsnp, a.LP, part,
                                                                                  nchunks, sp, omg, G, g32);
  PCAONE_LAUNCH_CHECK();
}

void launch_window_h_finish(const WindowArgs& a, const float* hpart, int nsplit, double* Hx, cudaStream_t s) {
  const int64_t n = (int64_t)a.v.nsamples * a.LP;
  k_window_h_finish<<<ceil_div(n, 256), 256, 0, s>>>(a.v.nsamples, a.npad, a.LP, hpart, nsplit, Hx);
  PCAONE_LAUNCH_CHECK();
}

}  // namespace pcaone
