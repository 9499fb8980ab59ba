// Small utility kernels: the missing-genotype lists (by position, and grouped
// by window and sample, with the device prefix sum of the group offsets), the
// segmented gather of the missing-entry terms, the EM term of H in the FP32
// form, the sign convention flip_UV, and the row-major -> column-major copy of
// outputs.
#include <algorithm>

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

// Missing genotypes grouped by (window, sample).  Window w holds positions
// [w*wsize, min((w+1)*wsize, M)); bucket w*N + i lists, in increasing
// position, the positions of window w at which sample i is missing (code 01).
// One thread per 32-bit word of a row (16 samples), grid row = window; the
// count pass writes cnt[w*N + i], the fill pass (after an exclusive scan of the
// counts into ptr) writes the positions and samples.  Each thread keeps its 16
// counters or write offsets in its own column of shared memory, so a missing
// entry costs one indexed update.
template <bool kFill>
__global__ void __launch_bounds__(128) k_buckets(BedView v, const int32_t* __restrict__ perm, int64_t wsize,
                                                 int32_t* __restrict__ cnt, const int64_t* __restrict__ ptr,
                                                 int32_t* __restrict__ bpos, int32_t* __restrict__ bsample) {
  __shared__ long long soff[kFill ? 16 : 1][128];
  __shared__ int scnt[kFill ? 1 : 16][128];
  const int tx = threadIdx.x;
  const int wd = blockIdx.x * blockDim.x + tx;
  const int nwords = (v.nsamples + 15) >> 4;
  if (wd >= nwords) return;
  const int64_t win = blockIdx.y;
  const int64_t p0 = win * wsize;
  const int64_t p1 = p0 + wsize < v.nsnps ? p0 + wsize : v.nsnps;
  const int i0 = wd * 16;
  const int nloc = v.nsamples - i0 < 16 ? v.nsamples - i0 : 16;
  const uint32_t valid = nloc == 16 ? 0x55555555u : (((1u << (2 * nloc)) - 1u) & 0x55555555u);
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    if (kFill)
      soff[kFill ? q : 0][tx] = q < nloc ? ptr[win * v.nsamples + i0 + q] : 0;
    else
      scnt[kFill ? 0 : q][tx] = 0;
  }
#pragma unroll 8
  for (int64_t p = p0; p < p1; ++p) {
    const int64_t r = perm ? (int64_t)perm[p] : p;
    const uint32_t word = reinterpret_cast<const uint32_t*>(v.bed + r * v.stride)[wd];
    uint32_t miss = word & ~(word >> 1) & valid;  // low bit set, high bit clear
    while (miss) {
      const int q = (__ffs(miss) - 1) >> 1;
      if (kFill) {
        const long long e = soff[kFill ? q : 0][tx]++;
        bpos[e] = (int32_t)p;
        bsample[e] = i0 + q;
      } else {
        scnt[kFill ? 0 : q][tx] += 1;
      }
      miss &= miss - 1u;
    }
  }
  if (!kFill) {
    for (int q = 0; q < nloc; ++q) cnt[win * v.nsamples + i0 + q] = scnt[kFill ? 0 : q][tx];
  }
}

// Exclusive prefix sum of n int32 counts into int64 offsets, out[0..n] with
// out[n] the total, in three passes over tiles of kScanTile counts: tile sums,
// an exclusive scan of the tile sums (one block, which also writes out[n]),
// then each tile's own scan from its offset.  Integer sums, so the result does
// not depend on the order of the passes' additions.
constexpr int kScanThreads = 512;
constexpr int kScanPerThread = 8;
constexpr int kScanTile = kScanThreads * kScanPerThread;

// exclusive scan of one value per thread over the block (blockDim.x = kScanThreads);
// *total receives the block's sum
__device__ __forceinline__ long long block_exclusive_scan(long long v, long long* total) {
  __shared__ long long wsum[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    long long w = lane < kScanThreads / 32 ? wsum[lane] : 0;
    long long wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kScanThreads / 32) wsum[lane] = wi - w;  // exclusive warp offsets
    if (lane == kScanThreads / 32 - 1) *total = wi;
  }
  __syncthreads();
  const long long r = wsum[warp] + incl - v;
  __syncthreads();  // wsum is reused by the next call
  return r;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tile_sums(const int32_t* __restrict__ in, int64_t n,
                                                                 long long* __restrict__ tsum) {
  __shared__ long long tot;
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPerThread;
  long long v = 0;
#pragma unroll
  for (int q = 0; q < kScanPerThread; ++q)
    if (base + q < n) v += in[base + q];
  block_exclusive_scan(v, &tot);
  if (threadIdx.x == 0) tsum[blockIdx.x] = tot;
}

// one block: tsum[0..ntiles) becomes exclusive; out_total = the sum of all
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(long long* __restrict__ tsum, int ntiles,
                                                             int64_t* __restrict__ out_total) {
  __shared__ long long tot;
  long long carry = 0;
  for (int c0 = 0; c0 < ntiles; c0 += kScanThreads) {
    const int i = c0 + threadIdx.x;
    const long long v = i < ntiles ? tsum[i] : 0;
    const long long ex = block_exclusive_scan(v, &tot);
    __syncthreads();
    if (i < ntiles) tsum[i] = carry + ex;
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *out_total = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int32_t* __restrict__ in, int64_t n,
                                                             const long long* __restrict__ tsum,
                                                             int64_t* __restrict__ out) {
  __shared__ long long tot;
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPerThread;
  int32_t c[kScanPerThread];
  long long v = 0;
#pragma unroll
  for (int q = 0; q < kScanPerThread; ++q) {
    c[q] = base + q < n ? in[base + q] : 0;
    v += c[q];
  }
  long long run = tsum[blockIdx.x] + block_exclusive_scan(v, &tot);
#pragma unroll
  for (int q = 0; q < kScanPerThread; ++q) {
    if (base + q < n) out[base + q] = run;
    run += c[q];
  }
}

// The EM term of H in the FP32 form for window `win` (positions
// [pos0, pos0+nsnp)): for each sample i, over the entries e of bucket (win, i)
// at positions p, Hx[i] += sum_e s_p v_e G32[p - pos0], with v_e the EM fill
// value and G32 the window's FP32 G rows; error-free FP32 pairs.  One warp
// per sample: the lanes fetch 32 entries at once, then every lane loads 16
// broadcast rows before accumulating them.
template <int NQ>
__global__ void k_h_buckets(int64_t win, int N, int L, int LP, const int64_t* __restrict__ ptr,
                            const int32_t* __restrict__ bpos, const double* __restrict__ bval,
                            const int32_t* __restrict__ perm, const double* __restrict__ scale,
                            const float* __restrict__ Rf, int64_t rbase, double* __restrict__ Hx) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= N) return;
  const int64_t e0 = ptr[win * N + i], e1 = ptr[win * N + i + 1];
  if (e0 == e1) return;
  FloatPair esum[NQ];
  for (int64_t eb = e0; eb < e1; eb += 32) {
    const int ne = (int)(e1 - eb < 32 ? e1 - eb : 32);
    int roff = 0;
    float vh = 0.f, vl = 0.f;
    if (lane < ne) {
      const int64_t p = bpos[eb + lane];
      roff = (int)(p - rbase) * LP;
      fp_split(scale[perm ? (int64_t)perm[p] : p] * bval[eb + lane], vh, vl);
    }
#pragma unroll 1
    for (int h = 0; h < ne; h += 16) {
      float w[16][NQ];
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int t = h + u;
        const int ro = __shfl_sync(0xffffffffu, roff, t);
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int l = lane + 32 * q;
          w[u][q] = (t < ne && l < L) ? Rf[ro + l] : 0.f;
        }
      }
#pragma unroll
      for (int u = 0; u < 16; ++u) {  // entries t >= ne carry a zero coefficient
        const float ch = __shfl_sync(0xffffffffu, vh, h + u);
        const float cl = __shfl_sync(0xffffffffu, vl, h + u);
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          fp_add_prod(esum[q], ch, w[u][q]);
          esum[q].lo = fmaf(cl, w[u][q], esum[q].lo);
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int l = lane + 32 * q;
    if (l < L) Hx[i * LP + l] += fp_value(esum[q]);
  }
}

// Lane groups: gsize = max(8, ceil(L/4)) lanes share one entry, lane c of a
// group loading columns 4c .. 4c+3 of the entry's source row with one 16-byte
// load, so a warp gathers 32/gsize rows per load instruction (three rows of
// 40 columns).  Each group sums a run of kSegRun consecutive entries: lanes
// c < 8 fetch the keys, source offsets and quantised values of 8 entries at
// once (4 with EM values, to keep registers for two loads per entry), the
// group loads their rows (all loads independent), then adds them
// in entry order while the key is unchanged; a key change (group-uniform)
// flushes the running sums into the int64 output with atomics.  The row sums
// are int64 (|R| <= 2^26: a run of 64 entries reaches 2^32).
constexpr int kSegRun = 64;
constexpr int kSegFetch = 8;  // lanes per group that fetch entry indices (the minimum group size)

template <bool VALS>
__global__ void __launch_bounds__(256) k_seg_gather(SegGatherArgs a, int gsize, int ngroups) {
  constexpr int kSegBatch = VALS ? 4 : 8;
  const int lane = threadIdx.x & 31;
  const int grp = lane / gsize;
  const bool active = grp < ngroups;
  const int gbase = active ? grp * gsize : 0;
  const int c = active ? lane - gbase : gsize;  // idle lanes fetch and sum nothing
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t wb = a.e0 + w * ngroups * kSegRun;
  if (wb >= a.e1) return;  // warp-uniform
  const int64_t rb = wb + (int64_t)(active ? grp : 0) * kSegRun;
  const int64_t re = active ? (rb + kSegRun < a.e1 ? rb + kSegRun : a.e1) : rb;
  const int col = 4 * c;
  const bool cols = col < a.L;
  const bool same = a.R2 == a.R;  // G side: the value products use the same integer rows
  long long acc[4] = {0, 0, 0, 0};
  long long acc2[4] = {0, 0, 0, 0};
  int cur = -1;
  auto flush = [&]() {
    if (cur >= 0 && cols) {
      unsigned long long* o = a.out + (size_t)cur * a.LP + col;
      unsigned long long* o2 = VALS ? a.out2 + (size_t)cur * a.LP + col : nullptr;
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        if (col + t < a.L) {
          atomicAdd(o + t, (unsigned long long)acc[t]);
          if (VALS) atomicAdd(o2 + t, (unsigned long long)acc2[t]);
        }
      }
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      acc[t] = 0;
      acc2[t] = 0;
    }
  };
  for (int b = 0; b < kSegRun; b += kSegBatch) {
    const int64_t ef = rb + b + c;
    int krow = -1, soff = 0, vi = 0;
    if (c < kSegBatch && ef < re) {
      krow = (int)(a.key[ef] - a.key_base);
      soff = (int)(a.src[ef] - a.src_base) * a.LP;
      if (VALS) vi = __double2int_rn(a.val[ef] * kSegValueScale);
    }
    int kr[kSegBatch], vt[kSegBatch];
    int4 r[kSegBatch], r2[VALS ? kSegBatch : 1];
#pragma unroll
    for (int u = 0; u < kSegBatch; ++u) {
      const int so = __shfl_sync(0xffffffffu, soff, gbase + u);
      kr[u] = __shfl_sync(0xffffffffu, krow, gbase + u);
      vt[u] = VALS ? __shfl_sync(0xffffffffu, vi, gbase + u) : 0;
      const bool ok = kr[u] >= 0 && cols;
      r[u] = ok ? __ldg(reinterpret_cast<const int4*>(a.R + so + col)) : make_int4(0, 0, 0, 0);
      if (VALS)
        r2[VALS ? u : 0] = same ? r[u] : (ok ? __ldg(reinterpret_cast<const int4*>(a.R2 + so + col)) : make_int4(0, 0, 0, 0));
    }
#pragma unroll
    for (int u = 0; u < kSegBatch; ++u) {
      if (kr[u] >= 0) {
        if (kr[u] != cur) {
          flush();
          cur = kr[u];
        }
        acc[0] += r[u].x;
        acc[1] += r[u].y;
        acc[2] += r[u].z;
        acc[3] += r[u].w;
        if (VALS) {
          const int4 q = r2[VALS ? u : 0];
          const long long v = vt[u];
          acc2[0] += (v * (long long)q.x) >> kSegValueShift;
          acc2[1] += (v * (long long)q.y) >> kSegValueShift;
          acc2[2] += (v * (long long)q.z) >> kSegValueShift;
          acc2[3] += (v * (long long)q.w) >> kSegValueShift;
        }
      }
    }
  }
  flush();
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

void launch_bucket_count(const BedView& v, const int32_t* perm, int64_t wsize, int nwin, int32_t* cnt,
                         cudaStream_t s) {
  if (nwin == 0 || v.nsamples == 0) return;
  dim3 grid(ceil_div((v.nsamples + 15) / 16, 128), nwin);
  k_buckets<false><<<grid, 128, 0, s>>>(v, perm, wsize, cnt, nullptr, nullptr, nullptr);
  PCAONE_LAUNCH_CHECK();
}

void launch_bucket_fill(const BedView& v, const int32_t* perm, int64_t wsize, int nwin, const int64_t* ptr,
                        int32_t* bpos, int32_t* bsample, cudaStream_t s) {
  if (nwin == 0 || v.nsamples == 0) return;
  dim3 grid(ceil_div((v.nsamples + 15) / 16, 128), nwin);
  k_buckets<true><<<grid, 128, 0, s>>>(v, perm, wsize, nullptr, ptr, bpos, bsample);
  PCAONE_LAUNCH_CHECK();
}

void launch_exclusive_scan(const int32_t* in, int64_t n, int64_t* out, long long* tile_sums, cudaStream_t s) {
  if (n <= 0) {
    PCAONE_CUDA(cudaMemsetAsync(out, 0, sizeof(int64_t), s));
    return;
  }
  const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  if (ntiles > 0x7fffffff) throw Error(-6, "prefix sum: too many counts");
  k_scan_tile_sums<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, tile_sums);
  PCAONE_LAUNCH_CHECK();
  k_scan_tiles<<<1, kScanThreads, 0, s>>>(tile_sums, (int)ntiles, out + n);
  PCAONE_LAUNCH_CHECK();
  k_scan_apply<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, tile_sums, out);
  PCAONE_LAUNCH_CHECK();
}

int64_t scan_tiles_needed(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

void launch_h_buckets(int64_t win, int N, int L, int LP, const int64_t* ptr, const int32_t* bpos, const double* bval,
                      const int32_t* perm, const double* scale, const float* Rf, int64_t rbase, double* Hx,
                      cudaStream_t s) {
  if (N == 0 || !bval) return;
  const unsigned nb = ceil_div((int64_t)N * 32, 256);
#define PCAONE_HB(NQ) k_h_buckets<NQ><<<nb, 256, 0, s>>>(win, N, L, LP, ptr, bpos, bval, perm, scale, Rf, rbase, Hx)
  switch ((L + 31) / 32) {
    case 1: PCAONE_HB(1); break;
    case 2: PCAONE_HB(2); break;
    case 3: PCAONE_HB(3); break;
    default: PCAONE_HB(4); break;
  }
#undef PCAONE_HB
  PCAONE_LAUNCH_CHECK();
}

void launch_seg_gather(const SegGatherArgs& a, cudaStream_t s) {
  if (a.e1 <= a.e0) return;
  if (a.LP % 4 != 0 || a.L > a.LP || a.L > 128)
    throw Error(-6, "missing-entry gather: row width must be a multiple of 4 and at most 128");
  const int gsize = std::max(kSegFetch, (a.L + 3) / 4);
  const int ngroups = 32 / gsize;
  const int64_t warps = (a.e1 - a.e0 + (int64_t)ngroups * kSegRun - 1) / ((int64_t)ngroups * kSegRun);
  const unsigned nb = ceil_div(warps * 32, 256);
  if (a.val)
    k_seg_gather<true><<<nb, 256, 0, s>>>(a, gsize, ngroups);
  else
    k_seg_gather<false><<<nb, 256, 0, s>>>(a, gsize, ngroups);
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
