// Small utility kernels: the missing-genotype lists (by position, and grouped
// by window and sample), the missing-entry term of the H product, the sign
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

// Missing genotypes grouped by (window, sample).  Window w holds positions
// [w*wsize, min((w+1)*wsize, M)); bucket w*N + i lists, in increasing
// position, the positions of window w at which sample i is missing (code 01).
// One thread per 32-bit word of a row (16 samples), grid row = window; the
// count pass writes cnt[w*N + i], the fill pass (after an exclusive scan of the
// counts into ptr) writes the positions and samples.
template <bool kFill>
__global__ void k_buckets(BedView v, const int32_t* __restrict__ perm, int64_t wsize, int32_t* __restrict__ cnt,
                          const int64_t* __restrict__ ptr, int32_t* __restrict__ bpos,
                          int32_t* __restrict__ bsample) {
  const int wd = blockIdx.x * blockDim.x + threadIdx.x;
  const int nwords = (v.nsamples + 15) >> 4;
  if (wd >= nwords) return;
  const int64_t win = blockIdx.y;
  const int64_t p0 = win * wsize;
  const int64_t p1 = p0 + wsize < v.nsnps ? p0 + wsize : v.nsnps;
  const int i0 = wd * 16;
  const int nloc = v.nsamples - i0 < 16 ? v.nsamples - i0 : 16;
  const uint32_t valid = nloc == 16 ? 0x55555555u : (((1u << (2 * nloc)) - 1u) & 0x55555555u);
  int n[16];
  int64_t off[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    n[q] = 0;
    off[q] = (kFill && q < nloc) ? ptr[win * v.nsamples + i0 + q] : 0;
  }
#pragma unroll 8
  for (int64_t p = p0; p < p1; ++p) {
    const int64_t r = perm ? (int64_t)perm[p] : p;
    const uint32_t word = reinterpret_cast<const uint32_t*>(v.bed + r * v.stride)[wd];
    uint32_t miss = word & ~(word >> 1) & valid;  // low bit set, high bit clear
    while (miss) {
      const int q = (__ffs(miss) - 1) >> 1;
      if (kFill) {
#pragma unroll
        for (int t = 0; t < 16; ++t) {
          if (t == q) {
            bpos[off[t]] = (int32_t)p;
            bsample[off[t]] = i0 + t;
            ++off[t];
          }
        }
      } else {
#pragma unroll
        for (int t = 0; t < 16; ++t) n[t] += (t == q);
      }
      miss &= miss - 1u;
    }
  }
  if (!kFill) {
#pragma unroll
    for (int q = 0; q < 16; ++q)
      if (q < nloc) cnt[win * v.nsamples + i0 + q] = n[q];
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

// One warp per chunk of 64 consecutive entries: the lanes fetch 32 entries'
// keys, source rows and quantised values at once, load the broadcast source
// rows 16 at a time (all loads independent), and sum them per key while the
// key is unchanged; a key change (warp-uniform) flushes the running sums with
// int64 atomics.
template <int NQ, bool VALS>
__global__ void k_seg_gather(SegGatherArgs a) {
  constexpr int SB = VALS ? 8 : 16;  // entries whose rows are loaded together
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t cb = a.e0 + w * 64;
  if (cb >= a.e1) return;
  const int64_t ce = cb + 64 < a.e1 ? cb + 64 : a.e1;
  const int LP = a.LP, L = a.L;
  long long acc[NQ], acc2[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = acc2[q] = 0;
  int cur = -1;
  auto flush = [&]() {
    if (cur < 0) return;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const int l = lane + 32 * q;
      if (l < L) {
        atomicAdd(a.out + (size_t)cur * LP + l, (unsigned long long)acc[q]);
        if (VALS) atomicAdd(a.out2 + (size_t)cur * LP + l, (unsigned long long)acc2[q]);
      }
      acc[q] = acc2[q] = 0;
    }
  };
  for (int64_t eb = cb; eb < ce; eb += 32) {
    const int ne = (int)(ce - eb < 32 ? ce - eb : 32);
    int krow = -1, soff = 0, vi = 0;
    if (lane < ne) {
      krow = (int)(a.key[eb + lane] - a.key_base);
      soff = (int)(a.src[eb + lane] - a.src_base) * LP;
      if (VALS) vi = __double2int_rn(a.val[eb + lane] * kSegValueScale);
    }
#pragma unroll 1
    for (int h = 0; h < ne; h += SB) {
      int m[SB][NQ], m2[VALS ? SB : 1][NQ];
#pragma unroll
      for (int u = 0; u < SB; ++u) {
        const int t = h + u;
        const int so = __shfl_sync(0xffffffffu, soff, t);
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int l = lane + 32 * q;
          const bool ok = t < ne && l < L;
          m[u][q] = ok ? a.R[so + l] : 0;
          if (VALS) m2[VALS ? u : 0][q] = ok ? a.R2[so + l] : 0;
        }
      }
#pragma unroll
      for (int u = 0; u < SB; ++u) {
        const int t = h + u;
        const int kr = __shfl_sync(0xffffffffu, krow, t);
        const int vt = VALS ? __shfl_sync(0xffffffffu, vi, t) : 0;
        if (t < ne) {
          if (kr != cur) {
            flush();
            cur = kr;
          }
#pragma unroll
          for (int q = 0; q < NQ; ++q) {
            acc[q] += m[u][q];
            if (VALS) acc2[q] += ((long long)vt * (long long)m2[VALS ? u : 0][q]) >> kSegValueShift;
          }
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

template <bool VALS>
void launch_seg_gather_v(const SegGatherArgs& a, unsigned nb, cudaStream_t s) {
  switch ((a.L + 31) / 32) {
    case 1: k_seg_gather<1, VALS><<<nb, 256, 0, s>>>(a); break;
    case 2: k_seg_gather<2, VALS><<<nb, 256, 0, s>>>(a); break;
    case 3: k_seg_gather<3, VALS><<<nb, 256, 0, s>>>(a); break;
    default: k_seg_gather<4, VALS><<<nb, 256, 0, s>>>(a); break;
  }
}

void launch_seg_gather(const SegGatherArgs& a, cudaStream_t s) {
  if (a.e1 <= a.e0) return;
  const int64_t warps = (a.e1 - a.e0 + 63) / 64;
  const unsigned nb = ceil_div(warps * 32, 256);
  if (a.val)
    launch_seg_gather_v<true>(a, nb, s);
  else
    launch_seg_gather_v<false>(a, nb, s);
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
