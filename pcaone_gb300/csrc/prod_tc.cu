// Window block products on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// With d the raw dosage (0/1/2, missing -> 0), m the missing indicator, f the
// allele frequency and s the per-SNP scale, the standardised genotype is
//     x(i,j) = s_j * (d_ij/2 - f_j + f_j m_ij)
// (mean imputation of missing entries, src/FilePlink.cpp:102-109, scaled as in
// src/Data.cpp:351-362).  The products of one SNP window are formed from the
// exact operands d and m, which are exact in BF16, and an affine epilogue:
//   G_j  = s_j * ( 1/2 (D W)_j - f_j * colsum(W) + f_j (M W)_j )
//   H_i += (D Gh)_i - c + (M Gm)_i,  Gh_j = 1/2 s_j G_j,  Gm_j = 2 f_j Gh_j,
//                                     c = sum_j 2 f_j Gh_j
// where W is the test matrix Omega as held in BF16 slices (W = sum of up to
// three BF16 slices, so that three slices carry 24 significand bits).  The
// centring terms use the same sliced values as the products, so the operator
// applied is exactly X times the sliced matrix.
//
// Kernels (one CTA = 128 threads = one warpgroup; thread 0 issues TMA and MMA):
//   k_tc_g : tile of 128 SNPs x one chunk of samples.  TMA brings the packed
//            tile (128 rows x 16 bytes) and the Omega^T slice tiles (L x 64,
//            128B swizzle); threads decode the packed bytes into the A tile(s)
//            (128 x 64 BF16, K-major, 128B swizzle); tcgen05.mma accumulates
//            D*W and M*W in TMEM; the epilogue (tcgen05.ld) writes FP32
//            partial sums, combined in FP64 by k_tc_g_finish.
//   k_tc_h : tile of 128 samples x one split of the window's SNPs.  TMA brings
//            the packed tile (64 SNP rows x 32 bytes) and the Gh^T / Gm^T slice
//            tiles; threads decode and transpose into D^T / M^T A tiles.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>

#include "internal.cuh"
#include "prod_tc.cuh"

namespace pcaone {
namespace tc {

namespace {

constexpr int kThreads = 128;
constexpr int kStepK = 64;              // K elements per pipeline stage (128 B of BF16 per row)
constexpr int kMaxStages = 4;
constexpr long long kTimeoutCycles = 4000000000ll;  // about 2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase: false after ~2 s without completion.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > kTimeoutCycles) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem desc] * B[smem desc]^T, kind::f16 (BF16 in, FP32 accumulate)
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 lanes x 8 consecutive 32-bit columns starting at taddr
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r0, r1, r2, r3, r4, r5, r6, r7;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3), "=r"(r4), "=r"(r5), "=r"(r6), "=r"(r7)
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  v[0] = __uint_as_float(r0);
  v[1] = __uint_as_float(r1);
  v[2] = __uint_as_float(r2);
  v[3] = __uint_as_float(r3);
  v[4] = __uint_as_float(r4);
  v[5] = __uint_as_float(r5);
  v[6] = __uint_as_float(r6);
  v[7] = __uint_as_float(r7);
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// core-matrix groups 1024 bytes apart (tcgen05 descriptor format, version 1).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;               // leading-dimension offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;     // stride-dimension offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;               // descriptor version
  d |= (uint64_t)2 << 61;               // SWIZZLE_128B
  return d;
}

// Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

constexpr uint16_t kBf16One = 0x3F80, kBf16Two = 0x4000;

__device__ __forceinline__ uint32_t dosage_bf16(uint32_t code) {
  // 00 -> 2, 10 -> 1, 01 and 11 -> 0
  return code == 0u ? kBf16Two : (code == 2u ? kBf16One : 0u);
}
__device__ __forceinline__ uint32_t missing_bf16(uint32_t code) { return code == 1u ? kBf16One : 0u; }

__device__ __forceinline__ uint32_t swz(uint32_t row, uint32_t chunk) {
  // byte offset of 16-byte chunk `chunk` of row `row` in a 128B-swizzled K-major tile
  return row * 128u + ((chunk ^ (row & 7u)) << 4);
}

struct SmemLayout {
  uint32_t a_d, a_m, b, p, stage_bytes;
};

__host__ __device__ inline SmemLayout layout_for(int LP, int nslice, int bparts, bool mask, int pbytes) {
  SmemLayout s{};
  uint32_t off = 0;
  s.a_d = off;
  off += 128 * 128;
  s.a_m = off;
  if (mask) off += 128 * 128;
  s.b = off;
  off += (uint32_t)(bparts * nslice * LP * 128);
  s.p = off;
  off += (uint32_t)pbytes;
  s.stage_bytes = (off + 1023u) & ~1023u;
  return s;
}

// ---------------------------------------------------------------------------
// G product
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 1)
    k_tc_g(const __grid_constant__ CUtensorMap map_bed, const __grid_constant__ CUtensorMap map_w, GArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  __shared__ uint64_t full_bar[kMaxStages], mma_bar[kMaxStages];
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh, miss_sh;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int LP = a.LP, S = a.nslice;
  const SmemLayout lay = layout_for(LP, S, 1, a.mask != 0, 128 * 16);
  const int row0 = blockIdx.x * 128;                  // window-local first SNP of the tile
  const int kbeg = blockIdx.y * a.chunk;
  const int kend = min(kbeg + a.chunk, a.npad);
  const int nk = (kend - kbeg + kStepK - 1) / kStepK;
  const int nst = a.nstages;

  if (tid == 0) {
    abort_sh = 0;
    miss_sh = 0;
    for (int s = 0; s < nst; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&mma_bar[s], 1);
    }
    fence_mbar_init();
  }
  __syncthreads();
  // does the tile hold a missing genotype? (the mask product is skipped if not)
  if (a.mask) {
    const int j = row0 + tid;
    int has = 0;
    if (j < a.nsnp) {
      const int64_t pos = a.pos0 + j;
      const int64_t snp = a.perm ? (int64_t)a.perm[pos] : pos;
      has = a.counts[snp * 4 + 1] > 0;
    }
    if (__syncthreads_or(has) && tid == 0) miss_sh = 1;
  }
  if (warp == 0) tmem_alloc(&tmem_sh, (uint32_t)a.tmem_cols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_sh;
  const bool use_m = a.mask && miss_sh;
  const uint32_t idesc = idesc_bf16(128, LP);
  const uint32_t tx_bytes = 128 * 16 + (uint32_t)(S * LP * 128);

  auto issue = [&](int stage, int kb) {
    uint8_t* base = smem + stage * lay.stage_bytes;
    const int k0 = kbeg + kb * kStepK;
    mbar_expect_tx(&full_bar[stage], tx_bytes);
    tma_load_2d(base + lay.p, &map_bed, k0 >> 2, (int)(a.pos0 + row0), &full_bar[stage]);
    for (int s = 0; s < S; ++s) tma_load_2d(base + lay.b + s * LP * 128, &map_w, k0, s * LP, &full_bar[stage]);
  };

  if (tid == 0)
    for (int s = 0; s < nst && s < nk; ++s) issue(s, s);
  int issued_upto = min(nst, nk);  // k-steps whose loads have been issued (thread 0's view)

  for (int kb = 0; kb < nk; ++kb) {
    const int stage = kb % nst;
    const uint32_t ph = (uint32_t)(kb / nst) & 1u;
    if (tid == 0 && kb >= 1 && kb - 1 + nst < nk) {
      const int ps = (kb - 1) % nst;
      if (!mbar_wait(&mma_bar[ps], (uint32_t)((kb - 1) / nst) & 1u)) {
        abort_sh = 1;
      } else {
        issue(ps, kb - 1 + nst);
        issued_upto = kb - 1 + nst + 1;
      }
    }
    if (!mbar_wait(&full_bar[stage], ph)) abort_sh = 1;
    uint8_t* base = smem + stage * lay.stage_bytes;
    // decode: thread = SNP row of the tile, 16 packed bytes = 64 samples
    {
      const uint4 pk = *reinterpret_cast<const uint4*>(base + lay.p + tid * 16);
      const uint32_t w[4] = {pk.x, pk.y, pk.z, pk.w};
#pragma unroll
      for (int c = 0; c < 8; ++c) {        // 16-byte chunk c = samples 8c .. 8c+7 (two packed bytes)
        const uint32_t bits = (w[c >> 1] >> ((c & 1) * 16)) & 0xFFFFu;
        uint32_t q[4], qm[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const uint32_t c0 = (bits >> (4 * t)) & 3u, c1 = (bits >> (4 * t + 2)) & 3u;
          q[t] = dosage_bf16(c0) | (dosage_bf16(c1) << 16);
          qm[t] = missing_bf16(c0) | (missing_bf16(c1) << 16);
        }
        *reinterpret_cast<uint4*>(base + lay.a_d + swz(tid, c)) = make_uint4(q[0], q[1], q[2], q[3]);
        if (use_m) *reinterpret_cast<uint4*>(base + lay.a_m + swz(tid, c)) = make_uint4(qm[0], qm[1], qm[2], qm[3]);
      }
    }
    fence_proxy_async();
    __syncthreads();
    if (abort_sh) break;
    if (tid == 0) {
      tc_fence_after();
      const uint32_t ad = smem_u32(base + lay.a_d), am = smem_u32(base + lay.a_m), bb = smem_u32(base + lay.b);
#pragma unroll
      for (int kk = 0; kk < kStepK / 16; ++kk) {
        for (int s = 0; s < S; ++s) {
          const uint64_t bdesc = desc_sw128(bb + s * LP * 128 + kk * 32);
          const uint32_t acc = (kb | kk | s) != 0;
          mma_bf16(tmem, desc_sw128(ad + kk * 32), bdesc, idesc, acc);
          if (use_m) mma_bf16(tmem + LP, desc_sw128(am + kk * 32), bdesc, idesc, acc);
        }
      }
      mma_commit(&mma_bar[stage]);
    }
  }
  // drain: the last committed MMA group, then any loads still in flight
  if (tid == 0) {
    if (!abort_sh && nk > 0) {
      if (!mbar_wait(&mma_bar[(nk - 1) % nst], (uint32_t)((nk - 1) / nst) & 1u)) abort_sh = 1;
    }
    if (abort_sh) {
      *a.err = 1;
      // wait (bounded) for every issued load so no copy lands after exit
      for (int kb = 0; kb < issued_upto; ++kb) mbar_wait(&full_bar[kb % nst], (uint32_t)(kb / nst) & 1u);
    }
  }
  __syncthreads();
  tc_fence_after();
  if (!abort_sh) {
    const int j = row0 + tid;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    float v[8];
    for (int c0 = 0; c0 < LP; c0 += 8) {
      if (nk > 0) {
        tmem_ld8(lane_base + c0, v);
      } else {
        for (int t = 0; t < 8; ++t) v[t] = 0.f;
      }
      if (j < a.nsnp) {
        float* dst = a.part_d + ((size_t)blockIdx.y * a.nsnp + j) * LP + c0;
        *reinterpret_cast<float4*>(dst) = make_float4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<float4*>(dst + 4) = make_float4(v[4], v[5], v[6], v[7]);
      }
      if (a.mask) {
        if (use_m && nk > 0) {
          tmem_ld8(lane_base + LP + c0, v);
        } else {
          for (int t = 0; t < 8; ++t) v[t] = 0.f;
        }
        if (j < a.nsnp) {
          float* dst = a.part_m + ((size_t)blockIdx.y * a.nsnp + j) * LP + c0;
          *reinterpret_cast<float4*>(dst) = make_float4(v[0], v[1], v[2], v[3]);
          *reinterpret_cast<float4*>(dst + 4) = make_float4(v[4], v[5], v[6], v[7]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
}

// ---------------------------------------------------------------------------
// H product
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 1)
    k_tc_h(const __grid_constant__ CUtensorMap map_bed, const __grid_constant__ CUtensorMap map_g, HArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  __shared__ uint64_t full_bar[kMaxStages], mma_bar[kMaxStages];
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  __shared__ uint2 lut[256];   // packed byte -> dosage (BF16) of its 4 samples
  __shared__ uint2 lutm[256];  // packed byte -> missing indicator (BF16) of its 4 samples
  const int tid = threadIdx.x, warp = tid >> 5;
  const int LP = a.LP, S = a.nslice;
  const bool mask = a.mask != 0;
  const SmemLayout lay = layout_for(LP, S, mask ? 2 : 1, mask, 64 * 32);
  const int samp0 = blockIdx.x * 128;
  const int jb = blockIdx.y * a.per_split;
  const int je = min(jb + a.per_split, a.nsnp);
  const int nk = je > jb ? (je - jb + kStepK - 1) / kStepK : 0;
  const int nst = a.nstages;

  for (int b = tid; b < 256; b += kThreads) {
    const uint32_t d0 = dosage_bf16(b & 3), d1 = dosage_bf16((b >> 2) & 3), d2 = dosage_bf16((b >> 4) & 3),
                   d3 = dosage_bf16((b >> 6) & 3);
    lut[b] = make_uint2(d0 | (d1 << 16), d2 | (d3 << 16));
    const uint32_t m0 = missing_bf16(b & 3), m1 = missing_bf16((b >> 2) & 3), m2 = missing_bf16((b >> 4) & 3),
                   m3 = missing_bf16((b >> 6) & 3);
    lutm[b] = make_uint2(m0 | (m1 << 16), m2 | (m3 << 16));
  }
  if (tid == 0) {
    abort_sh = 0;
    for (int s = 0; s < nst; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&mma_bar[s], 1);
    }
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(&tmem_sh, (uint32_t)a.tmem_cols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_sh;
  const uint32_t idesc = idesc_bf16(128, LP);
  const int bparts = mask ? 2 : 1;
  const uint32_t tx_bytes = 64 * 32 + (uint32_t)(bparts * S * LP * 128);

  auto issue = [&](int stage, int kb) {
    uint8_t* base = smem + stage * lay.stage_bytes;
    const int j0 = jb + kb * kStepK;
    mbar_expect_tx(&full_bar[stage], tx_bytes);
    tma_load_2d(base + lay.p, &map_bed, samp0 >> 2, (int)(a.pos0 + j0), &full_bar[stage]);
    for (int r = 0; r < bparts * S; ++r)
      tma_load_2d(base + lay.b + r * LP * 128, &map_g, j0, r * LP, &full_bar[stage]);
  };
  if (tid == 0)
    for (int s = 0; s < nst && s < nk; ++s) issue(s, s);
  int issued_upto = min(nst, nk);

  // decode assignment: byte column q (4 samples), SNP group g (16 SNPs)
  const int q = tid & 31, g = tid >> 5;
  for (int kb = 0; kb < nk; ++kb) {
    const int stage = kb % nst;
    const uint32_t ph = (uint32_t)(kb / nst) & 1u;
    if (tid == 0 && kb >= 1 && kb - 1 + nst < nk) {
      const int ps = (kb - 1) % nst;
      if (!mbar_wait(&mma_bar[ps], (uint32_t)((kb - 1) / nst) & 1u)) {
        abort_sh = 1;
      } else {
        issue(ps, kb - 1 + nst);
        issued_upto = kb - 1 + nst + 1;
      }
    }
    if (!mbar_wait(&full_bar[stage], ph)) abort_sh = 1;
    uint8_t* base = smem + stage * lay.stage_bytes;
    {
      // 16 SNP rows of byte column q -> for each of the 4 samples 4q..4q+3,
      // 16 consecutive K elements (two 16-byte chunks 2g, 2g+1)
      uint2 lv[16];
#pragma unroll
      for (int jj = 0; jj < 16; ++jj) lv[jj] = lut[base[lay.p + (g * 16 + jj) * 32 + q]];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const uint32_t row = (uint32_t)(q * 4 + t);
        const uint32_t sel = (t & 1) ? 0x7632u : 0x5410u;
        uint32_t w[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const uint32_t lo = (t < 2) ? lv[2 * e].x : lv[2 * e].y;
          const uint32_t hi = (t < 2) ? lv[2 * e + 1].x : lv[2 * e + 1].y;
          w[e] = __byte_perm(lo, hi, sel);
        }
        *reinterpret_cast<uint4*>(base + lay.a_d + swz(row, 2 * g)) = make_uint4(w[0], w[1], w[2], w[3]);
        *reinterpret_cast<uint4*>(base + lay.a_d + swz(row, 2 * g + 1)) = make_uint4(w[4], w[5], w[6], w[7]);
      }
      if (mask) {
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) lv[jj] = lutm[base[lay.p + (g * 16 + jj) * 32 + q]];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const uint32_t row = (uint32_t)(q * 4 + t);
          const uint32_t sel = (t & 1) ? 0x7632u : 0x5410u;
          uint32_t w[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            const uint32_t lo = (t < 2) ? lv[2 * e].x : lv[2 * e].y;
            const uint32_t hi = (t < 2) ? lv[2 * e + 1].x : lv[2 * e + 1].y;
            w[e] = __byte_perm(lo, hi, sel);
          }
          *reinterpret_cast<uint4*>(base + lay.a_m + swz(row, 2 * g)) = make_uint4(w[0], w[1], w[2], w[3]);
          *reinterpret_cast<uint4*>(base + lay.a_m + swz(row, 2 * g + 1)) = make_uint4(w[4], w[5], w[6], w[7]);
        }
      }
    }
    fence_proxy_async();
    __syncthreads();
    if (abort_sh) break;
    if (tid == 0) {
      tc_fence_after();
      const uint32_t ad = smem_u32(base + lay.a_d), am = smem_u32(base + lay.a_m), bb = smem_u32(base + lay.b);
#pragma unroll
      for (int kk = 0; kk < kStepK / 16; ++kk) {
        for (int s = 0; s < S; ++s) {
          const uint32_t acc = (kb | kk | s) != 0;
          mma_bf16(tmem, desc_sw128(ad + kk * 32), desc_sw128(bb + s * LP * 128 + kk * 32), idesc, acc);
          if (mask)
            mma_bf16(tmem, desc_sw128(am + kk * 32), desc_sw128(bb + (S + s) * LP * 128 + kk * 32), idesc, 1u);
        }
      }
      mma_commit(&mma_bar[stage]);
    }
  }
  if (tid == 0) {
    if (!abort_sh && nk > 0) {
      if (!mbar_wait(&mma_bar[(nk - 1) % nst], (uint32_t)((nk - 1) / nst) & 1u)) abort_sh = 1;
    }
    if (abort_sh) {
      *a.err = 1;
      for (int kb = 0; kb < issued_upto; ++kb) mbar_wait(&full_bar[kb % nst], (uint32_t)(kb / nst) & 1u);
    }
  }
  __syncthreads();
  tc_fence_after();
  if (!abort_sh) {
    const int i = samp0 + tid;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    float v[8];
    for (int c0 = 0; c0 < LP; c0 += 8) {
      if (nk > 0) {
        tmem_ld8(lane_base + c0, v);
      } else {
        for (int t = 0; t < 8; ++t) v[t] = 0.f;
      }
      float* dst = a.hpart + ((size_t)blockIdx.y * a.npad + i) * LP + c0;
      *reinterpret_cast<float4*>(dst) = make_float4(v[0], v[1], v[2], v[3]);
      *reinterpret_cast<float4*>(dst + 4) = make_float4(v[4], v[5], v[6], v[7]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
}

// ---------------------------------------------------------------------------
// FP64 epilogues and operand preparation
// ---------------------------------------------------------------------------

// W slices (BF16, S*LP rows x npad, K-major) of Omega (npad x LP FP64) and the
// column sums of the sliced matrix over the real samples.  One thread per
// (sample, column); column sums by a second kernel.
__global__ void k_omega_slices(const double* __restrict__ omg, int npad, int N, int LP, int S,
                               __nv_bfloat16* __restrict__ w) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)npad * LP) return;
  const int i = (int)(idx / LP), l = (int)(idx % LP);
  double r = i < N ? omg[idx] : 0.0;
  for (int s = 0; s < S; ++s) {
    const __nv_bfloat16 h = __double2bfloat16(r);
    w[((size_t)s * LP + l) * npad + i] = h;
    r -= (double)__bfloat162float(h);
  }
}

__global__ void k_omega_colsum(const __nv_bfloat16* __restrict__ w, int npad, int N, int LP, int S,
                               double* __restrict__ colsum) {
  const int l = blockIdx.x;
  double acc = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double v = 0.0;
    for (int s = 0; s < S; ++s) v += (double)__bfloat162float(w[((size_t)s * LP + l) * npad + i]);
    acc += v;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) colsum[l] = red[0];
}

// G rows: FP64 epilogue of the chunk partials plus the EM sparse term; B
// operand slices of Gh = 1/2 s G and Gm = 2 f Gh for the H product (columns
// nsnp .. ld-1 zeroed).
__global__ void k_tc_g_finish(GFinishArgs a) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t total = (int64_t)a.ldg * a.LP;
  if (idx >= total) return;
  const int j = (int)(idx / a.LP), l = (int)(idx % a.LP);
  const int S = a.nslice, LP = a.LP;
  double gm = 0.0;
  if (j < a.nsnp && l < a.L) {
    const int64_t pos = a.pos0 + j;
    const int64_t snp = a.perm ? (int64_t)a.perm[pos] : pos;
    const double f = a.F[snp], s = a.scale[snp];
    double pd = 0.0, pm = 0.0;
    for (int c = 0; c < a.nchunks; ++c) {
      pd += (double)a.part_d[((size_t)c * a.nsnp + j) * LP + l];
      if (a.part_m) pm += (double)a.part_m[((size_t)c * a.nsnp + j) * LP + l];
    }
    double g = s * (0.5 * pd - f * a.colsum[l] + f * pm);
    if (a.sp.active) {
      double sacc = 0.0;
      for (int64_t e = a.sp.rowptr[pos]; e < a.sp.rowptr[pos + 1]; ++e)
        sacc += a.sp.value[e] * a.omg[(size_t)a.sp.sample[e] * LP + l];
      g += s * sacc;
    }
    a.G[pos * LP + l] = g;
    // Gh slices; Gm from the sliced Gh so that the centring stays consistent
    double r = 0.5 * s * g, ghq = 0.0;
    for (int t = 0; t < S; ++t) {
      const __nv_bfloat16 h = __double2bfloat16(r);
      a.gt[((size_t)t * LP + l) * a.ldg + j] = h;
      const double hv = (double)__bfloat162float(h);
      ghq += hv;
      r -= hv;
    }
    gm = 2.0 * f * ghq;
    if (a.mask) {
      double rm = gm;
      for (int t = 0; t < S; ++t) {
        const __nv_bfloat16 h = __double2bfloat16(rm);
        a.gt[((size_t)(S + t) * LP + l) * a.ldg + j] = h;
        rm -= (double)__bfloat162float(h);
      }
    }
    a.cpart[(size_t)j * LP + l] = gm;  // c_l = sum_j 2 f_j Gh_j
  } else {
    for (int t = 0; t < S; ++t) a.gt[((size_t)t * LP + l) * a.ldg + j] = __float2bfloat16(0.f);
    if (a.mask)
      for (int t = 0; t < S; ++t) a.gt[((size_t)(S + t) * LP + l) * a.ldg + j] = __float2bfloat16(0.f);
    if (j < a.nsnp) a.cpart[(size_t)j * LP + l] = 0.0;
  }
}

__global__ void k_colreduce(const double* __restrict__ part, int rows, int LP, double* __restrict__ out) {
  const int l = blockIdx.x;
  double acc = 0.0;
  for (int r = threadIdx.x; r < rows; r += blockDim.x) acc += part[(size_t)r * LP + l];
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[l] = red[0];
}

__global__ void k_tc_h_finish(int nsamples, int npad, int L, int LP, const float* __restrict__ hpart, int nsplit,
                              const double* __restrict__ c, double* __restrict__ Hx) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nsamples * LP) return;
  const int64_t i = idx / LP;
  const int l = (int)(idx - i * LP);
  if (l >= L) return;
  double acc = 0.0;
  for (int s = 0; s < nsplit; ++s) acc += (double)hpart[((size_t)s * npad + i) * LP + l];
  Hx[idx] += acc - c[l];
}

__global__ void k_gather_rows(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, int64_t stride,
                              const int32_t* __restrict__ perm, int64_t nrows) {
  const int64_t r = blockIdx.x;
  if (r >= nrows) return;
  const uint4* s = reinterpret_cast<const uint4*>(src + (int64_t)perm[r] * stride);
  uint4* d = reinterpret_cast<uint4*>(dst + r * stride);
  for (int64_t q = threadIdx.x; q < stride / 16; q += blockDim.x) d[q] = s[q];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    PCAONE_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p) throw Error(-2, "cuTensorMapEncodeTiled unavailable");
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

}  // namespace

void make_map_2d(CUtensorMap* map, const void* base, bool bf16, uint64_t inner, uint64_t outer, uint64_t pitch_bytes,
                 uint32_t box_inner, uint32_t box_outer, bool swizzle128) {
  const cuuint64_t dims[2] = {inner, outer};
  const cuuint64_t strides[1] = {pitch_bytes};
  const cuuint32_t box[2] = {box_inner, box_outer};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = encode_fn()(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_UINT8, 2,
                                 const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(-2, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

int stages_for(int LP, int nslice, int bparts, bool mask, int pbytes) {
  const SmemLayout l = layout_for(LP, nslice, bparts, mask, pbytes);
  const int budget = 200 * 1024;
  return std::max(1, std::min(kMaxStages, budget / (int)l.stage_bytes));
}

size_t smem_bytes(int LP, int nslice, int bparts, bool mask, int pbytes, int nstages) {
  return (size_t)layout_for(LP, nslice, bparts, mask, pbytes).stage_bytes * nstages + 1024;
}

int tmem_cols_for(int ncols) {
  int c = 32;
  while (c < ncols) c <<= 1;
  return c;
}

void launch_g(const CUtensorMap& map_bed, const CUtensorMap& map_w, const GArgs& a, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    PCAONE_CUDA(cudaFuncSetAttribute(k_tc_g, cudaFuncAttributeMaxDynamicSharedMemorySize, 210 * 1024));
    attr = true;
  }
  const size_t smem = smem_bytes(a.LP, a.nslice, 1, a.mask != 0, 128 * 16, a.nstages);
  dim3 grid((a.nsnp + 127) / 128, a.nchunks);
  k_tc_g<<<grid, kThreads, smem, s>>>(map_bed, map_w, a);
  PCAONE_LAUNCH_CHECK();
}

void launch_h(const CUtensorMap& map_bed, const CUtensorMap& map_g, const HArgs& a, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    PCAONE_CUDA(cudaFuncSetAttribute(k_tc_h, cudaFuncAttributeMaxDynamicSharedMemorySize, 210 * 1024));
    attr = true;
  }
  const size_t smem = smem_bytes(a.LP, a.nslice, a.mask ? 2 : 1, a.mask != 0, 64 * 32, a.nstages);
  dim3 grid(a.npad / 128, a.nsplit);
  k_tc_h<<<grid, kThreads, smem, s>>>(map_bed, map_g, a);
  PCAONE_LAUNCH_CHECK();
}

void launch_omega_slices(const double* omg, int npad, int N, int LP, int S, __nv_bfloat16* w, double* colsum,
                         cudaStream_t s) {
  const int64_t n = (int64_t)npad * LP;
  k_omega_slices<<<ceil_div(n, 256), 256, 0, s>>>(omg, npad, N, LP, S, w);
  PCAONE_LAUNCH_CHECK();
  k_omega_colsum<<<LP, 256, 0, s>>>(w, npad, N, LP, S, colsum);
  PCAONE_LAUNCH_CHECK();
}

void launch_g_finish(const GFinishArgs& a, double* c_out, cudaStream_t s) {
  const int64_t n = (int64_t)a.ldg * a.LP;
  k_tc_g_finish<<<ceil_div(n, 256), 256, 0, s>>>(a);
  PCAONE_LAUNCH_CHECK();
  k_colreduce<<<a.LP, 256, 0, s>>>(a.cpart, a.nsnp, a.LP, c_out);
  PCAONE_LAUNCH_CHECK();
}

void launch_h_finish(int nsamples, int npad, int L, int LP, const float* hpart, int nsplit, const double* c,
                     double* Hx, cudaStream_t s) {
  const int64_t n = (int64_t)nsamples * LP;
  k_tc_h_finish<<<ceil_div(n, 256), 256, 0, s>>>(nsamples, npad, L, LP, hpart, nsplit, c, Hx);
  PCAONE_LAUNCH_CHECK();
}

void launch_gather_rows(const uint8_t* src, uint8_t* dst, int64_t stride, const int32_t* perm, int64_t nrows,
                        cudaStream_t s) {
  if (nrows == 0) return;
  k_gather_rows<<<(unsigned)nrows, 128, 0, s>>>(src, dst, stride, perm, nrows);
  PCAONE_LAUNCH_CHECK();
}

}  // namespace tc
}  // namespace pcaone
