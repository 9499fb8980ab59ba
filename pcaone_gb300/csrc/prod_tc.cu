// Window block products on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// With d the raw dosage (0/1/2, missing -> 0), m the missing indicator, f the
// allele frequency, s the per-SNP scale and e the EM fill value of a missing
// entry (0 under mean imputation), the standardised genotype is
//     x(i,j) = s_j * (d_ij/2 - f_j + (f_j + e_ij) m_ij)
// (mean imputation of missing entries, src/FilePlink.cpp:102-109, scaled as in
// src/Data.cpp:351-362; the EM fill of src/Data.cpp:318-348).  The products of
// one SNP window are formed from the dosages d, which are exact in BF16, an
// affine epilogue, and a sparse term over the missing entries only:
//   G_j  = s_j * ( 1/2 (D W)_j - f_j * colsum(W) + sum_{i missing} (f_j + e_ij) W_i )
//   H_i += (D Gh)_i - c + sum_{j missing} 2 (f_j + e_ij) Gh_j,
//          Gh_j = 1/2 s_j G_j,  c = sum_j 2 f_j Gh_j
// where W is the test matrix Omega held as S integer slices (S = 1 or 3):
// per column l a power-of-two unit u_ls = 2^(E_l - 8 - 9s) with
// max_i |Omega_il| < 2^E_l, and W_il = sum_s u_ls * w_sil with integers
// |w_sil| <= 256, exact in BF16 (Ozaki-style error-free splitting with
// balanced base-512 digits; three slices carry 27 significand bits).  Each
// slice has its own TMEM accumulator: the products d*w are integers of
// magnitude <= 512 and every partial sum of a CTA (K <= kMaxKExact = 16384)
// stays below 2^23, so the tensor core accumulates exactly and no rounding
// enters; the epilogue combines the slices exactly in int64, and one FP64
// conversion per output follows.  Gh is split the same way (per-column units
// over the window).  The centring and missing-entry terms use the same
// represented values as the products, so the operator applied is exactly X
// times the sliced matrix.
//
// Kernels (one CTA = 320 threads in three roles, see role_wait below; two
// CTAs share an SM when their TMEM plans fit in half of it, see pair_per_sm):
//   k_tc_g : tile of 128 SNPs x one chunk of samples.  TMA brings the packed
//            tile (128 rows x 16 bytes) and the W^T slice tiles (S*L rows x 64,
//            128B swizzle, K-major B operand); decoder warps turn the packed
//            bytes into the BF16 dosage operand D, written straight into TMEM
//            (tcgen05.st); tcgen05.mma (A from TMEM, B from shared memory, the
//            S slices concatenated along N) accumulates D*W in TMEM; the
//            epilogue (tcgen05.ld) writes FP32 partial sums, combined by
//            k_tc_g_finish.
//   k_tc_h : tile of 128 samples x one split of the window's SNPs.  TMA brings
//            the packed tile (64 SNP rows x 32 bytes) and the Gh^T slice tiles;
//            decoder warps transpose into the D^T A operand.
//
// Dense input (FileBinary values held as FP16, src/FileBinary.cpp:54-64): the
// same kernels with kDense, where the A tile is FP16 values instead of packed
// codes (copied, or transposed for H, into a 128B-swizzled A tile in shared
// memory, so that both MMA operands come from shared memory), the slices are FP16 integer
// digits (both operands of kind::f16 FP16), the centring is by the per-SNP
// mean mu with no scale (x = v - mu), and the FP32 accumulation is ordinary
// rounding arithmetic since the values are not integers.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cuda_fp8.h>

#include <algorithm>
#include <cstring>

#include "internal.cuh"
#include "prod_tc.cuh"

namespace pcaone {
namespace tc {

namespace {

constexpr int kThreads = 320;          // 10 warps: TMA producer, MMA issuer, 8 decode / TMEM-epilogue warps
constexpr int kStepK = 64;              // K elements per pipeline stage (128 B of BF16 per row)
constexpr int kMaxStages = 8;
constexpr long long kTimeoutCycles = 4000000000ll;  // about 2 s at 2 GHz

// 2^e as a double (exact; the bit pattern directly for normal results)
__device__ __forceinline__ double exp2i(int e) {
  if (e < -1022 || e > 1023) return ldexp(1.0, e);
  return __longlong_as_double((long long)(e + 1023) << 52);
}

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

// Pull a 2-D box into L2 ahead of its TMA load (no shared-memory side effect).
__device__ __forceinline__ void tma_prefetch_2d(const CUtensorMap* map, int c0, int c1) {
  asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];" ::"l"(reinterpret_cast<uint64_t>(map)),
               "r"(c0), "r"(c1)
               : "memory");
}

constexpr int kPrefetchSteps = 8;  // packed tiles are pulled into L2 this many steps ahead

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

// D[tmem] (+)= A[tmem] * B[smem desc]^T, kind::f16; A rows = TMEM lanes, two
// BF16 K elements per 32-bit column
__device__ __forceinline__ void mma_bf16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// D[tmem] (+)= A[smem desc] * B[smem desc]^T, kind::f16 (both operands K-major
// in shared memory)
__device__ __forceinline__ void mma_bf16_ss(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// generic-proxy shared-memory writes made visible to the async proxy (the
// tensor core reads the decoded A operand)
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// one decoder thread's 64 bytes of an A row (K elements 32ch .. 32ch+31 of row
// r) into the 128B-swizzled K-major tile: 16-byte chunk c of row r sits at
// chunk position c ^ (r & 7)
__device__ __forceinline__ void st_a_row(uint8_t* tile, int r, int ch, const uint32_t* wd) {
  uint8_t* row = tile + r * 128;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int cpos = (ch * 4 + q) ^ (r & 7);
    *reinterpret_cast<uint4*>(row + cpos * 16) = make_uint4(wd[4 * q], wd[4 * q + 1], wd[4 * q + 2], wd[4 * q + 3]);
  }
}

// 32 lanes x 16 consecutive 32-bit columns from registers into TMEM
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t* r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

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

// Instruction descriptor, kind::f16: D FP32, A and B both BF16 (or both FP16),
// both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// Instruction descriptor, kind::f8f6f4: D FP32, A and B both E4M3 (format 0),
// both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_e4m3(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A[tmem] * B[smem desc]^T, kind::f8f6f4 (E4M3); A rows = TMEM
// lanes, four E4M3 K elements per 32-bit column
__device__ __forceinline__ void mma_e4m3_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}


// SWAR decode of two 2-bit codes held at bits 0-1 and 16-17 of x into two BF16
// values (low and high half-words): dosage 00 -> 2.0 (0x4000), 10 -> 1.0
// (0x3F80), 01 (missing) and 11 -> 0.
__device__ __forceinline__ uint32_t dosage_pair(uint32_t x) {
  const uint32_t lo = x & 0x00010001u, hi = (x >> 1) & 0x00010001u;
  return (0x40004000u - (hi << 7)) & ~(lo * 0xFFFFu);
}


// Decode table: the two BF16 dosages of a 4-bit pair of codes (two samples or
// two SNPs; the first code in bits 0-1 gives the low half-word), from
// dosage_pair.  32 copies, entry n of copy c at word n * 32 + c, so that lane c
// always reads bank c: a lookup is conflict-free whatever the codes.  It
// replaces the SWAR arithmetic (about eleven integer operations per word,
// which kept the ALU pipe at two thirds of its peak) by two and a load.
constexpr int kLutWords = 16 * 32;
__device__ __forceinline__ void lut_init(uint32_t* lut, int tid, int nthreads) {
  for (int i = tid; i < kLutWords; i += nthreads) {
    const uint32_t n = (uint32_t)i >> 5;
    lut[i] = dosage_pair((n & 3u) | (((n >> 2) & 3u) << 16));
  }
}

// The FP8 form's decode, in registers: four E4M3 words (four dosages each,
// first code in the low byte) from the 16 2-bit codes of w (code i in bits
// 2i .. 2i+1).  Each half-word's eight codes are spread to one per nibble
// (a byte permute and two shift-and-mask steps), and every nibble selects a
// byte of the table {0x40 (00: 2.0), 0x00 (01: missing), 0x38 (10: 1.0),
// 0x00 (11)} in a second byte permute: four integer operations per word and
// no shared-memory lookup (a table in shared memory cost two lookups and about
// eight operations per word).
__device__ __forceinline__ void e4m3_x16(uint32_t w, uint32_t* out) {
  constexpr uint32_t kTab = 0x00380040u;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    uint32_t x = __byte_perm(w, 0u, h ? 0x4342u : 0x4140u);  // bytes 2h, 2h+1 -> bytes 0, 2
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    out[2 * h] = __byte_perm(kTab, 0u, x);  // selectors: the low four nibbles
    out[2 * h + 1] = __byte_perm(kTab, 0u, x >> 16);
  }
}

// One stage of a warp transpose of a 32 x 32 matrix of 2-bit codes held as
// 64 bits per lane (lo: positions 0-15, hi: 16-31): lanes exchange lane bit K
// with position bit K (Hacker's Delight 7-3, across lanes with shuffles).
// Stage 4 swaps whole words; stages 3..0 move the masked halves of each word.
template <int K>
__device__ __forceinline__ void xpose2_stage(uint32_t& lo, uint32_t& hi, int lane) {
  constexpr uint32_t m = K == 3 ? 0x0000FFFFu : K == 2 ? 0x00FF00FFu : K == 1 ? 0x0F0F0F0Fu : 0x33333333u;
  constexpr int sh = 2 << K;  // bits per block of 2^K positions
  const bool up = (lane >> K) & 1;
  const uint32_t sm = up ? m : ~m;
  const uint32_t rl = __shfl_xor_sync(0xffffffffu, lo & sm, 1 << K);
  const uint32_t rh = __shfl_xor_sync(0xffffffffu, hi & sm, 1 << K);
  lo = up ? ((lo & ~m) | (rl >> sh)) : ((lo & m) | (rl << sh));
  hi = up ? ((hi & ~m) | (rh >> sh)) : ((hi & m) | (rh << sh));
}
__device__ __forceinline__ void xpose2_warp(uint32_t& lo, uint32_t& hi, int lane) {
  const bool up = (lane >> 4) & 1;
  const uint32_t r = __shfl_xor_sync(0xffffffffu, up ? lo : hi, 16);
  if (up)
    lo = r;
  else
    hi = r;
  xpose2_stage<3>(lo, hi, lane);
  xpose2_stage<2>(lo, hi, lane);
  xpose2_stage<1>(lo, hi, lane);
  xpose2_stage<0>(lo, hi, lane);
}

struct SmemLayout {
  uint32_t b, a, p, stage_bytes;
};

// one pipeline stage in shared memory: the B slices (nslice * LP rows of 128
// bytes, 128B-swizzled), for dense input the A tile (128 rows of 64 FP16 K
// elements, the same layout), and the packed (or FP16) input tile.  LP is a
// multiple of 16, so every region starts on a 1024-byte swizzle atom.
//
// Where the A operand lives: genotype A tiles go to TMEM (tcgen05.st), dense
// ones to shared memory.  With A in shared memory the MMAs read both operands
// there, which on the 100,000 x 7,812 genotype window made the products 20%
// (two CTAs per SM) to 50% (one CTA) slower than A in TMEM; for FP16 input,
// whose A tile is a copy rather than a decode, shared memory was 18% faster
// end to end (100,000 x 100,000).
constexpr uint32_t kATileBytes = 128 * 128;
__host__ __device__ inline SmemLayout layout_for(int LP, int nslice, int pbytes, bool a_smem) {
  SmemLayout s{};
  s.b = 0;
  s.a = (uint32_t)(nslice * LP * 128);
  s.p = s.a + (a_smem ? kATileBytes : 0u);
  s.stage_bytes = (s.p + (uint32_t)pbytes + 1023u) & ~1023u;
  return s;
}

// Issue D[tmem col0 ...] (+)= A * [B rows b_row0 .. b_row0+ncols)^T for one
// 16-wide K step, the B rows (the slices of one operand, contiguous in shared
// memory) concatenated along N and cut into MMAs of at most kMaxNTmemA columns
// (n0 is a multiple of 256 rows, so every B sub-tile starts on a 1024-byte
// swizzle-atom boundary).
// MMA shape limit for M = 128: N <= 256 columns.
constexpr int kMaxNTmemA = 256;

// Kernel forms: genotypes with BF16 operands (dosages in TMEM), dense FP16
// values (A in shared memory), genotypes with E4M3 operands (the FP8 form).
// A pipeline stage covers 64 K elements of 16-bit operands or 128 of 8-bit
// ones: 128-byte rows of B either way, 32 TMEM columns of A, four MMAs of 32
// bytes of K.
constexpr int kModeGeno = 0, kModeDense = 1, kModeGeno8 = 2;

// The MMAs of one pipeline stage: four K steps of 32 bytes over the slices
// concatenated along N, cut into MMAs of at most 256 columns.  The issuing
// thread shares its SM sub-partition with decoder warps, so every instruction
// it needs costs several cycles: the shared-memory descriptors are advanced by
// adding offsets to precomputed ones (their address field counts 16-byte
// units; 32 bytes of K = 2, 256 B rows = 2048), and the instruction
// descriptors of the two column chunks come precomputed.  a_tmem: the stage's
// A operand in TMEM (!kASmem), a_desc: its shared-memory descriptor (kASmem).
template <int kMode, bool kASmem>
__device__ __forceinline__ void mma_stage(uint32_t tmem_d, uint32_t a_tmem, uint64_t a_desc, uint64_t b_desc,
                                          int ncat, uint32_t id0, uint32_t id1, bool first) {
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    const uint32_t acc = (first && kk == 0) ? 0u : 1u;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      if (c == 1 && ncat <= kMaxNTmemA) break;
      const uint64_t bd = b_desc + (uint64_t)(2 * kk + c * (kMaxNTmemA * 128 / 16));
      const uint32_t id = c ? id1 : id0;
      const uint32_t d = tmem_d + (uint32_t)(c * kMaxNTmemA);
      if constexpr (kMode == kModeGeno8)
        mma_e4m3_ta(d, a_tmem + kk * 8, bd, id, acc);
      else if constexpr (kASmem)
        mma_bf16_ss(d, a_desc + (uint64_t)(2 * kk), bd, id, acc);
      else
        mma_bf16_ta(d, a_tmem + kk * 8, bd, id, acc);
    }
  }
}

template <int kMode>
__host__ __device__ constexpr uint32_t idesc_of(int n) {
  return kMode == kModeGeno8 ? idesc_e4m3(128, n) : kMode == kModeDense ? idesc_f16(128, n) : idesc_bf16(128, n);
}

// Warp roles of both kernels (320 threads): warp 0 lane 0 issues the TMA
// loads of each pipeline stage, warp 1 lane 0 issues the MMAs, warps 2-9
// decode the packed tile into the A operand(s) and finally read the
// accumulators out of TMEM (warp w may only reach lanes 32*(w%4) .. +31;
// warps 2-5 cover the four lane quarters for the first half of the columns
// and warps 6-9 for the second).  Per stage s: full[s]
// (TMA bytes landed), dec[s] (256 decoder arrivals), empty[s]
// (tcgen05.commit of the stage's MMAs).  Every wait is bounded; a role that gives up sets the shared
// abort flag, which makes every other wait return, so the CTA always reaches
// its final barrier and frees its TMEM.
constexpr int kDecodeWarp0 = 2;
constexpr int kDecoders = 256;

// limit: cycles before the wait gives up (the kernel argument wait_cycles;
// kTimeoutCycles when it is 0)
__device__ __forceinline__ bool role_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          long long limit) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (*abort_flag) return false;
    if (clock64() - t0 > limit) {
      *abort_flag = 1;
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// After an abort: wait (each wait bounded) for the TMA copies that may still
// be in flight.  Stage st is reused only after its previous copy was consumed,
// so only the last nst issued copies can be pending; waiting on older phases
// would alias their parity with the stage's current phase.
__device__ __forceinline__ void drain_copies(uint64_t* full_bar, int issued, int nst) {
  for (int kb = issued > nst ? issued - nst : 0; kb < issued; ++kb)
    mbar_wait(&full_bar[kb % nst], (uint32_t)(kb / nst) & 1u);
}

// End of a CTA: after an abort the epilogue has not waited for the MMAs (acc_bar
// arrives once every issued MMA has completed; the MMA thread always commits
// it), so warp 0 waits for it, bounded, before it frees the TMEM.
__device__ __forceinline__ void cta_release(uint64_t& acc_bar, volatile int& abort_flag, int warp, int lane,
                                            uint32_t tmem, uint32_t cols) {
  if (warp != 0) return;
  if (abort_flag && lane == 0) mbar_wait(&acc_bar, 0u);
  __syncwarp();
  tc_fence_after();
  tmem_dealloc(tmem, cols);
}

// Epilogue helpers.  The accumulator of slice s for columns c0 .. c0+7 of a
// lane sits at TMEM columns s*LP + c0 ...
//
// Genotype input: each slice sum is an exact integer (|v| <= 512 K <= 2^23),
// so the slices combine exactly in int64, in units of the last slice:
//   P = sum_s v_s B^(S-1-s)   (digit base B = 2^db: 512, or 16 in the FP8
//   form; |P| < 2^42 for three 9-bit slices)
__device__ __forceinline__ void combine_slices_exact(uint32_t lane_base, int c0, int LP, int S, long long* acc,
                                                     int db) {
  float v[8];
  for (int s = 0; s < S; ++s) {
    tmem_ld8(lane_base + s * LP + c0, v);
#pragma unroll
    for (int t = 0; t < 8; ++t) acc[t] = acc[t] * (1 << db) + __float2ll_rn(v[t]);
  }
}
// Dense input: slice sums times their power-of-two units, smallest units first
// so that the FP32 sum rounds as little as possible
__device__ __forceinline__ void store_slice_sum(uint32_t lane_base, int c0, int LP, int S, const float* unit,
                                                float* sum) {
  float v[8];
  for (int s = S - 1; s >= 0; --s) {
    tmem_ld8(lane_base + s * LP + c0, v);
#pragma unroll
    for (int t = 0; t < 8; ++t) sum[t] = fmaf(unit[s * LP + c0 + t], v[t], sum[t]);
  }
}
// More than kIntSlices slices (the 54-bit form): the leading three and the
// remaining slices each combine exactly in int64 (below 2^42), then
// P = hi * 512^(S-3) + lo in FP64 (one rounding)
__device__ __forceinline__ void combine_slices_fp64(uint32_t lane_base, int c0, int LP, int S, double* out) {
  float v[8];
  long long hi[8] = {0, 0, 0, 0, 0, 0, 0, 0}, lo[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int s = 0; s < S; ++s) {
    tmem_ld8(lane_base + s * LP + c0, v);
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      if (s < kIntSlices)
        hi[t] = hi[t] * (1 << kDigitBits) + __float2ll_rn(v[t]);
      else
        lo[t] = lo[t] * (1 << kDigitBits) + __float2ll_rn(v[t]);
    }
  }
  const double sh = exp2i(kDigitBits * (S - kIntSlices));
#pragma unroll
  for (int t = 0; t < 8; ++t) out[t] = fma((double)hi[t], sh, (double)lo[t]);
}
__device__ __forceinline__ void store_f64x8(double* dst, const double* v) {
#pragma unroll
  for (int t = 0; t < 8; t += 2) *reinterpret_cast<double2*>(dst + t) = make_double2(v[t], v[t + 1]);
}
__device__ __forceinline__ void store_f32x8(float* dst, const float* v) {
  *reinterpret_cast<float4*>(dst) = make_float4(v[0], v[1], v[2], v[3]);
  *reinterpret_cast<float4*>(dst + 4) = make_float4(v[4], v[5], v[6], v[7]);
}
__device__ __forceinline__ void store_i64x8(long long* dst, const long long* v) {
#pragma unroll
  for (int t = 0; t < 8; t += 2) *reinterpret_cast<longlong2*>(dst + t) = make_longlong2(v[t], v[t + 1]);
}

// ---------------------------------------------------------------------------
// G product
// ---------------------------------------------------------------------------
// Work items: (row tile of 128 positions, K chunk) pairs q = tile + chunk *
// ntile; CTA b takes items b, b + gridDim.x, ...  With one CTA per item the
// grid is the item count; a persistent launch (GArgs.persist) keeps the
// resident CTAs (two per SM where the plan pairs) and lets each take items in
// turn, paying TMEM allocation, barrier and table set-up once.  The producer
// runs ahead into a CTA's next item while its decoder warps read the last
// item's accumulators; those warps then decode the next item, and their arrival
// on its first stage's dec barrier orders their TMEM reads before the MMA that
// overwrites the accumulators.  Every item accumulates the same MMAs, in the
// same order, from a zeroed accumulator, so its partial sums do not depend on
// the launch form.  acc_bar completes once per item (the commit after its last
// MMA); done_bar once, after the MMA thread's last MMA, before TMEM is freed.
template <int kMode>
__global__ void __launch_bounds__(kThreads, 2)
    k_tc_g(const __grid_constant__ CUtensorMap map_bed, const __grid_constant__ CUtensorMap map_w, GArgs a) {
  constexpr bool kDense = kMode == kModeDense, kFp8 = kMode == kModeGeno8;
  constexpr int kK = kFp8 ? 128 : kStepK;  // K elements (samples) per stage
  // A tile per stage: 128 SNP rows x kK samples, packed (kK/4 B per row) or
  // FP16 (128 B per row, 128-byte swizzle)
  constexpr int kTileBytes = kDense ? 128 * 128 : 128 * (kK / 4);
  constexpr bool kASmem = kDense;  // A operand in shared memory (else TMEM)
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  __shared__ uint64_t full_bar[kMaxStages], dec_bar[kMaxStages], empty_bar[kMaxStages], acc_bar, done_bar;
  __shared__ uint32_t tmem_sh;
  __shared__ volatile int abort_sh;
  __shared__ float unit[3 * 112];
  __shared__ uint32_t lut[kDense || kFp8 ? 1 : kLutWords];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int LP = a.LP, S = a.nslice;
  const SmemLayout lay = layout_for(LP, S, kTileBytes, kASmem);
  if (!kDense && !kFp8) lut_init(lut, tid, kThreads);
  const int ntile = (a.nsnp + 127) / 128;
  const int nitems = ntile * a.nchunks;
  // K steps of the item whose chunk starts at kbeg
  auto steps_of = [&](int kbeg) { return (min(kbeg + a.chunk, a.npad) - kbeg + kK - 1) / kK; };
  const int nst = a.nstages;
  const int ncat = S * LP;  // slices concatenated along N
  const long long wlim = a.wait_cycles > 0 ? a.wait_cycles : kTimeoutCycles;

  if (tid == 0) {
    abort_sh = 0;
    for (int s = 0; s < nst; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&dec_bar[s], kDecoders);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&acc_bar, 1);
    mbar_init(&done_bar, 1);
    fence_mbar_init();
  }
  if (kDense)
    for (int e = tid; e < S * LP; e += kThreads) unit[e] = (float)a.wscale[e];
  if (warp == 0) tmem_alloc(&tmem_sh, (uint32_t)a.tmem_cols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_sh;
  // TMEM columns: accumulators [0, ncat), then (A in TMEM) per stage the dosage
  // operand (32 columns = 64 BF16 K elements)
  const uint32_t a_col0 = (uint32_t)ncat;

  if (warp == 0) {
    // ---- TMA producer ----
    if (lane == 0) {
      const uint32_t tx_bytes = kTileBytes + (uint32_t)(ncat * 128);
      const int kdiv = kDense ? 0 : 2;  // inner TMA coordinate: samples, or packed bytes
      const int kofs = (int)a.kofs;
      int issued = 0, st = 0, round = 0;
      for (int q = blockIdx.x; q < nitems && !abort_sh; q += gridDim.x) {
        const int row0 = (q % ntile) * 128, kbeg = (q / ntile) * a.chunk;
        const int nk = steps_of(kbeg);
        const int prow = (int)(a.pos0 + row0);
        for (int kb = 0; kb < nk && kb < kPrefetchSteps; ++kb)
          tma_prefetch_2d(&map_bed, (kofs + kbeg + kb * kK) >> kdiv, prow);
        for (int kb = 0; kb < nk; ++kb) {
          const int k0 = kbeg + kb * kK;
          if (kb + kPrefetchSteps < nk) tma_prefetch_2d(&map_bed, (kofs + k0 + kPrefetchSteps * kK) >> kdiv, prow);
          if (round > 0 && !role_wait(&empty_bar[st], (uint32_t)(round - 1) & 1u, &abort_sh, wlim)) break;
          uint8_t* base = smem + st * lay.stage_bytes;
          mbar_expect_tx(&full_bar[st], tx_bytes);
          tma_load_2d(base + lay.p, &map_bed, (kofs + k0) >> kdiv, prow, &full_bar[st]);
          for (int s = 0; s < S; ++s) tma_load_2d(base + lay.b + s * LP * 128, &map_w, k0, s * LP, &full_bar[st]);
          ++issued;
          if (++st == nst) {
            st = 0;
            ++round;
          }
        }
      }
      if (abort_sh) drain_copies(full_bar, issued, nst);
    }
  } else if (warp == 1) {
    // ---- MMA issuer ----
    if (lane == 0) {
      const uint32_t id0 = idesc_of<kMode>(min(ncat, kMaxNTmemA));
      const uint32_t id1 = idesc_of<kMode>(ncat > kMaxNTmemA ? ncat - kMaxNTmemA : 16);
      const uint64_t b_desc0 = desc_sw128(smem_u32(smem + lay.b));
      const uint64_t a_desc0 = desc_sw128(smem_u32(smem + lay.a));
      const uint64_t stage_units = lay.stage_bytes >> 4;
      int st = 0, round = 0;
      bool ok = true;
      for (int q = blockIdx.x; q < nitems && ok; q += gridDim.x) {
        const int nk = steps_of((q / ntile) * a.chunk);
        for (int kb = 0; kb < nk; ++kb) {
          if (!role_wait(&dec_bar[st], (uint32_t)round & 1u, &abort_sh, wlim)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint64_t so = (uint64_t)st * stage_units;
          mma_stage<kMode, kASmem>(tmem, tmem + a_col0 + (uint32_t)st * 32u, a_desc0 + so, b_desc0 + so, ncat, id0,
                                   id1, kb == 0);
          mma_commit(&empty_bar[st]);
          if (++st == nst) {
            st = 0;
            ++round;
          }
        }
        if (ok) mma_commit(&acc_bar);  // the item's accumulators are complete
      }
      mma_commit(&done_bar);  // arrives once every MMA above has completed
    }
  } else if (warp >= kDecodeWarp0) {
    // ---- decoders: TMEM lane quarter q4 = warp % 4 (row r = SNP 32*q4 + lane of
    // the tile), K half ch: samples 32ch .. 32ch+31 of the step (8 packed bytes)
    // -> 16 columns of BF16 pairs into the stage's operand in TMEM (or, for
    // dense input, 32 FP16 values into the stage's A tile) ----
    const int q4 = warp & 3, ch = (warp - kDecodeWarp0) >> 2;
    const int r = q4 * 32 + lane;
    const uint32_t lane_off = (uint32_t)(q4 * 32) << 16;
    int st = 0, round = 0, li = 0;
    for (int q = blockIdx.x; q < nitems && !abort_sh; q += gridDim.x, ++li) {
      const int row0 = (q % ntile) * 128, chunk = q / ntile;
      const int nk = steps_of(chunk * a.chunk);
      for (int kb = 0; kb < nk; ++kb) {
        // the warp leaves together: the TMEM stores and loads below are warp-wide
        if (!__all_sync(0xffffffffu, role_wait(&full_bar[st], (uint32_t)round & 1u, &abort_sh, wlim))) break;
        uint8_t* base = smem + st * lay.stage_bytes;
        uint32_t wd[16];
        if (kDense) {
          // row r holds 8 chunks of 16 B (8 FP16 values each), chunk c stored at
          // position c ^ (r & 7) by the 128-byte swizzle; this thread takes
          // chunks 4ch .. 4ch+3 (samples 32ch .. 32ch+31)
#pragma unroll
          for (int qq = 0; qq < 4; ++qq) {
            const int cpos = (ch * 4 + qq) ^ (r & 7);
            const uint4 v = *reinterpret_cast<const uint4*>(base + lay.p + r * 128 + cpos * 16);
            wd[4 * qq] = v.x;
            wd[4 * qq + 1] = v.y;
            wd[4 * qq + 2] = v.z;
            wd[4 * qq + 3] = v.w;
          }
        } else if (kFp8) {
          // samples 64ch .. 64ch+63 of the step: 16 packed bytes, one per word
          const uint4 pk = *reinterpret_cast<const uint4*>(base + lay.p + r * 32 + ch * 16);
          e4m3_x16(pk.x, wd);
          e4m3_x16(pk.y, wd + 4);
          e4m3_x16(pk.z, wd + 8);
          e4m3_x16(pk.w, wd + 12);
        } else {
          const uint2 pk = *reinterpret_cast<const uint2*>(base + lay.p + r * 16 + ch * 8);
          const uint32_t* lut_l = lut + lane;
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const uint32_t w32 = e < 8 ? pk.x : pk.y;
            const int sh = 4 * (e & 7);
            wd[e] = lut_l[((w32 >> sh) & 15u) << 5];
          }
        }
        if constexpr (kASmem) {
          st_a_row(base + lay.a, r, ch, wd);
          fence_proxy_async_smem();
        } else {
          tmem_st16(tmem + lane_off + a_col0 + st * 32 + ch * 16, wd);
          tmem_wait_st();
          tc_fence_before();
        }
        mbar_arrive(&dec_bar[st]);
        if (++st == nst) {
          st = 0;
          ++round;
        }
      }
      // ---- epilogue of the item ----
      if (!__all_sync(0xffffffffu, !abort_sh && role_wait(&acc_bar, (uint32_t)li & 1u, &abort_sh, wlim))) break;
      tc_fence_after();
      const int quarter = warp & 3, chalf = (warp - kDecodeWarp0) >> 2;
      const int j = row0 + quarter * 32 + lane;
      const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
      const bool any = nk > 0;  // an item without K steps holds zeros
      for (int c0 = chalf * (LP / 2); c0 < (chalf + 1) * (LP / 2); c0 += 8) {
        if constexpr (kDense) {
          // FP16 values: slice sums times their power-of-two units (FP32 FMAs)
          float sum[8] = {0, 0, 0, 0, 0, 0, 0, 0};
          if (any) store_slice_sum(lane_base, c0, LP, S, unit, sum);
          if (j < a.nsnp) store_f32x8(reinterpret_cast<float*>(a.part) + ((size_t)chunk * a.nsnp + j) * LP + c0, sum);
        } else {
          // genotypes: every slice sum is an integer below 2^23, combined
          // exactly in int64 in units of the last slice
          const size_t off = ((size_t)chunk * a.nsnp + j) * LP + c0;
          if (S <= kIntSlices) {
            long long acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (any) combine_slices_exact(lane_base, c0, LP, S, acc, kFp8 ? kDigitBits8 : kDigitBits);
            if (j < a.nsnp) store_i64x8(reinterpret_cast<long long*>(a.part) + off, acc);
          } else {
            double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (any) combine_slices_fp64(lane_base, c0, LP, S, acc);
            if (j < a.nsnp) store_f64x8(reinterpret_cast<double*>(a.part) + off, acc);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && abort_sh) *a.err = 1;
  // the MMA thread's last commit may still be on its way after the last
  // epilogue (or an abort): wait for it (bounded) before freeing TMEM
  if (warp == 0) {
    if (lane == 0) mbar_wait(&done_bar, 0u);
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
  }
}

// ---------------------------------------------------------------------------
// H product
// ---------------------------------------------------------------------------
template <int kMode>
__global__ void __launch_bounds__(kThreads, 2)
    k_tc_h(const __grid_constant__ CUtensorMap map_bed, const __grid_constant__ CUtensorMap map_g, HArgs a) {
  constexpr bool kDense = kMode == kModeDense, kFp8 = kMode == kModeGeno8;
  constexpr int kK = kFp8 ? 128 : kStepK;  // K elements (SNPs) per stage
  // A tile per stage: kK SNP rows x 128 samples, packed (32 B per row) or FP16
  // (256 B per row, unswizzled)
  constexpr int kRowBytes = kDense ? 256 : 32;
  constexpr int kTileBytes = kK * kRowBytes;
  constexpr bool kASmem = kDense;  // A operand in shared memory (else TMEM)
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  __shared__ uint64_t full_bar[kMaxStages], dec_bar[kMaxStages], empty_bar[kMaxStages], acc_bar;
  __shared__ uint32_t tmem_sh;
  __shared__ volatile int abort_sh;
  __shared__ float unit[3 * 112];
  __shared__ uint32_t lut[kDense || kFp8 ? 1 : kLutWords];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (!kDense && !kFp8) lut_init(lut, tid, kThreads);
  const int LP = a.LP, S = a.nslice;
  const SmemLayout lay = layout_for(LP, S, kTileBytes, kASmem);
  const int samp0 = blockIdx.x * 128;
  const int jb = blockIdx.y * a.per_split;
  const int je = min(jb + a.per_split, a.nsnp);
  const int nk = je > jb ? (je - jb + kK - 1) / kK : 0;
  const int nst = a.nstages;
  const int ncat = S * LP;
  const long long wlim = a.wait_cycles > 0 ? a.wait_cycles : kTimeoutCycles;

  if (kDense)
    for (int e = tid; e < ncat; e += kThreads) unit[e] = (float)a.hscale[e];
  if (tid == 0) {
    abort_sh = 0;
    for (int s = 0; s < nst; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&dec_bar[s], kDecoders);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&acc_bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(&tmem_sh, (uint32_t)a.tmem_cols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_sh;
  // TMEM columns: accumulators [0, ncat), then (A in TMEM) per stage the dosage
  // operand (32 columns = 64 BF16 K elements)
  const uint32_t a_col0 = (uint32_t)ncat;

  if (warp == 0) {
    if (lane == 0) {
      const uint32_t tx_bytes = kTileBytes + (uint32_t)(ncat * 128);
      const int scol = kDense ? samp0 : (samp0 >> 2);  // inner TMA coordinate
      int issued = 0;
      for (int kb = 0; kb < nk && kb < kPrefetchSteps; ++kb)
        tma_prefetch_2d(&map_bed, scol, (int)(a.pos0 + jb + kb * kK));
      int st = 0, round = 0;
      for (int kb = 0; kb < nk; ++kb) {
        const int j0 = jb + kb * kK;
        if (kb + kPrefetchSteps < nk) tma_prefetch_2d(&map_bed, scol, (int)(a.pos0 + j0 + kPrefetchSteps * kK));
        if (round > 0 && !role_wait(&empty_bar[st], (uint32_t)(round - 1) & 1u, &abort_sh, wlim)) break;
        uint8_t* base = smem + st * lay.stage_bytes;
        mbar_expect_tx(&full_bar[st], tx_bytes);
        tma_load_2d(base + lay.p, &map_bed, scol, (int)(a.pos0 + j0), &full_bar[st]);
        for (int r = 0; r < S; ++r) tma_load_2d(base + lay.b + r * LP * 128, &map_g, j0, r * LP, &full_bar[st]);
        issued = kb + 1;
        if (++st == nst) {
          st = 0;
          ++round;
        }
      }
      if (abort_sh) drain_copies(full_bar, issued, nst);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t id0 = idesc_of<kMode>(min(ncat, kMaxNTmemA));
      const uint32_t id1 = idesc_of<kMode>(ncat > kMaxNTmemA ? ncat - kMaxNTmemA : 16);
      const uint64_t b_desc0 = desc_sw128(smem_u32(smem + lay.b));
      const uint64_t a_desc0 = desc_sw128(smem_u32(smem + lay.a));
      const uint64_t stage_units = lay.stage_bytes >> 4;
      int st = 0, round = 0;
      for (int kb = 0; kb < nk; ++kb) {
        if (!role_wait(&dec_bar[st], (uint32_t)round & 1u, &abort_sh, wlim)) break;
        tc_fence_after();
        const uint64_t so = (uint64_t)st * stage_units;
        mma_stage<kMode, kASmem>(tmem, tmem + a_col0 + (uint32_t)st * 32u, a_desc0 + so, b_desc0 + so, ncat, id0, id1,
                                 kb == 0);
        mma_commit(&empty_bar[st]);
        if (++st == nst) {
          st = 0;
          ++round;
        }
      }
      mma_commit(&acc_bar);
    }
  } else if (warp >= kDecodeWarp0) {
    // ---- decoders: TMEM lane quarter q4 (row r = sample 32*q4 + lane of the
    // tile), K half ch: SNPs 32ch .. 32ch+31 of the step, one packed byte each
    // (column r/4 of the SNP row) -> 16 columns of BF16 pairs in TMEM (or, for
    // dense input, 32 FP16 values into the stage's A tile) ----
    const int q4 = warp & 3, ch = (warp - kDecodeWarp0) >> 2;
    const int r = q4 * 32 + lane;
    const uint32_t lane_off = (uint32_t)(q4 * 32) << 16;
    int st = 0, round = 0;
    for (int kb = 0; kb < nk; ++kb) {
      // warp-uniform outcome: the genotype decode below shuffles across the warp
      if (!__all_sync(0xffffffffu, role_wait(&full_bar[st], (uint32_t)round & 1u, &abort_sh, wlim))) break;
      uint8_t* base = smem + st * lay.stage_bytes;
      uint32_t wd[16];
      if (kDense) {
        // value of SNP row j, sample r at j*256 + 2r: lanes read neighbouring
        // 2-byte values; two SNPs per 32-bit column
        const uint16_t* pt = reinterpret_cast<const uint16_t*>(smem + st * lay.stage_bytes + lay.p) + r;
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const uint32_t v0 = pt[(ch * 32 + 2 * e) * 128], v1 = pt[(ch * 32 + 2 * e + 1) * 128];
          wd[e] = v0 | (v1 << 16);
        }
      } else if (kFp8) {
        // SNP rows 64ch .. 64ch+63 of the step in two blocks of 32: lane l loads
        // row 64ch + 32t + l of the warp's 32 samples; after the transpose lane
        // r holds sample r's 32 codes, byte q of lo / hi = rows 4q .. 4q+3 /
        // 16+4q .. 16+4q+3, one E4M3 word each
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          const uint2 rowv = *reinterpret_cast<const uint2*>(base + lay.p + (ch * 64 + t * 32 + lane) * 32 + q4 * 8);
          uint32_t lo = rowv.x, hi = rowv.y;
          xpose2_warp(lo, hi, lane);
          e4m3_x16(lo, wd + 8 * t);
          e4m3_x16(hi, wd + 8 * t + 4);
        }
      } else {
        // lane l loads SNP row 32ch + l of the warp's 32 samples (8 bytes); the
        // warp transpose leaves lane r with sample r's codes of those 32 rows,
        // row j in bits 2j .. 2j+1 (lo: rows 0-15, hi: rows 16-31)
        const uint2 rowv = *reinterpret_cast<const uint2*>(base + lay.p + (ch * 32 + lane) * 32 + q4 * 8);
        uint32_t lo = rowv.x, hi = rowv.y;
        xpose2_warp(lo, hi, lane);
        const uint32_t* lut_l = lut + lane;
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const uint32_t w32 = e < 8 ? lo : hi;
          wd[e] = lut_l[((w32 >> (4 * (e & 7))) & 15u) << 5];
        }
      }
      if constexpr (kASmem) {
        st_a_row(base + lay.a, r, ch, wd);
        fence_proxy_async_smem();
      } else {
        tmem_st16(tmem + lane_off + a_col0 + st * 32 + ch * 16, wd);
        tmem_wait_st();
        tc_fence_before();
      }
      mbar_arrive(&dec_bar[st]);
      if (++st == nst) {
        st = 0;
        ++round;
      }
    }
    const bool ok = nk > 0 && role_wait(&acc_bar, 0u, &abort_sh, wlim);
    tc_fence_after();
    const int quarter = warp & 3, chalf = (warp - kDecodeWarp0) >> 2;
    const int i = samp0 + quarter * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
    if (!abort_sh) {
      for (int c0 = chalf * (LP / 2); c0 < (chalf + 1) * (LP / 2); c0 += 8) {
        const size_t row = (size_t)blockIdx.y * a.npad + i;
        if constexpr (kDense) {
          float sum[8] = {0, 0, 0, 0, 0, 0, 0, 0};
          if (ok) store_slice_sum(lane_base, c0, LP, S, unit, sum);
          store_f32x8(reinterpret_cast<float*>(a.hpart) + row * LP + c0, sum);
        } else {
          if (S <= kIntSlices) {
            long long acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (ok) combine_slices_exact(lane_base, c0, LP, S, acc, kFp8 ? kDigitBits8 : kDigitBits);
            store_i64x8(reinterpret_cast<long long*>(a.hpart) + row * LP + c0, acc);
          } else {
            double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (ok) combine_slices_fp64(lane_base, c0, LP, S, acc);
            store_f64x8(reinterpret_cast<double*>(a.hpart) + row * LP + c0, acc);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && abort_sh) *a.err = 1;
  cta_release(acc_bar, abort_sh, warp, lane, tmem, (uint32_t)a.tmem_cols);
}

// ---------------------------------------------------------------------------
// FP64 epilogues and operand preparation
// ---------------------------------------------------------------------------

// Column reductions of a row-major FP64 matrix (rows x LP): the maximum of
// |A| (kMax; the result is the exponent E_l with max_r |A_rl| < 2^E_l) or the
// sum.  Block b reduces rows [b*per, (b+1)*per) with coalesced loads (thread t
// keeps column t % LP) and writes one partial per column; the last block to
// finish combines the partials in block order, so the result does not depend
// on the order in which blocks run.  cnt is zero on entry and again on exit.
template <bool kMax>
__global__ void __launch_bounds__(256) k_colred(const double* __restrict__ A, int64_t rows, int LP, int64_t per,
                                               double* __restrict__ part, unsigned* __restrict__ cnt,
                                               double* __restrict__ sum_out, int* __restrict__ exp_out) {
  __shared__ double red[256];
  __shared__ bool last;
  const int tid = threadIdx.x;
  const int step = (256 / LP) * LP;
  const int64_t r0 = (int64_t)blockIdx.x * per;
  const int64_t r1 = r0 + per < rows ? r0 + per : rows;
  double v = 0.0;
  if (tid < step) {
    const int64_t f1 = r1 * LP;
    for (int64_t f = r0 * LP + tid; f < f1; f += step) {
      const double x = A[f];
      v = kMax ? fmax(v, fabs(x)) : v + x;
    }
  }
  red[tid] = v;
  __syncthreads();
  if (tid < LP) {
    double t = red[tid];
    for (int q = tid + LP; q < step; q += LP) t = kMax ? fmax(t, red[q]) : t + red[q];
    part[(size_t)blockIdx.x * LP + tid] = t;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) last = atomicAdd(cnt, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  // one warp per column: the lanes combine blocks lane, lane+32, ..., then a
  // butterfly (a fixed order)
  const int warp = tid >> 5, lane = tid & 31;
  for (int l = warp; l < LP; l += 8) {
    double t = 0.0;
    for (unsigned b = lane; b < gridDim.x; b += 32) {
      const double x = __ldcg(part + (size_t)b * LP + l);
      t = kMax ? fmax(t, x) : t + x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_xor_sync(0xffffffffu, t, o);
      t = kMax ? fmax(t, y) : t + y;
    }
    if (lane == 0) {
      if (kMax) {
        int e = 0;
        if (t > 0.0) frexp(t, &e);  // t = m * 2^e, 0.5 <= m < 1, so |A| < 2^e
        exp_out[l] = e;
      } else {
        sum_out[l] = t;
      }
    }
  }
  if (tid == 0) *cnt = 0u;
}

// Split v (|v| < 2^E) into S integer slices of db-bit digits: m = rint(v *
// 2^(db*S-1-E)) has |m| <= 2^(db*S-1) (at most 2^53: exact in FP64), and its
// balanced base-2^db digits w_s (m = sum_s w_s 2^(db(S-1-s)), |w_s| <= 2^(db-1))
// are the slices, with units u_s = 2^(E-(db-1)-db*s).  Returns the represented
// value m * u_(S-1).  Integer digit arithmetic keeps the FP64 work to one
// multiply and one conversion.  The digits are stored in the operand format:
// BF16 or FP16 (db = 9, |w| <= 256) or E4M3 (db = 4, |w| <= 8), exact in each.
// *m_out (optional) receives the integer the sparse terms use: m itself for
// S <= kIntSlices, else the rounding of v to kIntSlices slices (27 bits; unit
// u_(kIntSlices-1)).
__device__ __forceinline__ void put_digit(uint16_t* dst, int w, int fmt) {
  *dst = fmt == kFmtF16 ? __half_as_ushort(__int2half_rn(w)) : __bfloat16_as_ushort(__float2bfloat16_rn((float)w));
}
__device__ __forceinline__ void put_digit(uint8_t* dst, int w, int) {
  *dst = (uint8_t)__nv_cvt_float_to_fp8((float)w, __NV_SATFINITE, __NV_E4M3);
}
template <class D>
__device__ __forceinline__ double split_store(double v, int E, int S, int db, D* dst, size_t slice_stride, int fmt,
                                              int* m_out = nullptr) {
  const long long kBase = 1ll << db, kHalf = kBase / 2;
  const long long m = __double2ll_rn(v * exp2i(db * S - 1 - E));
  if (m_out) *m_out = S <= kIntSlices ? (int)m : __double2int_rn(v * exp2i(db * kIntSlices - 1 - E));
  long long rest = m;
  for (int s = S - 1; s > 0; --s) {
    const long long w = ((rest + kHalf) & (kBase - 1)) - kHalf;
    put_digit(dst + (size_t)s * slice_stride, (int)w, fmt);
    rest = (rest - w) / kBase;  // exact: rest - w is a multiple of the base
  }
  put_digit(dst, (int)rest, fmt);
  return (double)m * exp2i(E - db * S + 1);
}

// W slices of Omega (S*LP rows x npad, K-major) and the represented W, in FP64
// and as the integer of the sparse terms (|m| <= 2^26, see split_store).
// A block takes 32 rows of Omega (coalesced reads, and coalesced writes of the
// represented values), keeps their digits in shared memory and writes each
// slice row's 32 digits as one 64-byte run.  npad is a multiple of 32.
constexpr int kOmgRows = 32;
template <class D>
__global__ void __launch_bounds__(256) k_omega_slices(const double* __restrict__ omg, int npad, int N, int LP, int S,
                                                      int db, const int* __restrict__ E, D* __restrict__ w,
                                                      double* __restrict__ rep, int32_t* __restrict__ wint, int fmt) {
  __shared__ D dg[kMaxSlices * 112 * kOmgRows];  // [s][l][row]
  const int i0 = blockIdx.x * kOmgRows;
  for (int e = threadIdx.x; e < kOmgRows * LP; e += blockDim.x) {
    const int il = e / LP, l = e % LP;
    const int i = i0 + il;
    const size_t idx = (size_t)i * LP + l;
    const double v = i < N ? omg[idx] : 0.0;
    int m = 0;
    const double r = split_store(v, E[l], S, db, dg + l * kOmgRows + il, (size_t)LP * kOmgRows, fmt, &m);
    rep[idx] = r;
    wint[idx] = m;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < S * LP * kOmgRows; e += blockDim.x) {
    const int row = e / kOmgRows, il = e % kOmgRows;  // row = s * LP + l
    w[(size_t)row * npad + i0 + il] = dg[e];
  }
}

__global__ void k_units(const int* __restrict__ E, int LP, int S, int db, int eoff, double* __restrict__ unit) {
  const int idx = threadIdx.x + blockIdx.x * blockDim.x;
  if (idx >= S * LP) return;
  const int s = idx / LP, l = idx % LP;
  unit[idx] = ldexp(1.0, E[l] + eoff - (db - 1) - db * s);
}

// G rows of the window: FP64 sum of the chunk partials, the centring term, and
// the missing-entry term
//   sum_{i missing} (f + e_i) W_i = f u_l sum_i m_il + 2^-16 u_l sum_i q(e_i m_il)
// from the exact integer sums of the represented W (W_il = m_il u_l) gathered
// by k_seg_gather (gisum, and gesum with EM fill values), which are read and
// cleared here; then Gh = 1/2 s G (FP64) for the H operand.
__global__ void k_tc_g_finish(GFinishArgs a) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)a.nsnp * a.LP) return;
  const int j = (int)(idx / a.LP), l = (int)(idx % a.LP);
  const int LP = a.LP;
  double gh = 0.0;
  if (l < a.L) {
    const int64_t pos = a.pos0 + j;
    const int64_t snp = a.perm ? (int64_t)a.perm[pos] : pos;
    const double f = a.F[snp], s = a.scale[snp];
    double pd;
    if (a.vfac == 1.0) {
      // dense input: FP32 chunk partials summed as an FP32 pair (TwoSum, about
      // 48 bits: far below the FP32 rounding of each partial)
      const float* part = reinterpret_cast<const float*>(a.part);
      float ph = 0.f, pl = 0.f;
      for (int c = 0; c < a.nchunks; ++c) {
        const float v = part[((size_t)c * a.nsnp + j) * LP + l];
        const float t = __fadd_rn(ph, v);
        const float bv = __fsub_rn(t, ph);
        pl = __fadd_rn(pl, __fadd_rn(__fsub_rn(ph, __fsub_rn(t, bv)), __fsub_rn(v, bv)));
        ph = t;
      }
      pd = (double)ph + (double)pl;
    } else if (a.nslice <= kIntSlices) {
      // genotypes: exact int64 sum of the chunks' slice combinations (below
      // 2^53), one conversion, scaled by the last slice unit (a power of two)
      const long long* part = reinterpret_cast<const long long*>(a.part);
      long long ps = 0;
      for (int c = 0; c < a.nchunks; ++c) ps += part[((size_t)c * a.nsnp + j) * LP + l];
      pd = (double)ps * a.wunit_p[l];
    } else {
      // the 54-bit form: FP64 chunk sums
      const double* part = reinterpret_cast<const double*>(a.part);
      double ps = 0.0;
      for (int c = 0; c < a.nchunks; ++c) ps += part[((size_t)c * a.nsnp + j) * LP + l];
      pd = ps * a.wunit_p[l];
    }
    double miss = 0.0;
    if (a.gisum) {
      miss = f * a.wunit_m[l] * (double)(long long)a.gisum[idx];
      a.gisum[idx] = 0ull;
      if (a.gesum) {
        miss += exp2i(-24 + kSegValueShift) * a.wunit_m[l] * (double)(long long)a.gesum[idx];
        a.gesum[idx] = 0ull;
      }
    }
    const double g = s * (a.vfac * pd - f * a.colsum[l] + miss);
    a.G[pos * LP + l] = g;
    gh = a.vfac * s * g;
  }
  a.gh[idx] = gh;
}

// Gh slices (columns nsnp .. ldg-1 zeroed) with per-column exponents Eh, the
// represented Gh as integers (ghint, for the EM term of H), and Gm = 2 f Gh
// represented as an integer per entry (exponent Eh + 1: |Gm| <= 2 |Gh|; the
// value is gmint * u'_l, u'_l the unit of slice min(S, kIntSlices) - 1)
// together with its terms of c = sum_j Gm_j, so that the centring and
// missing-entry terms of H use the same represented Gm.  With more than
// kIntSlices slices (the 54-bit form) c takes 2 f Gh at full precision
// instead, and only the missing entries use the 27-bit Gm.
template <class D>
__global__ void k_tc_gh_slices(GFinishArgs a, const int* __restrict__ Eh) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)a.ldg * a.LP) return;
  const int j = (int)(idx / a.LP), l = (int)(idx % a.LP);
  const int S = a.nslice, LP = a.LP;
  const size_t sstride = (size_t)LP * a.ldg;
  D* dh = reinterpret_cast<D*>(a.gt) + (size_t)l * a.ldg + j;
  const bool f16 = a.vfac == 1.0;  // dense input: FP16 operands
  const int db = a.digit_bits;
  if (j < a.nsnp && l < a.L) {
    const int64_t pos = a.pos0 + j;
    const int64_t snp = a.perm ? (int64_t)a.perm[pos] : pos;
    int mh = 0;
    const double ghq = split_store(a.gh[(size_t)j * LP + l], Eh[l], S, db, dh, sstride, a.fmt, &mh);
    a.ghint[(size_t)j * LP + l] = mh;
    if (f16) {
      // dense: c = sum_j mu_j Gh_j (no missing entries)
      a.gmint[(size_t)j * LP + l] = 0;
      a.cpart[(size_t)j * LP + l] = a.F[snp] * ghq;
    } else {
      const int e = Eh[l] + 1, Si = min(S, kIntSlices);
      const double gm = 2.0 * a.F[snp] * ghq;
      const int m = __double2int_rn(gm * exp2i(db * Si - 1 - e));
      a.gmint[(size_t)j * LP + l] = m;
      a.cpart[(size_t)j * LP + l] = S > kIntSlices ? gm : (double)m * exp2i(e - db * Si + 1);
    }
  } else {
    for (int s = 0; s < S; ++s) dh[s * sstride] = 0;
    if (j < a.nsnp) {
      a.ghint[(size_t)j * LP + l] = 0;
      a.gmint[(size_t)j * LP + l] = 0;
      a.cpart[(size_t)j * LP + l] = 0.0;
    }
  }
}

// H rows: the split partials, the missing-entry terms and the centring term.
// Genotypes: the dosage part P (units u = the last Gh slice unit), the Gm sums
// (units 2u) and the EM products (units 2^-15 u) are combined exactly in int64
// in units of 2^-15 u (below 2^56 in magnitude), converted once and scaled;
// the int64 missing-entry sums are cleared for the next window.  Dense input:
// FP64 sum of the FP32 split partials.
__global__ void k_tc_h_finish(HFinishArgs a) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int LP = a.LP;
  if (idx >= (int64_t)a.nsamples * LP) return;
  const int64_t i = idx / LP;
  const int l = (int)(idx - i * LP);
  if (l >= a.L) return;
  double h;
  if (a.dense) {
    const float* hp = reinterpret_cast<const float*>(a.hpart);
    h = 0.0;
    for (int s = 0; s < a.nsplit; ++s) h += (double)hp[((size_t)s * a.npad + i) * LP + l];
  } else if (a.nslice <= kIntSlices) {
    const long long* hp = reinterpret_cast<const long long*>(a.hpart);
    long long t = 0;
    for (int s = 0; s < a.nsplit; ++s) t += hp[((size_t)s * a.npad + i) * LP + l];
    t *= 32768;
    if (a.hisum) {
      t += (long long)a.hisum[idx] * 65536;
      a.hisum[idx] = 0ull;
      if (a.hesum) {
        t += (long long)a.hesum[idx];
        a.hesum[idx] = 0ull;
      }
    }
    h = (double)t * (a.hunit_m[l] * (1.0 / 32768.0));
  } else {
    // the 54-bit form: FP64 split sums (units of the last slice) and the
    // missing-entry sums of the 27-bit integers
    const double* hp = reinterpret_cast<const double*>(a.hpart);
    double t = 0.0;
    for (int s = 0; s < a.nsplit; ++s) t += hp[((size_t)s * a.npad + i) * LP + l];
    h = t * a.hunit_p[l];
    if (a.hisum) {
      double m = (double)(long long)a.hisum[idx] * 65536.0;
      a.hisum[idx] = 0ull;
      if (a.hesum) {
        m += (double)(long long)a.hesum[idx];
        a.hesum[idx] = 0ull;
      }
      h += m * (a.hunit_m[l] * (1.0 / 32768.0));
    }
  }
  a.Hx[idx] += h - a.c[l];
}

__global__ void k_gather_rows(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, int64_t stride,
                              const int32_t* __restrict__ perm, int64_t nrows) {
  const int64_t r = blockIdx.x;
  if (r >= nrows) return;
  const uint4* s = reinterpret_cast<const uint4*>(src + (int64_t)perm[r] * stride);
  uint4* d = reinterpret_cast<uint4*>(dst + r * stride);
  for (int64_t q = threadIdx.x; q < stride / 16; q += blockDim.x) d[q] = s[q];
}

// Sample-major copy of the packed rows (launch_transpose_codes): sample row i,
// block w holds the codes of window w's positions w*ws + j (j < ldw, four per
// byte, position j in bits 2(j%4) of byte j/4), as a .bed would with samples
// and SNPs swapped, so that an H tile (128 samples x 128 positions) is read and
// decoded like a G tile.  Positions past the window or the matrix hold code
// 00 (their Gh rows are zero).  A CTA iteration reads a 128-position x
// 256-sample tile (64-byte row pieces in 16-byte loads), then
// warp v transposes the 32-sample block v in four 32 x 32 code blocks with
// the shuffle transpose of the H decoder and writes each of its samples' 128
// positions as one 32-byte piece.
constexpr int kXposeSamples = 256;
__global__ void __launch_bounds__(256) k_transpose_codes(const uint8_t* __restrict__ bed, int64_t stride, int64_t M,
                                                         int64_t ws, int64_t ldw, int npad, uint8_t* __restrict__ bt,
                                                         int64_t tpitch) {
  __shared__ __align__(16) uint8_t tile[128][kXposeSamples / 4];  // positions x packed samples
  const int jt = blockIdx.x, w = blockIdx.z;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t p0 = (int64_t)w * ws + (int64_t)jt * 128;
  const int64_t jlim = min((int64_t)128, min(ws - (int64_t)jt * 128, M - p0));  // positions of this tile
  const int nbytes = npad / 4;
  for (int b0 = blockIdx.y * (kXposeSamples / 4); b0 < nbytes; b0 += gridDim.y * (kXposeSamples / 4)) {
    const int cb = min(kXposeSamples / 4, nbytes - b0);  // packed bytes of this tile (a multiple of 32)
    __syncthreads();
    // 128 rows x 64 bytes: four 16-byte pieces per row, 512 pieces over 256 threads
    for (int e = tid; e < 128 * 4; e += blockDim.x) {
      const int j = e >> 2, q = e & 3;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (j < jlim && q * 16 < cb) v = *reinterpret_cast<const uint4*>(bed + (p0 + j) * stride + b0 + q * 16);
      *reinterpret_cast<uint4*>(&tile[j][q * 16]) = v;
    }
    __syncthreads();
    // warp v: samples 32v .. 32v+31 of the tile (packed bytes 8v .. 8v+7)
    if (warp * 8 < cb) {
      uint32_t out[8];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const uint2 r = *reinterpret_cast<const uint2*>(&tile[32 * t + lane][8 * warp]);
        uint32_t lo = r.x, hi = r.y;
        xpose2_warp(lo, hi, lane);  // lane = sample; lo / hi = positions 32t .. +15 / +16 .. +31
        out[2 * t] = lo;
        out[2 * t + 1] = hi;
      }
      const int64_t row = (int64_t)b0 * 4 + 32 * warp + lane;
      uint4* dst = reinterpret_cast<uint4*>(bt + row * tpitch + (int64_t)w * (ldw >> 2) + jt * 32);
      dst[0] = make_uint4(out[0], out[1], out[2], out[3]);
      dst[1] = make_uint4(out[4], out[5], out[6], out[7]);
    }
  }
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

void make_map_2d(CUtensorMap* map, const void* base, int dtype, uint64_t inner, uint64_t outer, uint64_t pitch_bytes,
                 uint32_t box_inner, uint32_t box_outer, bool swizzle128) {
  const cuuint64_t dims[2] = {inner, outer};
  const cuuint64_t strides[1] = {pitch_bytes};
  const cuuint32_t box[2] = {box_inner, box_outer};
  const cuuint32_t es[2] = {1, 1};
  const CUtensorMapDataType t = dtype == kMapBF16   ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                : dtype == kMapF16  ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                    : CU_TENSOR_MAP_DATA_TYPE_UINT8;
  const CUresult r = encode_fn()(map, t, 2,
                                 const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(-2, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

// Genotype input (A in TMEM): two CTAs per SM when the slice accumulators
// leave room for two 32-column operand stages within half of the SM's 512
// TMEM columns.  The tensor core then runs one CTA's MMAs while the other
// decodes and stores its next operand into TMEM; on the 7,812 x 100,000
// genotype window this cut both products by a third against one CTA per SM
// with eight stages.  Dense input (A in shared memory): one CTA per SM.
bool pair_per_sm(int LP, int nslice, bool dense) { return !dense && nslice * LP + 2 * 32 <= 256; }

int cta_slots(int LP, int nslice, bool dense) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    PCAONE_CUDA(cudaGetDevice(&dev));
    PCAONE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  return sms * (pair_per_sm(LP, nslice, dense) ? 2 : 1);
}

// A CTA's fixed cost (TMEM allocation, barrier and table set-up, pipeline
// fill, epilogue) in K elements: about the time of 12 pipeline steps of 64.
constexpr int kCtaCostK = 768;

int k_parts(int tiles, int K, int kmax, int slots) {
  if (K <= 0) return 1;
  const int lo = std::max(1, ceil_div(K, kmax));
  const int hi = std::max(lo, std::min(ceil_div(K, 1024), lo + 128));
  int best = lo;
  double best_cost = 1e300;
  for (int p = lo; p <= hi; ++p) {
    const int kp = round_up(ceil_div(K, p), 64);
    const int parts = ceil_div(K, kp);
    const int64_t ctas = (int64_t)tiles * parts;
    const int64_t waves = (ctas + slots - 1) / slots;
    const double cost = (double)waves * (kp + kCtaCostK);
    if (cost < best_cost * 0.999) {
      best_cost = cost;
      best = parts;
    }
  }
  return best;
}

int stages_for(int LP, int nslice, int pbytes, bool dense) {
  const SmemLayout l = layout_for(LP, nslice, pbytes, dense);
  const bool pair = pair_per_sm(LP, nslice, dense);
  // dynamic shared memory (static use is under 12 KB); 228 KB per SM
  const int budget = (pair ? 104 : 212) * 1024;
  const int by_smem = budget / (int)l.stage_bytes;
  // TMEM: slice accumulators + (A in TMEM) 32 columns of A operand per stage
  const int by_tmem = dense ? kMaxStages : ((pair ? 256 : 512) - nslice * LP) / 32;
  return std::max(1, std::min(kMaxStages, std::min(by_smem, by_tmem)));
}

int tmem_cols_needed(int LP, int nslice, int nstages, bool dense) { return nslice * LP + (dense ? 0 : nstages * 32); }

// A plan that takes more than half of the TMEM, or that does not pair, asks
// for more than half of the shared memory too, so that a second CTA never
// shares its SM and waits in tcgen05.alloc.
size_t smem_bytes(int LP, int nslice, int pbytes, int nstages, int tmem_cols, bool dense) {
  const size_t b = (size_t)layout_for(LP, nslice, pbytes, dense).stage_bytes * nstages + 1024;
  const bool pair = tmem_cols <= 256 && pair_per_sm(LP, nslice, dense);
  return pair ? b : std::max(b, (size_t)120 * 1024);
}

int tmem_cols_for(int ncols) {
  int c = 32;
  while (c < ncols) c <<= 1;
  return c;
}

template <int kMode>
void launch_g_t(const CUtensorMap& map_bed, const CUtensorMap& map_w, const GArgs& a, size_t smem, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    PCAONE_CUDA(cudaFuncSetAttribute(k_tc_g<kMode>, cudaFuncAttributeMaxDynamicSharedMemorySize, 214 * 1024));
    attr = true;
  }
  const int nitems = (a.nsnp + 127) / 128 * a.nchunks;
  const int grid = a.persist ? std::min(nitems, cta_slots(a.LP, a.nslice, a.dense != 0)) : nitems;
  k_tc_g<kMode><<<std::max(grid, 1), kThreads, smem, s>>>(map_bed, map_w, a);
}

template <int kMode>
void launch_h_t(const CUtensorMap& map_bed, const CUtensorMap& map_g, const HArgs& a, size_t smem, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    PCAONE_CUDA(cudaFuncSetAttribute(k_tc_h<kMode>, cudaFuncAttributeMaxDynamicSharedMemorySize, 214 * 1024));
    attr = true;
  }
  dim3 grid(a.npad / 128, a.nsplit);
  k_tc_h<kMode><<<grid, kThreads, smem, s>>>(map_bed, map_g, a);
}

void launch_g(const CUtensorMap& map_bed, const CUtensorMap& map_w, const GArgs& a, cudaStream_t s) {
  if (a.nstages < 1 || a.nstages > kMaxStages || a.tmem_cols > 512 ||
      a.tmem_cols < tmem_cols_needed(a.LP, a.nslice, a.nstages, a.dense != 0))
    throw Error(-6, "tensor-core G product: pipeline plan exceeds TMEM or the stage limit");
  const size_t smem =
      smem_bytes(a.LP, a.nslice, g_tile_bytes(a.dense != 0, a.fp8 != 0), a.nstages, a.tmem_cols, a.dense != 0);
  if (smem > 214 * 1024) throw Error(-6, "tensor-core G product: pipeline plan exceeds shared memory");
  if (a.dense && a.fp8) throw Error(-1, "tensor-core G product: no E4M3 form for dense input");
  if (a.fp8 && a.chunk % 128 != 0) throw Error(-1, "tensor-core G product: E4M3 chunks must hold whole 128-sample stages");
  if (a.dense)
    launch_g_t<kModeDense>(map_bed, map_w, a, smem, s);
  else if (a.fp8)
    launch_g_t<kModeGeno8>(map_bed, map_w, a, smem, s);
  else
    launch_g_t<kModeGeno>(map_bed, map_w, a, smem, s);
  PCAONE_LAUNCH_CHECK();
}

void launch_h(const CUtensorMap& map_bed, const CUtensorMap& map_g, const HArgs& a, cudaStream_t s) {
  if (a.nstages < 1 || a.nstages > kMaxStages || a.tmem_cols > 512 ||
      a.tmem_cols < tmem_cols_needed(a.LP, a.nslice, a.nstages, a.dense != 0))
    throw Error(-6, "tensor-core H product: pipeline plan exceeds TMEM or the stage limit");
  const size_t smem =
      smem_bytes(a.LP, a.nslice, h_tile_bytes(a.dense != 0, a.fp8 != 0), a.nstages, a.tmem_cols, a.dense != 0);
  if (smem > 214 * 1024) throw Error(-6, "tensor-core H product: pipeline plan exceeds shared memory");
  if (a.dense && a.fp8) throw Error(-1, "tensor-core H product: no E4M3 form for dense input");
  if (a.fp8 && a.per_split % 128 != 0)
    throw Error(-1, "tensor-core H product: E4M3 splits must hold whole 128-SNP stages");
  if (a.dense)
    launch_h_t<kModeDense>(map_bed, map_g, a, smem, s);
  else if (a.fp8)
    launch_h_t<kModeGeno8>(map_bed, map_g, a, smem, s);
  else
    launch_h_t<kModeGeno>(map_bed, map_g, a, smem, s);
  PCAONE_LAUNCH_CHECK();
}

template <bool kMax>
void launch_colred(const double* A, int64_t rows, int LP, const ColRedScratch& cr, double* sum_out, int* exp_out,
                   cudaStream_t s) {
  if (LP < 1 || LP > 256) throw Error(-6, "column reduction: row width out of range");
  if (rows <= 0) {
    // an empty column has sum 0 and exponent 0
    if (kMax)
      PCAONE_CUDA(cudaMemsetAsync(exp_out, 0, sizeof(int) * LP, s));
    else
      PCAONE_CUDA(cudaMemsetAsync(sum_out, 0, sizeof(double) * LP, s));
    return;
  }
  const int64_t nb0 = std::min<int64_t>(kColRedBlocks, (rows + 31) / 32);
  const int64_t per = (rows + nb0 - 1) / nb0;
  const int nb = (int)((rows + per - 1) / per);
  k_colred<kMax><<<nb, 256, 0, s>>>(A, rows, LP, per, cr.part, cr.cnt, sum_out, exp_out);
  PCAONE_LAUNCH_CHECK();
}

void launch_omega_slices(const double* omg, int npad, int N, int LP, int S, void* w, double* wunit,
                         double* colsum, int* E, double* rep, int32_t* wint, int fmt, const ColRedScratch& cr,
                         cudaStream_t s) {
  launch_colred<true>(omg, N, LP, cr, nullptr, E, s);
  if (npad % kOmgRows != 0 || S > kMaxSlices || LP > 112) throw Error(-6, "test-matrix slices: unsupported shape");
  const int db = digit_bits_of(fmt);
  if (fmt == kFmtE4M3)
    k_omega_slices<uint8_t><<<npad / kOmgRows, 256, 0, s>>>(omg, npad, N, LP, S, db, E, reinterpret_cast<uint8_t*>(w),
                                                           rep, wint, fmt);
  else
    k_omega_slices<uint16_t><<<npad / kOmgRows, 256, 0, s>>>(omg, npad, N, LP, S, db, E,
                                                            reinterpret_cast<uint16_t*>(w), rep, wint, fmt);
  PCAONE_LAUNCH_CHECK();
  k_units<<<ceil_div(S * LP, 128), 128, 0, s>>>(E, LP, S, db, 0, wunit);
  PCAONE_LAUNCH_CHECK();
  launch_colred<false>(rep, N, LP, cr, colsum, nullptr, s);
}

void launch_g_finish(const GFinishArgs& a, int* Eh, double* hunit, double* gmunit, double* c_out,
                     const ColRedScratch& cr, cudaStream_t s) {
  k_tc_g_finish<<<ceil_div((int64_t)a.nsnp * a.LP, 256), 256, 0, s>>>(a);
  PCAONE_LAUNCH_CHECK();
  launch_colred<true>(a.gh, a.nsnp, a.LP, cr, nullptr, Eh, s);
  if (a.fmt == kFmtE4M3)
    k_tc_gh_slices<uint8_t><<<ceil_div((int64_t)a.ldg * a.LP, 256), 256, 0, s>>>(a, Eh);
  else
    k_tc_gh_slices<uint16_t><<<ceil_div((int64_t)a.ldg * a.LP, 256), 256, 0, s>>>(a, Eh);
  PCAONE_LAUNCH_CHECK();
  k_units<<<ceil_div(a.nslice * a.LP, 128), 128, 0, s>>>(Eh, a.LP, a.nslice, a.digit_bits, 0, hunit);
  PCAONE_LAUNCH_CHECK();
  k_units<<<ceil_div(a.nslice * a.LP, 128), 128, 0, s>>>(Eh, a.LP, a.nslice, a.digit_bits, 1, gmunit);
  PCAONE_LAUNCH_CHECK();
  launch_colred<false>(a.cpart, a.nsnp, a.LP, cr, c_out, nullptr, s);
}

void launch_h_finish(const HFinishArgs& a, cudaStream_t s) {
  const int64_t n = (int64_t)a.nsamples * a.LP;
  k_tc_h_finish<<<ceil_div(n, 256), 256, 0, s>>>(a);
  PCAONE_LAUNCH_CHECK();
}

void launch_transpose_codes(const uint8_t* bed, int64_t stride, int64_t M, int64_t ws, int64_t ldw, int nwin,
                            int npad, uint8_t* bt, int64_t tpitch, cudaStream_t s) {
  if (M == 0 || nwin == 0) return;
  if (ldw % 128 != 0 || ldw < ws || npad % 128 != 0 || (int64_t)npad / 4 > stride || tpitch < nwin * (ldw / 4))
    throw Error(-1, "internal: sample-major copy layout");
  if (stride % 16 != 0 || tpitch % 16 != 0 || ((uintptr_t)bed & 15u) != 0 || ((uintptr_t)bt & 15u) != 0)
    throw Error(-1, "internal: sample-major copy alignment");
  const int ytiles = std::max(1, std::min(ceil_div(npad, kXposeSamples), 4));
  dim3 grid((unsigned)(ldw / 128), (unsigned)ytiles, (unsigned)nwin);
  k_transpose_codes<<<grid, 256, 0, s>>>(bed, stride, M, ws, ldw, npad, bt, tpitch);
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
