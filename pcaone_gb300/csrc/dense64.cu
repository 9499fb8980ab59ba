// Dense kernels of the RSVD driver: tall-skinny Gram / cross products,
// Cholesky and triangular inverse of (k+p)^2 matrices, tall x small products,
// the Householder sign rule, flipOmg, the Jacobi eigensolver for the small
// SVD of B, mev, the EM fill and the Arnoldi matvec.
//
// All matrices are stored in FP64.  FP64 arithmetic runs at a small fraction
// of the FP32 rate on this GPU, so the two O(rows * L^2) kernels (the Gram /
// cross product and the tall x small product) compute in FP32 pairs
// (double-float: error-free TwoProduct / TwoSum, about 44 significand bits),
// which is far below the 24-bit integer slices the window products use.  The
// (k+p)^2 Cholesky and inverse are latency-bound chains of square roots and
// reciprocals and run in double-float too (dd.cuh); the Jacobi eigensolver,
// the Householder sign rule and the small products stay in FP64.  The
// FP64-grade form (the GPU oracle) runs these four kernels in plain FP64
// arithmetic instead (template flag F64; the same shared-memory bytes hold one
// double where the FP32-pair form keeps a float pair).
//
// Tall matrices (N x L, M x L) are row-major with leading dimension LP (the
// sketch width padded to a multiple of 8; padding columns are zero).  Small
// matrices are LP x LP row-major.
#include <algorithm>

#include "dd.cuh"
#include "internal.cuh"

namespace pcaone {

namespace {

constexpr int kRowsTile = 32;

// part[b] = A[rows of block b]^T B[rows of block b] (na x nb entries, row-major
// na x nb).  sym: A == B and only the upper triangle is formed (mirrored by the
// reduction).  Row tiles are staged in shared memory as float pairs; each
// thread accumulates Q entries in FP32 pairs.
template <int Q, bool F64>
__global__ void __launch_bounds__(256) k_cross_partial(const double* __restrict__ A, int lda, int na,
                                                       const double* __restrict__ B, int ldb, int nb, int64_t rows,
                                                       int64_t rows_per_block, int sym, double* __restrict__ part,
                                                       const int* __restrict__ only_if) {
  if (only_if && *only_if == 0) return;
  extern __shared__ float smf[];
  float* Ah = smf;                       // kRowsTile x na
  float* Al = Ah + kRowsTile * na;
  float* Bh = Al + kRowsTile * na;       // kRowsTile x nb (not used when sym)
  float* Bl = Bh + kRowsTile * nb;
  double* Ad = reinterpret_cast<double*>(smf);  // F64: the same bytes as doubles
  double* Bd = Ad + kRowsTile * na;
  uint16_t* pi = reinterpret_cast<uint16_t*>(Bl + kRowsTile * nb);
  uint16_t* pj = pi + na * nb;
  const int tid = threadIdx.x;
  int nent = 0;
  if (sym) {
    nent = na * (na + 1) / 2;
    for (int e = tid; e < nent; e += blockDim.x) {
      // row i of the upper triangle starts at i*na - i*(i-1)/2
      int i = 0, base = 0;
      while (base + (na - i) <= e) { base += na - i; ++i; }
      pi[e] = (uint16_t)i;
      pj[e] = (uint16_t)(i + (e - base));
    }
  } else {
    nent = na * nb;
    for (int e = tid; e < nent; e += blockDim.x) {
      pi[e] = (uint16_t)(e / nb);
      pj[e] = (uint16_t)(e % nb);
    }
  }
  const int64_t r0 = blockIdx.x * rows_per_block;
  const int64_t r1 = min(r0 + rows_per_block, rows);
  FloatPair acc[Q];
  double accd[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) accd[q] = 0.0;
  __syncthreads();
  for (int64_t rt = r0; rt < r1; rt += kRowsTile) {
    const int nr = (int)min((int64_t)kRowsTile, r1 - rt);
    for (int e = tid; e < kRowsTile * na; e += blockDim.x) {
      const int r = e / na, c = e % na;
      const double v = r < nr ? A[(rt + r) * lda + c] : 0.0;
      if constexpr (F64)
        Ad[e] = v;
      else
        dd_split_bits(v, Ah[e], Al[e]);
    }
    if (!sym)
      for (int e = tid; e < kRowsTile * nb; e += blockDim.x) {
        const int r = e / nb, c = e % nb;
        const double v = r < nr ? B[(rt + r) * ldb + c] : 0.0;
        if constexpr (F64)
          Bd[e] = v;
        else
          dd_split_bits(v, Bh[e], Bl[e]);
      }
    __syncthreads();
    const int ldt = sym ? na : nb;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int e = tid + q * 256;
      if (e < nent) {
        const int i = pi[e], j = pj[e];
        if constexpr (F64) {
          const double* Td = sym ? Ad : Bd;
          double s = accd[q];
#pragma unroll 8
          for (int r = 0; r < kRowsTile; ++r) s = fma(Ad[r * na + i], Td[r * ldt + j], s);
          accd[q] = s;
        } else {
          const float* Th = sym ? Ah : Bh;
          const float* Tl = sym ? Al : Bl;
          FloatPair s = acc[q];
#pragma unroll 8
          for (int r = 0; r < kRowsTile; ++r)
            fp_add_prod2(s, Ah[r * na + i], Al[r * na + i], Th[r * ldt + j], Tl[r * ldt + j]);
          acc[q] = s;
        }
      }
    }
    __syncthreads();
  }
  double* out = part + (size_t)blockIdx.x * na * nb;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int e = tid + q * 256;
    if (e < nent) out[pi[e] * nb + pj[e]] = F64 ? accd[q] : dd_merge_bits(acc[q].hi, acc[q].lo);
  }
}

// W (ldw columns) = sum over blocks of part, one warp per entry: the lanes sum
// blocks lane, lane+32, ... and a butterfly combines them (a fixed order, so
// the result does not depend on scheduling); sym mirrors the upper triangle.
__global__ void k_cross_reduce(const double* __restrict__ part, int nblocks, int na, int nb, int sym,
                               double* __restrict__ W, int ldw, const int* __restrict__ only_if) {
  if (only_if && *only_if == 0) return;
  const int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (e >= (int64_t)na * nb) return;  // warp-uniform
  const int i = (int)(e / nb), j = (int)(e % nb);
  if (sym && j < i) return;  // warp-uniform
  double s = 0.0;
  for (int b = lane; b < nblocks; b += 32) s += part[(size_t)b * na * nb + e];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    W[i * ldw + j] = s;
    if (sym) W[j * ldw + i] = s;
  }
}

__global__ void k_zero(double* p, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0.0;
}

// Cholesky W = R^T R of the leading L x L block and R^{-1}, both right-looking
// in shared memory, in double-float arithmetic (dd.cuh, about 48 bits): FP64
// runs at a small fraction of the FP32 rate on this GPU, and the dependent
// chain of L pivots (a square root and a reciprocal each) sets the time.
//   factor, step k: row k scaled by 1/d_k, then the trailing upper triangle
//     a_ij -= a_ki a_kj; thread 0 updates a_(k+1)(k+1) first and takes the
//     next pivot's root and reciprocal while the others update;
//   inverse, step k = L-1 .. 0 of R X = I with X = I initially: row k of X
//     times 1/d_k, then rows i < k updated x_ic -= r_ik x_kc.
// The padding block of R and Rinv is the identity.  A non-positive or
// non-finite pivot ORs 1 into *status.  With retry_rows >= 0 a failed factor
// is taken again of W + shift I with the shift of shifted CholeskyQR3,
// 11 (m n + n (n + 1)) u ||A||_F^2 = 11 (rows L + L (L + 1)) 2^-53 trace(W)
// (Fukaya, Kannan, Nakatsukasa, Yamamoto, Yanagisawa 2020), and *shifted (when
// given) records whether it was.  With only_if given and *only_if == 0 the
// kernel does nothing: the later passes of CholeskyQR3 run only when the
// first factor needed the shift, decided on the device.
constexpr int kCholThreads = 512;
// the arithmetic of the factor: double-float (dd) or, in the FP64-grade form,
// FP64 (sqrt and division as CUDA provides them)
__device__ __forceinline__ dd num_from(double v, dd*) { return dd_from_double(v); }
__device__ __forceinline__ double num_from(double v, double*) { return v; }
__device__ __forceinline__ double num_to_double(dd a) { return dd_to_double(a); }
__device__ __forceinline__ double num_to_double(double a) { return a; }
__device__ __forceinline__ dd num_mul(dd a, dd b) { return dd_mul(a, b); }
__device__ __forceinline__ double num_mul(double a, double b) { return a * b; }
__device__ __forceinline__ dd num_fms(dd c, dd a, dd b) { return dd_fms(c, a, b); }
__device__ __forceinline__ double num_fms(double c, double a, double b) { return fma(-a, b, c); }
__device__ __forceinline__ bool num_pos(dd d) { return d.hi > 0.f && isfinite(d.hi); }
__device__ __forceinline__ bool num_pos(double d) { return d > 0.0 && isfinite(d); }
__device__ __forceinline__ dd num_sqrt(dd a) { return dd_sqrt(a); }
__device__ __forceinline__ double num_sqrt(double a) { return sqrt(a); }
__device__ __forceinline__ dd num_recip(dd a) { return dd_div(dd{1.f, 0.f}, a); }
__device__ __forceinline__ double num_recip(double a) { return 1.0 / a; }

template <class T>
__device__ __forceinline__ void chol_pivot(const T* a, int L, int k, T* dg, T* rdg, int* fail) {
  const T d = a[k * L + k];
  const bool ok = num_pos(d);
  if (!ok) *fail = 1;
  const T dk = ok ? num_sqrt(d) : num_from(1.0, (T*)nullptr);
  dg[k] = dk;
  rdg[k] = num_recip(dk);
}

template <class T>
__global__ void __launch_bounds__(kCholThreads) k_chol_inv(const double* __restrict__ W, int L, int LP,
                                                           int64_t retry_rows, double* __restrict__ R,
                                                           double* __restrict__ Rinv, int* __restrict__ status,
                                                           int* __restrict__ shifted, const int* __restrict__ only_if) {
  if (only_if && *only_if == 0) return;
  extern __shared__ dd sdd[];  // L x L factor, L x L inverse, L roots, L reciprocals
  T* a = reinterpret_cast<T*>(sdd);
  T* x = a + L * L;
  T* dg = x + L * L;
  T* rdg = dg + L;
  __shared__ int fail;
  __shared__ double shift;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int attempt = 0; attempt < 2; ++attempt) {
    if (tid == 0) {
      fail = 0;
      double sh = 0.0;
      if (attempt == 1) {
        double tr = 0.0;
        for (int i = 0; i < L; ++i) tr += W[i * LP + i];
        sh = 11.0 * ((double)retry_rows * L + (double)L * (L + 1)) * 1.1102230246251565e-16 * tr;
      }
      shift = sh;
    }
    __syncthreads();
    for (int e = tid; e < L * L; e += nt) {
      const int i = e / L, j = e % L;
      a[e] = num_from(W[i * LP + j] + (i == j ? shift : 0.0), (T*)nullptr);
      x[e] = num_from(i == j ? 1.0 : 0.0, (T*)nullptr);
    }
    __syncthreads();
    if (tid == 0) chol_pivot(a, L, 0, dg, rdg, &fail);
    __syncthreads();
    for (int k = 0; k < L; ++k) {
      const T rk = rdg[k];
      for (int j = k + 1 + tid; j < L; j += nt) a[k * L + j] = num_mul(a[k * L + j], rk);
      __syncthreads();
      const int m = L - k - 1;
      for (int e = tid; e < m * m; e += nt) {
        const int i = k + 1 + e / m, j = k + 1 + e % m;
        if (j >= i) a[i * L + j] = num_fms(a[i * L + j], a[k * L + i], a[k * L + j]);
        if (e == 0) chol_pivot(a, L, k + 1, dg, rdg, &fail);  // element (k+1, k+1) is final now
      }
      __syncthreads();
    }
    if (tid == 0 && shifted) *shifted = attempt;
    if (!fail || retry_rows < 0) break;  // fail and retry_rows are uniform over the block
    __syncthreads();
  }
  for (int k = L - 1; k >= 0; --k) {
    const T rk = rdg[k];
    for (int c = k + tid; c < L; c += nt) x[k * L + c] = num_mul(x[k * L + c], rk);
    __syncthreads();
    const int w = L - k;  // columns k .. L-1
    for (int e = tid; e < k * w; e += nt) {
      const int i = e / w, c = k + e % w;
      x[i * L + c] = num_fms(x[i * L + c], a[i * L + k], x[k * L + c]);
    }
    __syncthreads();
  }
  for (int e = tid; e < LP * LP; e += nt) {
    const int i = e / LP, j = e % LP;
    double v, w;
    if (i < L && j < L) {
      v = j > i ? num_to_double(a[i * L + j]) : (j == i ? num_to_double(dg[i]) : 0.0);
      w = j >= i ? num_to_double(x[i * L + j]) : 0.0;
    } else {
      v = w = i == j ? 1.0 : 0.0;
    }
    R[e] = v;
    Rinv[e] = w;
  }
  if (tid == 0 && fail) atomicOr(status, 1);
}

// C[rows x n] = A[rows x LP] * B[LP x n]; B (zero-padded to a multiple of 48
// columns) and a 32-row tile of A in shared memory as float pairs.  Thread
// (row pair rp, column lane cg) forms rows 2rp, 2rp+1 and columns cg, cg+16,
// cg+32 of each 48-column chunk in FP32 pairs, so every pair of operands it
// loads serves three or two products.  C may alias A (ldc == LP, n <= LP):
// each CTA reads a row tile into shared memory before it writes the same rows.
constexpr int kTallCols = 48;
template <bool F64>
__global__ void __launch_bounds__(256) k_gemm_tall(const double* A, int64_t rows, int LP,
                                                   const double* __restrict__ B, int ldb, int n, double* C,
                                                   int ldc) {
  extern __shared__ float smf[];
  const int npd = (n + kTallCols - 1) / kTallCols * kTallCols;
  float* Bh = smf;              // LP x npd
  float* Bl = Bh + LP * npd;
  const int las = LP + 1;       // row stride of the A tile (odd: no bank conflicts between row pairs)
  float* Ah = Bl + LP * npd;    // 32 x las
  float* Al = Ah + kRowsTile * las;
  double* Bd = reinterpret_cast<double*>(smf);  // F64: the same bytes as doubles
  double* Ad = Bd + LP * npd;
  const int tid = threadIdx.x;
  for (int e = tid; e < LP * npd; e += blockDim.x) {
    const int t = e / npd, c = e % npd;
    const double v = c < n ? B[t * ldb + c] : 0.0;
    if constexpr (F64)
      Bd[e] = v;
    else
      dd_split_bits(v, Bh[e], Bl[e]);
  }
  const int r = 2 * (tid >> 4), cg = tid & 15;
  for (int64_t rt = (int64_t)blockIdx.x * kRowsTile; rt < rows; rt += (int64_t)gridDim.x * kRowsTile) {
    __syncthreads();
    for (int e = tid; e < kRowsTile * LP; e += blockDim.x) {
      const int rr = e / LP, cc = e % LP;
      const int64_t row = rt + rr;
      const double v = row < rows ? A[row * LP + cc] : 0.0;
      if constexpr (F64)
        Ad[rr * las + cc] = v;
      else
        dd_split_bits(v, Ah[rr * las + cc], Al[rr * las + cc]);
    }
    __syncthreads();
    const int64_t row0 = rt + r;
    for (int c0 = 0; c0 < n; c0 += kTallCols) {
      FloatPair s[2][3];
      double sd[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
      if constexpr (F64) {
        const double* a0 = Ad + r * las;
        const double* b = Bd + c0 + cg;
#pragma unroll 4
        for (int t = 0; t < LP; ++t) {
          const double x0 = a0[t], x1 = a0[las + t];
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            const double y = b[t * npd + 16 * q];
            sd[0][q] = fma(x0, y, sd[0][q]);
            sd[1][q] = fma(x1, y, sd[1][q]);
          }
        }
      } else {
        const float* a0h = Ah + r * las;
        const float* a0l = Al + r * las;
        const float* bh = Bh + c0 + cg;
        const float* bl = Bl + c0 + cg;
#pragma unroll 4
        for (int t = 0; t < LP; ++t) {
          const float x0h = a0h[t], x0l = a0l[t], x1h = a0h[las + t], x1l = a0l[las + t];
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            const float yh = bh[t * npd + 16 * q], yl = bl[t * npd + 16 * q];
            fp_add_prod2(s[0][q], x0h, x0l, yh, yl);
            fp_add_prod2(s[1][q], x1h, x1l, yh, yl);
          }
        }
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (row0 + h < rows) {
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            const int c = c0 + cg + 16 * q;
            if (c < n) C[(row0 + h) * ldc + c] = F64 ? sd[h][q] : dd_merge_bits(s[h][q].hi, s[h][q].lo);
          }
        }
      }
    }
  }
}

// C = A * B in place (C == A, n == ldb == LP) for B upper triangular
// (B[t][c] = 0 for t > c: the R^{-1} factors of CholeskyQR), so column c needs
// only t <= c.  Lane = row of a 32-row tile; warp w takes the columns c whose
// position r = c % 16 in its 16-column block is w or 15 - w, which gives
// every warp the same number of products and warp-uniform loop bounds.  Each
// output accumulates the same FP32-pair terms in the same order as
// k_gemm_tall: the skipped terms are exact zeros there.
constexpr int kUpperMaxQ = 14;  // columns per warp: LP / 8 with LP <= 112
template <bool F64>
__global__ void __launch_bounds__(256) k_gemm_tall_upper(double* A, int64_t rows, int LP,
                                                         const double* __restrict__ B, const int* __restrict__ only_if) {
  if (only_if && *only_if == 0) return;
  extern __shared__ float smf[];
  const int las = LP + 1;  // odd row stride of the A tile: lanes hit distinct banks
  float* Bh = smf;         // LP x LP
  float* Bl = Bh + LP * LP;
  float* Ah = Bl + LP * LP;  // 32 x las
  float* Al = Ah + kRowsTile * las;
  double* Bd = reinterpret_cast<double*>(smf);  // F64: the same bytes as doubles
  double* Ad = Bd + LP * LP;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int e = tid; e < LP * LP; e += blockDim.x) {
    if constexpr (F64)
      Bd[e] = B[e];
    else
      dd_split_bits(B[e], Bh[e], Bl[e]);
  }
  int cmax = -1;
#pragma unroll
  for (int q = 0; q < kUpperMaxQ; ++q) {
    const int c = 16 * (q >> 1) + ((q & 1) ? 15 - warp : warp);
    if (c < LP) cmax = max(cmax, c);
  }
  for (int64_t rt = (int64_t)blockIdx.x * kRowsTile; rt < rows; rt += (int64_t)gridDim.x * kRowsTile) {
    __syncthreads();
    for (int e = tid; e < kRowsTile * LP; e += blockDim.x) {
      const int rr = e / LP, cc = e % LP;
      const int64_t row = rt + rr;
      const double v = row < rows ? A[row * LP + cc] : 0.0;
      if constexpr (F64)
        Ad[rr * las + cc] = v;
      else
        dd_split_bits(v, Ah[rr * las + cc], Al[rr * las + cc]);
    }
    __syncthreads();
    FloatPair s[kUpperMaxQ];
    double sd[kUpperMaxQ];
#pragma unroll
    for (int q = 0; q < kUpperMaxQ; ++q) sd[q] = 0.0;
    if constexpr (F64) {
      const double* ad = Ad + lane * las;
      for (int t = 0; t <= cmax; ++t) {
        const double x = ad[t];
#pragma unroll
        for (int q = 0; q < kUpperMaxQ; ++q) {
          const int c = 16 * (q >> 1) + ((q & 1) ? 15 - warp : warp);
          if (c < LP && t <= c) sd[q] = fma(x, Bd[t * LP + c], sd[q]);
        }
      }
    } else {
      const float* ah = Ah + lane * las;
      const float* al = Al + lane * las;
      for (int t = 0; t <= cmax; ++t) {
        const float xh = ah[t], xl = al[t];
#pragma unroll
        for (int q = 0; q < kUpperMaxQ; ++q) {
          const int c = 16 * (q >> 1) + ((q & 1) ? 15 - warp : warp);
          if (c < LP && t <= c) fp_add_prod2(s[q], xh, xl, Bh[t * LP + c], Bl[t * LP + c]);
        }
      }
    }
    const int64_t row = rt + lane;
    if (row < rows) {
#pragma unroll
      for (int q = 0; q < kUpperMaxQ; ++q) {
        const int c = 16 * (q >> 1) + ((q & 1) ? 15 - warp : warp);
        if (c < LP) A[row * LP + c] = F64 ? sd[q] : dd_merge_bits(s[q].hi, s[q].lo);
      }
    }
  }
}

// The same product in FP32 pairs, register-blocked: a CTA takes 64-row tiles
// of A (read once, split into float pairs in shared memory from the doubles'
// bits, no FP64 arithmetic), thread (rg, cg) forms rows 4rg .. 4rg+3 and
// columns cg, cg+16, ... (LP/16 of them), so each float pair it loads from
// shared memory serves four (A) or up to seven (B) products.  Column block j
// (columns 16j .. 16j+15) needs the rows t < 16(j+1) of B only; within the
// diagonal block the terms t > column are exact zeros of B and are skipped by
// a predicate.  Every output accumulates the same terms in the same order
// (t increasing) as k_gemm_tall_upper.
constexpr int kUpRows = 64;
constexpr int kUpMaxJ = 7;  // LP / 16 with LP <= 112
__global__ void __launch_bounds__(256) k_gemm_tall_upper_rb(double* A, int64_t rows, int LP,
                                                            const double* __restrict__ B,
                                                            const int* __restrict__ only_if) {
  if (only_if && *only_if == 0) return;
  extern __shared__ float2 smp[];
  float2* Bs = smp;                    // LP x LP (hi, lo)
  float2* As = Bs + LP * LP;           // kUpRows x (LP + 1): odd row stride
  const int las = LP + 1;
  const int tid = threadIdx.x, rg = tid >> 4, cg = tid & 15;
  const int J = LP >> 4;
  for (int e = tid; e < LP * LP; e += blockDim.x) {
    float h, l;
    dd_split_bits(B[e], h, l);
    Bs[e] = make_float2(h, l);
  }
  for (int64_t rt = (int64_t)blockIdx.x * kUpRows; rt < rows; rt += (int64_t)gridDim.x * kUpRows) {
    __syncthreads();
    // element e = rr * LP + cc of the tile, stepped by the block size without a division
    for (int e = tid, rr = tid / LP, cc = tid % LP; e < kUpRows * LP; e += blockDim.x) {
      const int64_t row = rt + rr;
      float h = 0.f, l = 0.f;
      if (row < rows) dd_split_bits(A[row * LP + cc], h, l);
      As[rr * las + cc] = make_float2(h, l);
      cc += blockDim.x;
      while (cc >= LP) {
        cc -= LP;
        ++rr;
      }
    }
    __syncthreads();
    FloatPair acc[4][kUpMaxJ];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < kUpMaxJ; ++j) acc[i][j] = FloatPair{};
    const float2* a0 = As + (4 * rg) * las;
    for (int tb = 0; tb < J; ++tb) {
      for (int tt = 0; tt < 16; ++tt) {
        const int t = 16 * tb + tt;
        const float2 x0 = a0[t], x1 = a0[las + t], x2 = a0[2 * las + t], x3 = a0[3 * las + t];
        const float2* brow = Bs + t * LP + cg;
#pragma unroll
        for (int j = 0; j < kUpMaxJ; ++j) {
          // column cg + 16j: rows t <= cg + 16j of B; blocks j < tb hold only zeros at row t
          if (j < J && j >= tb && (j > tb || tt <= cg)) {
            const float2 y = brow[16 * j];
            fp_add_prod2(acc[0][j], x0.x, x0.y, y.x, y.y);
            fp_add_prod2(acc[1][j], x1.x, x1.y, y.x, y.y);
            fp_add_prod2(acc[2][j], x2.x, x2.y, y.x, y.y);
            fp_add_prod2(acc[3][j], x3.x, x3.y, y.x, y.y);
          }
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t row = rt + 4 * rg + i;
      if (row >= rows) continue;
#pragma unroll
      for (int j = 0; j < kUpMaxJ; ++j)
        if (j < J) A[row * LP + cg + 16 * j] = dd_merge_bits(acc[i][j].hi, acc[i][j].lo);
    }
  }
}

// Signs d_i an Eigen/LAPACK Householder QR gives its Q relative to the
// positive-diagonal factor: the modified LU of the top L x L block of the
// orthonormal Q (Ballard et al., "Reconstructing Householder vectors from
// tall-skinny QR", 2015): s_i = -sign(a_ii) with sign(0) = +1, a_ii -= s_i,
// then eliminate below the pivot.  Mirrors beta = -sign(c0)*norm of the
// reflector (Eigen makeHouseholder; LAPACK dlarfg).
__global__ void k_house_signs(const double* __restrict__ Q, int L, int LP, double* __restrict__ sgn) {
  extern __shared__ double a[];  // L x L, then L multipliers
  double* mult = a + L * L;
  const int tid = threadIdx.x;
  for (int e = tid; e < L * L; e += blockDim.x) a[e] = Q[(e / L) * LP + (e % L)];
  __syncthreads();
  for (int i = 0; i < L; ++i) {
    if (tid == 0) {
      const double s = a[i * L + i] >= 0.0 ? -1.0 : 1.0;
      sgn[i] = s;
      a[i * L + i] -= s;
    }
    __syncthreads();
    const int m = L - i - 1;
    const double piv = a[i * L + i];
    // multipliers first (column i below the pivot, in its own buffer), then
    // the trailing update with the same rounding as a[r][i] / piv * a[i][c]
    for (int r = i + 1 + tid; r < L; r += blockDim.x) mult[r] = a[r * L + i] / piv;
    __syncthreads();
    for (int e = tid; e < m * m; e += blockDim.x) {
      const int r = i + 1 + e / m, c = i + 1 + e % m;
      a[r * L + c] -= mult[r] * a[i * L + c];
    }
    __syncthreads();
  }
  for (int c = L + tid; c < LP; c += blockDim.x) sgn[c] = 1.0;
}

__global__ void k_scale_cols(double* __restrict__ Q, int64_t rows, int LP, const double* __restrict__ sgn) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= rows * LP) return;
  Q[idx] *= sgn[idx % LP];
}

// column sums of |o2 - o| and |o2 + o| over a slab of rows: coalesced loads
// (thread t keeps column t % LP), then the threads of each column combined in
// shared memory
__global__ void __launch_bounds__(256) k_flip_partial(const double* __restrict__ o2, const double* __restrict__ o,
                                                      int64_t rows, int LP, int64_t rows_per_block,
                                                      double* __restrict__ part) {
  __shared__ double rm[256], rp[256];
  const int tid = threadIdx.x;
  const int step = (256 / LP) * LP;
  const int64_t r0 = blockIdx.x * rows_per_block, r1 = min(r0 + rows_per_block, rows);
  double dm = 0.0, dp = 0.0;
  if (tid < step) {
    for (int64_t f = r0 * LP + tid; f < r1 * LP; f += step) {
      const double a = o2[f], b = o[f];
      dm += fabs(a - b);
      dp += fabs(a + b);
    }
  }
  rm[tid] = dm;
  rp[tid] = dp;
  __syncthreads();
  if (tid < LP) {
    for (int q = tid + LP; q < step; q += LP) {
      dm += rm[q];
      dp += rp[q];
    }
    part[((size_t)blockIdx.x * 2 + 0) * LP + tid] = dm;
    part[((size_t)blockIdx.x * 2 + 1) * LP + tid] = dp;
  }
}

// one warp per column: the block partials summed by the lanes and a butterfly
__global__ void k_flip_flags(const double* __restrict__ part, int nblocks, int L, int LP, double* __restrict__ sgn) {
  const int c = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= LP) return;  // warp-uniform
  double dm = 0.0, dp = 0.0;
  for (int b = lane; b < nblocks; b += 32) {
    dm += part[((size_t)b * 2 + 0) * LP + c];
    dp += part[((size_t)b * 2 + 1) * LP + c];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dm += __shfl_xor_sync(0xffffffffu, dm, o);
    dp += __shfl_xor_sync(0xffffffffu, dp, o);
  }
  if (lane == 0) sgn[c] = (c < L && dm > 2.0 * dp) ? -1.0 : 1.0;
}

__global__ void k_flip_apply(double* __restrict__ o2, double* __restrict__ o, int64_t n, int LP,
                             const double* __restrict__ sgn) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const double v = o[idx] * sgn[idx % LP];
  o[idx] = v;
  o2[idx] = v;
}

__global__ void k_add(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ c, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) c[i] = a[i] + b[i];
}

__global__ void k_to_f32(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

// C = A * B for LP x LP row-major (single CTA, operands staged in shared memory)
__global__ void __launch_bounds__(512) k_mult_small(const double* __restrict__ A, const double* __restrict__ B,
                                                    double* __restrict__ C, int LP, const int* __restrict__ only_if) {
  if (only_if && *only_if == 0) return;
  extern __shared__ double sab[];
  double* As = sab;
  double* Bs = sab + LP * LP;
  for (int e = threadIdx.x; e < LP * LP; e += blockDim.x) {
    As[e] = A[e];
    Bs[e] = B[e];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < LP * LP; e += blockDim.x) {
    const int i = e / LP, j = e % LP;
    double s = 0.0;
    for (int t = 0; t < LP; ++t) s = fma(As[i * LP + t], Bs[t * LP + j], s);
    C[e] = s;
  }
}

// Rayleigh-Ritz / small SVD of B = R^{-T} H^T through C = B B^T =
// Rinv^T (H^T H) Rinv, eigen-decomposed by the cyclic Jacobi method with
// round-robin parallel ordering (Golub & Van Loan, Matrix Computations,
// sections 8.5.2 and 8.5.5).  Outputs: UB (LP x LP, eigenvectors by column,
// sorted by decreasing eigenvalue), sigma (L) = sqrt(eigenvalues) and
// T = Rinv * UB[:, :k] * diag(1/sigma_k) (LP x k) so that the right singular
// vectors of B are H*T.  Single CTA; C and the eigenvectors in shared memory.
__global__ void __launch_bounds__(1024) k_usv_small(const double* __restrict__ Rinv, const double* __restrict__ Wh,
                                                    int L, int LP, int k, double* __restrict__ UB,
                                                    double* __restrict__ sigma, double* __restrict__ T,
                                                    double* __restrict__ tmp, int* __restrict__ status) {
  extern __shared__ double sm[];
  double* C = sm;              // L x L
  double* V = sm + L * L;      // L x L, V[m*L + p] = component m of vector p
  __shared__ int order[128];
  __shared__ double cs[64], sn[64];
  __shared__ int pp[64], qq[64];
  __shared__ double offn, dn;
  __shared__ int perm_sorted[128];
  const int tid = threadIdx.x, nt = blockDim.x;
  // tmp = Wh * Rinv (L x L), then C = Rinv^T * tmp
  for (int e = tid; e < L * L; e += nt) {
    const int i = e / L, j = e % L;
    double s = 0.0;
    for (int t = 0; t <= j; ++t) s = fma(Wh[i * LP + t], Rinv[t * LP + j], s);
    tmp[e] = s;
  }
  __syncthreads();
  for (int e = tid; e < L * L; e += nt) {
    const int i = e / L, j = e % L;
    double s = 0.0;
    for (int t = 0; t <= i; ++t) s = fma(Rinv[t * LP + i], tmp[t * L + j], s);
    C[e] = s;
    V[e] = (i == j) ? 1.0 : 0.0;
  }
  const int n = (L + 1) & ~1;  // even player count; index L (if L odd) is a bye
  for (int i = tid; i < n; i += nt) order[i] = i;
  __syncthreads();
  // symmetrise
  for (int e = tid; e < L * L; e += nt) {
    const int i = e / L, j = e % L;
    if (j > i) {
      const double m = 0.5 * (C[i * L + j] + C[j * L + i]);
      C[i * L + j] = m;
      C[j * L + i] = m;
    }
  }
  __syncthreads();
  int sweep = 0;
  for (; sweep < 60; ++sweep) {
    if (tid == 0) {
      offn = 0.0;
      dn = 0.0;
    }
    __syncthreads();
    // convergence test on the Frobenius norms
    double lo = 0.0, ld = 0.0;
    for (int e = tid; e < L * L; e += nt) {
      const int i = e / L, j = e % L;
      const double v = C[e] * C[e];
      if (i == j) ld += v; else lo += v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      lo += __shfl_xor_sync(0xffffffffu, lo, o);
      ld += __shfl_xor_sync(0xffffffffu, ld, o);
    }
    if ((tid & 31) == 0) {
      atomicAdd(&offn, lo);
      atomicAdd(&dn, ld);
    }
    __syncthreads();
    if (!(offn > 1e-30 * dn) || L < 2) break;
    for (int round = 0; round < n - 1; ++round) {
      // rotation parameters for the n/2 disjoint pairs of this round
      for (int pr = tid; pr < n / 2; pr += nt) {
        int p = order[pr], q = order[n - 1 - pr];
        if (p > q) { const int t = p; p = q; q = t; }
        pp[pr] = p;
        qq[pr] = q;
        double c = 1.0, s = 0.0;
        if (q < L) {
          const double apq = C[p * L + q];
          if (fabs(apq) > 1e-300) {
            const double tau = (C[q * L + q] - C[p * L + p]) / (2.0 * apq);
            const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        }
        cs[pr] = c;
        sn[pr] = s;
      }
      __syncthreads();
      // C <- J^T C (rows p, q)
      for (int e = tid; e < (n / 2) * L; e += nt) {
        const int pr = e / L, m = e % L;
        const int p = pp[pr], q = qq[pr];
        if (q >= L) continue;
        const double c = cs[pr], s = sn[pr];
        const double ap = C[p * L + m], aq = C[q * L + m];
        C[p * L + m] = c * ap - s * aq;
        C[q * L + m] = s * ap + c * aq;
      }
      __syncthreads();
      // C <- C J (columns p, q) and V <- V J
      for (int e = tid; e < (n / 2) * L; e += nt) {
        const int pr = e / L, m = e % L;
        const int p = pp[pr], q = qq[pr];
        if (q >= L) continue;
        const double c = cs[pr], s = sn[pr];
        const double ap = C[m * L + p], aq = C[m * L + q];
        C[m * L + p] = c * ap - s * aq;
        C[m * L + q] = s * ap + c * aq;
        const double vp = V[m * L + p], vq = V[m * L + q];
        V[m * L + p] = c * vp - s * vq;
        V[m * L + q] = s * vp + c * vq;
      }
      __syncthreads();
      if (tid == 0) {  // round-robin: keep order[0], rotate the rest
        const int last = order[n - 1];
        for (int i = n - 1; i > 1; --i) order[i] = order[i - 1];
        order[1] = last;
      }
      __syncthreads();
    }
  }
  // sort by decreasing eigenvalue
  if (tid == 0) {
    for (int i = 0; i < L; ++i) perm_sorted[i] = i;
    for (int i = 0; i < L; ++i) {
      int best = i;
      for (int j = i + 1; j < L; ++j)
        if (C[perm_sorted[j] * L + perm_sorted[j]] > C[perm_sorted[best] * L + perm_sorted[best]]) best = j;
      const int t = perm_sorted[i];
      perm_sorted[i] = perm_sorted[best];
      perm_sorted[best] = t;
    }
    *status = sweep >= 60 ? 2 : 0;
  }
  __syncthreads();
  for (int e = tid; e < LP * LP; e += nt) {
    const int i = e / LP, j = e % LP;
    UB[e] = (i < L && j < L) ? V[i * L + perm_sorted[j]] : (i == j ? 1.0 : 0.0);
  }
  for (int j = tid; j < L; j += nt) {
    const double lam = C[perm_sorted[j] * L + perm_sorted[j]];
    sigma[j] = sqrt(lam > 0.0 ? lam : 0.0);
  }
  __syncthreads();
  // T = Rinv * UB[:, :k] * diag(1/sigma)
  for (int e = tid; e < LP * k; e += nt) {
    const int i = e / k, j = e % k;
    double s = 0.0;
    if (i < L)
      for (int t = i; t < L; ++t) s = fma(Rinv[i * LP + t], V[t * L + perm_sorted[j]], s);
    const double sg = sqrt(fmax(C[perm_sorted[j] * L + perm_sorted[j]], 0.0));
    T[e] = sg > 0.0 ? s / sg : 0.0;
  }
}

// mev(X, Y) = (1/k) sum_i || X^T y_i ||  from M = X^T Y (k x k)
__global__ void k_mev_finish(const double* __restrict__ Mxy, int k, double* __restrict__ out) {
  __shared__ double acc;
  if (threadIdx.x == 0) acc = 0.0;
  __syncthreads();
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < k; ++j) s += Mxy[j * k + i] * Mxy[j * k + i];
    atomicAdd(&acc, sqrt(s));
  }
  __syncthreads();
  if (threadIdx.x == 0) *out = acc / k;
}

// EM fill (Data::fit_with_pi EMU branches, src/Data.cpp:318-348): missing entry
// (position p, sample i) <- clamp(sum_k U[i][k] S[k] V[p][k], -F_j, 1 - F_j),
// F of the SNP at position p.
__global__ void k_em_fill(const int32_t* __restrict__ epos, const int32_t* __restrict__ sample,
                          double* __restrict__ value, int64_t nnz, const int32_t* __restrict__ perm,
                          const double* __restrict__ F, const double* __restrict__ U, const double* __restrict__ S,
                          const double* __restrict__ V, int k) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= nnz) return;
  const int64_t p = epos[e];
  const int64_t i = sample[e];
  const int64_t snp = perm ? (int64_t)perm[p] : p;
  double t = 0.0;
  for (int q = 0; q < k; ++q) t += U[i * k + q] * S[q] * V[p * k + q];
  const double f = F[snp];
  value[e] = fmin(fmax(t, -f), 1.0 - f);
}

// Arnoldi matvec, first half: t[j] = sum_i x(i,j) * xin[i] (one warp per SNP)
__global__ void k_matvec_t(BedView v, const double* __restrict__ F, const double* __restrict__ scale,
                           const double* __restrict__ xin, double* __restrict__ t) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= v.nsnps) return;
  const double f = F[warp], s = scale[warp];
  const double tab[4] = {(1.0 - f) * s, 0.0, (0.5 - f) * s, (0.0 - f) * s};
  const uint8_t* row = v.bed + warp * v.stride;
  double acc = 0.0;
  const int nbytes = (v.nsamples + 3) >> 2;
  for (int b = lane; b < nbytes; b += 32) {
    const uint32_t w = row[b];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = b * 4 + q;
      if (i < v.nsamples) {
        const uint32_t c = (w >> (2 * q)) & 3u;
        const double x = c == 0 ? tab[0] : (c == 1 ? 0.0 : (c == 2 ? tab[2] : tab[3]));
        acc = fma(x, xin[i], acc);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) t[warp] = acc;
}

// second half: ypart[split][i] = sum_{j in split} x(i,j) * t[j]
__global__ void k_matvec_y(BedView v, const double* __restrict__ F, const double* __restrict__ scale,
                           const double* __restrict__ t, int64_t per_split, double* __restrict__ ypart) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= v.nsamples) return;
  const int64_t j0 = blockIdx.y * per_split, j1 = min(j0 + per_split, v.nsnps);
  double acc = 0.0;
  const int64_t byte = i >> 2;
  const int sh = 2 * (int)(i & 3);
  for (int64_t j = j0; j < j1; ++j) {
    const uint32_t c = (v.bed[j * v.stride + byte] >> sh) & 3u;
    if (c == 1u) continue;
    const double g = c == 0 ? 1.0 : (c == 2 ? 0.5 : 0.0);
    acc = fma((g - F[j]) * scale[j], t[j], acc);
  }
  ypart[(size_t)blockIdx.y * v.nsamples + i] = acc;
}

__global__ void k_matvec_reduce(const double* __restrict__ ypart, int nsplit, int n, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int b = 0; b < nsplit; ++b) s += ypart[(size_t)b * n + i];
  y[i] = s;
}

// R = Y_n - X_n M for the leading n columns of two orthonormal N x k blocks
// (row-major, ld k) with M = X_n^T Y_n (n x n, row-major): the part of Y_n's
// columns outside span(X_n), in FP64
__global__ void k_subspace_residual(const double* __restrict__ X, const double* __restrict__ Y, int k, int n,
                                    const double* __restrict__ M, int64_t rows, double* __restrict__ R) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= rows * n) return;
  const int64_t r = e / n;
  const int c = (int)(e - r * n);
  double v = Y[r * k + c];
  for (int j = 0; j < n; ++j) v = fma(-X[r * k + j], M[j * n + c], v);
  R[e] = v;
}

__global__ void k_copy_if(const double* __restrict__ src, double* __restrict__ dst, int64_t n,
                          const int* __restrict__ only_if) {
  if (*only_if == 0) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

}  // namespace

// ---------------------------------------------------------------------------

int cross_blocks(int64_t rows) { return (int)std::max<int64_t>(1, std::min<int64_t>(304, (rows + 63) / 64)); }

size_t cross_smem(int na, int nb, int sym) {
  (void)sym;
  return 2 * sizeof(float) * kRowsTile * (na + nb) + 2 * sizeof(uint16_t) * na * nb + 64;
}

template <int Q, bool F64>
void launch_cross_qf(const double* A, int lda, int na, const double* B, int ldb, int nb, int64_t rows, int64_t per,
                     int sym, double* part, int nblocks, size_t smem, cudaStream_t s, const int* only_if) {
  static bool attr_set = false;
  if (!attr_set) {
    PCAONE_CUDA(
        cudaFuncSetAttribute(k_cross_partial<Q, F64>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_set = true;
  }
  k_cross_partial<Q, F64><<<nblocks, 256, smem, s>>>(A, lda, na, B, ldb, nb, rows, per, sym, part, only_if);
}
template <int Q>
void launch_cross_q(const double* A, int lda, int na, const double* B, int ldb, int nb, int64_t rows, int64_t per,
                    int sym, double* part, int nblocks, size_t smem, bool f64, cudaStream_t s, const int* only_if) {
  if (f64)
    launch_cross_qf<Q, true>(A, lda, na, B, ldb, nb, rows, per, sym, part, nblocks, smem, s, only_if);
  else
    launch_cross_qf<Q, false>(A, lda, na, B, ldb, nb, rows, per, sym, part, nblocks, smem, s, only_if);
}

void launch_cross(const double* A, int lda, int na, const double* B, int ldb, int nb, int64_t rows, int sym,
                  double* W, int ldw, double* part, int nblocks, cudaStream_t s, bool f64, const int* only_if) {
  if (na * nb > 64 * 256 || na > 0xffff) throw Error(-6, "cross product wider than 128 x 128");
  if (rows == 0) {
    k_zero<<<ceil_div((int64_t)na * ldw, 256), 256, 0, s>>>(W, (int64_t)na * ldw);
    PCAONE_LAUNCH_CHECK();
    return;
  }
  const int64_t per = round_up64((rows + nblocks - 1) / nblocks, kRowsTile);
  nblocks = (int)((rows + per - 1) / per);
  const size_t smem = cross_smem(na, nb, sym);
  const int nent = sym ? na * (na + 1) / 2 : na * nb;
  const int q = (nent + 255) / 256;
  const double* Bv = sym ? A : B;
  const int ldbv = sym ? lda : ldb;
  if (q <= 4)
    launch_cross_q<4>(A, lda, na, Bv, ldbv, nb, rows, per, sym, part, nblocks, smem, f64, s, only_if);
  else if (q <= 8)
    launch_cross_q<8>(A, lda, na, Bv, ldbv, nb, rows, per, sym, part, nblocks, smem, f64, s, only_if);
  else if (q <= 16)
    launch_cross_q<16>(A, lda, na, Bv, ldbv, nb, rows, per, sym, part, nblocks, smem, f64, s, only_if);
  else if (q <= 32)
    launch_cross_q<32>(A, lda, na, Bv, ldbv, nb, rows, per, sym, part, nblocks, smem, f64, s, only_if);
  else
    launch_cross_q<64>(A, lda, na, Bv, ldbv, nb, rows, per, sym, part, nblocks, smem, f64, s, only_if);
  PCAONE_LAUNCH_CHECK();
  k_cross_reduce<<<ceil_div((int64_t)na * nb * 32, 256), 256, 0, s>>>(part, nblocks, na, nb, sym, W, ldw, only_if);
  PCAONE_LAUNCH_CHECK();
}

template <class T>
void launch_chol_t(const double* W, int L, int LP, int64_t retry_rows, double* R, double* Rinv, int* status,
                   int* shifted, const int* only_if, cudaStream_t s) {
  static bool attr_set = false;
  if (!attr_set) {
    PCAONE_CUDA(cudaFuncSetAttribute(k_chol_inv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_set = true;
  }
  static_assert(sizeof(T) == sizeof(dd), "factor element size");
  k_chol_inv<T><<<1, kCholThreads, sizeof(T) * (2 * L * L + 2 * L), s>>>(W, L, LP, retry_rows, R, Rinv, status,
                                                                         shifted, only_if);
}

void launch_chol_inv(const double* W, int L, int LP, double* R, double* Rinv, int* status, cudaStream_t s, bool f64,
                     int64_t retry_rows, int* shifted, const int* only_if) {
  if (f64)
    launch_chol_t<double>(W, L, LP, retry_rows, R, Rinv, status, shifted, only_if, s);
  else
    launch_chol_t<dd>(W, L, LP, retry_rows, R, Rinv, status, shifted, only_if, s);
  PCAONE_LAUNCH_CHECK();
}

template <bool F64>
void launch_gemm_tall_t(const double* A, int64_t rows, int LP, const double* B, int ldb, int n, double* C, int ldc,
                        cudaStream_t s) {
  static bool attr_set = false;
  if (!attr_set) {
    PCAONE_CUDA(cudaFuncSetAttribute(k_gemm_tall<F64>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_set = true;
  }
  const size_t npd = (size_t)(n + kTallCols - 1) / kTallCols * kTallCols;
  const size_t smem = 2 * sizeof(float) * ((size_t)LP * npd + (size_t)kRowsTile * (LP + 1));
  const int grid = (int)std::min<int64_t>((rows + kRowsTile - 1) / kRowsTile, 152 * 8);
  k_gemm_tall<F64><<<grid, 256, smem, s>>>(A, rows, LP, B, ldb, n, C, ldc);
}

void launch_gemm_tall(const double* A, int64_t rows, int LP, const double* B, int ldb, int n, double* C, int ldc,
                      cudaStream_t s, bool f64) {
  if (rows == 0) return;
  if (f64)
    launch_gemm_tall_t<true>(A, rows, LP, B, ldb, n, C, ldc, s);
  else
    launch_gemm_tall_t<false>(A, rows, LP, B, ldb, n, C, ldc, s);
  PCAONE_LAUNCH_CHECK();
}

void launch_gemm_tall_upper_rb(double* A, int64_t rows, int LP, const double* B, cudaStream_t s, const int* only_if) {
  static bool attr_set = false;
  if (!attr_set) {
    PCAONE_CUDA(cudaFuncSetAttribute(k_gemm_tall_upper_rb, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_set = true;
  }
  const size_t smem = sizeof(float2) * ((size_t)LP * LP + (size_t)kUpRows * (LP + 1));
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    PCAONE_CUDA(cudaGetDevice(&dev));
    PCAONE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  const int per_sm = std::max(1, std::min(4, (int)((200 * 1024) / smem)));
  const int grid = (int)std::min<int64_t>((rows + kUpRows - 1) / kUpRows, (int64_t)sms * per_sm);
  k_gemm_tall_upper_rb<<<grid, 256, smem, s>>>(A, rows, LP, B, only_if);
}

template <bool F64>
void launch_gemm_tall_upper_t(double* A, int64_t rows, int LP, const double* B, cudaStream_t s, const int* only_if) {
  static bool attr_set = false;
  if (!attr_set) {
    PCAONE_CUDA(
        cudaFuncSetAttribute(k_gemm_tall_upper<F64>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_set = true;
  }
  const size_t smem = 2 * sizeof(float) * ((size_t)LP * LP + (size_t)kRowsTile * (LP + 1));
  const int grid = (int)std::min<int64_t>((rows + kRowsTile - 1) / kRowsTile, 152 * 8);
  k_gemm_tall_upper<F64><<<grid, 256, smem, s>>>(A, rows, LP, B, only_if);
}

void launch_gemm_tall_upper(double* A, int64_t rows, int LP, const double* B, cudaStream_t s, bool f64,
                            const int* only_if) {
  if (rows == 0) return;
  if (LP % 8 != 0 || LP > 8 * kUpperMaxQ) throw Error(-6, "triangular tall product: width must be a multiple of 8, at most 112");
  if (f64)
    launch_gemm_tall_upper_t<true>(A, rows, LP, B, s, only_if);
  else if (LP % 16 == 0)
    launch_gemm_tall_upper_rb(A, rows, LP, B, s, only_if);
  else
    launch_gemm_tall_upper_t<false>(A, rows, LP, B, s, only_if);
  PCAONE_LAUNCH_CHECK();
}

void launch_house_signs(double* Q, int64_t rows, int L, int LP, double* sgn, cudaStream_t s) {
  static bool attr_set = false;
  if (!attr_set) {
    PCAONE_CUDA(cudaFuncSetAttribute(k_house_signs, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_set = true;
  }
  k_house_signs<<<1, 256, sizeof(double) * (L * L + L), s>>>(Q, L, LP, sgn);
  PCAONE_LAUNCH_CHECK();
  k_scale_cols<<<ceil_div(rows * LP, 256), 256, 0, s>>>(Q, rows, LP, sgn);
  PCAONE_LAUNCH_CHECK();
}

int flip_blocks(int64_t rows) { return (int)std::max<int64_t>(1, std::min<int64_t>(304, (rows + 255) / 256)); }

void launch_flip_omg(double* omg2, double* omg, int64_t rows, int L, int LP, double* part, double* sgn,
                     cudaStream_t s) {
  int nb = flip_blocks(rows);
  const int64_t per = (rows + nb - 1) / nb;
  nb = (int)((rows + per - 1) / per);
  if (LP > 256) throw Error(-6, "flipOmg: sketch wider than 256 columns");
  k_flip_partial<<<nb, 256, 0, s>>>(omg2, omg, rows, LP, per, part);
  PCAONE_LAUNCH_CHECK();
  k_flip_flags<<<ceil_div((int64_t)LP * 32, 256), 256, 0, s>>>(part, nb, L, LP, sgn);
  PCAONE_LAUNCH_CHECK();
  k_flip_apply<<<ceil_div(rows * LP, 256), 256, 0, s>>>(omg2, omg, rows * LP, LP, sgn);
  PCAONE_LAUNCH_CHECK();
}

void launch_add(const double* a, const double* b, double* c, int64_t n, cudaStream_t s) {
  if (n == 0) return;
  k_add<<<ceil_div(n, 256), 256, 0, s>>>(a, b, c, n);
  PCAONE_LAUNCH_CHECK();
}

void launch_to_f32(const double* a, float* b, int64_t n, cudaStream_t s) {
  if (n == 0) return;
  k_to_f32<<<ceil_div(n, 256), 256, 0, s>>>(a, b, n);
  PCAONE_LAUNCH_CHECK();
}

void launch_mult_small(const double* A, const double* B, double* C, int LP, cudaStream_t s, const int* only_if) {
  static bool attr_set = false;
  if (!attr_set) {
    PCAONE_CUDA(cudaFuncSetAttribute(k_mult_small, cudaFuncAttributeMaxDynamicSharedMemorySize, 210 * 1024));
    attr_set = true;
  }
  k_mult_small<<<1, 512, sizeof(double) * 2 * LP * LP, s>>>(A, B, C, LP, only_if);
  PCAONE_LAUNCH_CHECK();
}

void launch_usv_small(const double* Rinv, const double* Wh, int L, int LP, int k, double* UB, double* sigma,
                      double* T, double* tmp, int* status, cudaStream_t s) {
  static bool attr_set = false;
  if (!attr_set) {
    PCAONE_CUDA(cudaFuncSetAttribute(k_usv_small, cudaFuncAttributeMaxDynamicSharedMemorySize, 210 * 1024));
    attr_set = true;
  }
  k_usv_small<<<1, 1024, sizeof(double) * 2 * L * L, s>>>(Rinv, Wh, L, LP, k, UB, sigma, T, tmp, status);
  PCAONE_LAUNCH_CHECK();
}

void launch_mev(const double* X, const double* Y, int64_t rows, int k, double* out, double* W, double* part,
                int nblocks, cudaStream_t s) {
  launch_cross(X, k, k, Y, k, k, rows, 0, W, k, part, nblocks, s);
  k_mev_finish<<<1, 128, 0, s>>>(W, k, out);
  PCAONE_LAUNCH_CHECK();
}

void launch_subspace_change(const double* X, const double* Y, int64_t rows, int k, int n, double* M, double* R,
                            double* W, double* part, int nblocks, cudaStream_t s) {
  launch_cross(X, k, n, Y, k, n, rows, 0, M, n, part, nblocks, s, true);
  k_subspace_residual<<<ceil_div(rows * n, 256), 256, 0, s>>>(X, Y, k, n, M, rows, R);
  PCAONE_LAUNCH_CHECK();
  launch_cross(R, n, n, R, n, n, rows, 1, W, n, part, nblocks, s, true);
}

void launch_copy_if(const double* src, double* dst, int64_t n, const int* only_if, cudaStream_t s) {
  k_copy_if<<<ceil_div(n, 256), 256, 0, s>>>(src, dst, n, only_if);
  PCAONE_LAUNCH_CHECK();
}

void launch_em_fill(const int32_t* epos, const int32_t* sample, double* value, int64_t nnz, const int32_t* perm,
                    const double* F, const double* U, const double* S, const double* V, int k, cudaStream_t s) {
  if (nnz == 0) return;
  k_em_fill<<<ceil_div(nnz, 256), 256, 0, s>>>(epos, sample, value, nnz, perm, F, U, S, V, k);
  PCAONE_LAUNCH_CHECK();
}

int matvec_splits(int64_t nsnps, int nsamples) {
  const int xt = ceil_div(nsamples, 256);
  int sp = std::max(1, 1216 / std::max(1, xt));
  return (int)std::min<int64_t>(sp, std::max<int64_t>(1, nsnps));
}

void launch_matvec(const BedView& v, const double* F, const double* scale, const double* x, double* t,
                   double* y, double* ypart, int nsplit, cudaStream_t s) {
  k_matvec_t<<<ceil_div(v.nsnps * 32, 256), 256, 0, s>>>(v, F, scale, x, t);
  PCAONE_LAUNCH_CHECK();
  const int64_t per = (v.nsnps + nsplit - 1) / nsplit;
  dim3 grid(ceil_div(v.nsamples, 256), nsplit);
  k_matvec_y<<<grid, 256, 0, s>>>(v, F, scale, t, per, ypart);
  PCAONE_LAUNCH_CHECK();
  k_matvec_reduce<<<ceil_div(v.nsamples, 256), 256, 0, s>>>(ypart, nsplit, v.nsamples, y);
  PCAONE_LAUNCH_CHECK();
}

}  // namespace pcaone
