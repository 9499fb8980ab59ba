// Internal declarations shared by the CUDA translation units of the library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

namespace pcaone {

// Error carried from any layer to the C-ABI, which turns it into a status code.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define PCAONE_CUDA(call)                                                                   \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      throw ::pcaone::Error(e_ == cudaErrorMemoryAllocation ? -3 : -2,                      \
                            std::string(#call) + ": " + cudaGetErrorString(e_));            \
  } while (0)

// every kernel launch of the library is followed by this check, which also
// counts the launch (pcaone_gpu_launch_count)
extern unsigned long long g_kernel_launches;
#define PCAONE_LAUNCH_CHECK()      \
  do {                             \
    ++::pcaone::g_kernel_launches; \
    PCAONE_CUDA(cudaGetLastError()); \
  } while (0)

constexpr int kMaxL = 112;  // sketch width limit (Jacobi state in shared memory)

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }
inline int64_t round_up64(int64_t x, int64_t m) { return (x + m - 1) / m * m; }
inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// ---------------------------------------------------------------------------
// Genotype data resident in HBM
//   bed     : nsnps rows of `stride` bytes (row j = SNP j of the .bed, 2-bit
//             lanes, sample i at bits 2*(i%4) of byte i/4).  stride is a
//             multiple of 16; lanes at and beyond nsamples hold code 00.
//   counts  : nsnps x 4 int32 (n00, n01, n10, n11)
//   F       : nsnps doubles (allele frequency of A1)
// ---------------------------------------------------------------------------
// Error-free FP32 accumulation of products (a "double-float" pair hi + lo).
// FP64 arithmetic runs at a small fraction of the FP32 rate on this GPU, so
// long sums of products in the sparse missing-entry terms use FP32 pairs:
// a * b = p + pe exactly (TwoProduct via fmaf), hi + p = s + se exactly
// (TwoSum, Knuth), and the error terms gather in lo.  The result hi + lo
// carries about 48 significand bits.  The _rn intrinsics keep the compiler
// from contracting the steps into fused operations, which would break the
// error-free identities.
struct FloatPair {
  float hi = 0.f, lo = 0.f;
};
__device__ __forceinline__ void fp_add_prod(FloatPair& acc, float a, float b) {
  const float p = __fmul_rn(a, b);
  const float pe = fmaf(a, b, -p);
  const float s = __fadd_rn(acc.hi, p);
  const float bv = __fsub_rn(s, acc.hi);
  const float se = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bv)), __fsub_rn(p, bv));
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(se, pe));
}
// acc += a * b with a = ah + al and b = bh + bl given as float pairs: the
// product of the high parts exactly (TwoProduct), the cross terms rounded
// (al * bl, below 2^-48 relative, is dropped)
__device__ __forceinline__ void fp_add_prod2(FloatPair& acc, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  const float pe = fmaf(ah, bh, -p);
  const float cross = fmaf(ah, bl, fmaf(al, bh, pe));
  const float s = __fadd_rn(acc.hi, p);
  const float bv = __fsub_rn(s, acc.hi);
  const float se = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bv)), __fsub_rn(p, bv));
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(se, cross));
}
__device__ __forceinline__ double fp_value(const FloatPair& acc) { return (double)acc.hi + (double)acc.lo; }
// a double coefficient as hi + lo floats (hi = nearest float, lo = the rest)
__device__ __forceinline__ void fp_split(double c, float& hi, float& lo) {
  hi = (float)c;
  lo = (float)(c - (double)hi);
}

// Segmented gather of integer rows over a range of missing-genotype entries,
// in the order the entries are stored (k_seg_gather in util.cu):
//   out[key_e][l]  += R[src_e][l]
//   out2[key_e][l] += (rint(v_e * 2^24) * R2[src_e][l]) >> 8   (with values v_e)
// key_e = key[e] - key_base (the output row), src_e = src[e] - src_base (the
// source row); rows have LP entries, columns < L are summed.  The sums are
// int64 (two's complement in unsigned storage) and flushed with atomics, so
// they are exact and independent of the order of the flushes.  Entries with
// the same key must be contiguous for few flushes.
struct SegGatherArgs {
  int64_t e0, e1;
  const int32_t* key;
  int64_t key_base;
  const int32_t* src;
  int64_t src_base;
  int L, LP;
  const int32_t* R;
  unsigned long long* out;
  const double* val;  // nullptr: no value products
  const int32_t* R2;
  unsigned long long* out2;
};
constexpr double kSegValueScale = 16777216.0;  // v quantised to 2^-24
constexpr int kSegValueShift = 8;              // out2 is in units of 2^-16 of R2

struct BedView {
  const uint8_t* bed;
  int64_t stride;
  int64_t nsnps;
  int nsamples;
};

// bed.cu
void launch_sanitize_padding(uint8_t* bed, int64_t stride, int64_t nsnps, int nsamples, cudaStream_t s);
// nrows rows of bps bytes: src (pitch src_pitch) -> dst (pitch dst_pitch)
void launch_repitch(const uint8_t* src, int64_t src_pitch, uint8_t* dst, int64_t dst_pitch, int64_t nrows, int64_t bps,
                    cudaStream_t s);
void launch_counts(const BedView& v, int32_t* counts, double* F, cudaStream_t s);
// PLINK 2 hard calls (ALT counts, 3 = missing) -> PLINK 1 codes (A1 = ALT), in
// place over nbytes bytes
void launch_genovec_to_bed(uint8_t* bytes, int64_t nbytes, cudaStream_t s);
// rows perm[0 .. nrows) (identity when perm is null) of src into consecutive
// rows of dst, many 16-byte loads in flight per thread (sources across the
// host link); ctas thread blocks of 256
void launch_gather_rows_deep(const uint8_t* src, uint8_t* dst, int64_t stride, const int32_t* perm, int64_t nrows,
                             int ctas, cudaStream_t s);
// per-SNP decode table: lut[j] = {x(00), x(01), x(10), x(11)} with x(c) =
// scale_j * (BED2GENO[c] - F_j), x(01) = 0; lut64 likewise in double.
void launch_lut(const double* F, int64_t nsnps, int standardize, int ploidy, float4* lut32, double* lut64,
                double* scale, cudaStream_t s);
// synthetic genotypes (counter-based hash); see synthetic.py for the model
void launch_synth(uint8_t* bed, int64_t stride, int64_t snp0, int64_t nsnps, int nsamples, int npop,
                  const double* freq, const double* weights, const double* miss_sample,
                  const double* miss_snp, uint64_t seed, cudaStream_t s);

// window products, FP32 SIMT form (prod_simt.cu)
struct WindowArgs {
  BedView v;
  const int32_t* perm;   // position -> SNP (nullptr: identity)
  const float4* lut;     // per SNP
  int64_t pos0;          // first position of the window
  int nsnp;              // SNPs in the window
  int LP;                // padded sketch width (multiple of 8, <= 112)
  int npad;              // padded samples (multiple of 128)
};
// part[c][j][l] = sum over samples of chunk c of x(sample, pos0+j) * omg32[sample][l]
int window_g_chunks(const WindowArgs& a);
void launch_window_g(const WindowArgs& a, const float* omg32, float* part, int nchunks, cudaStream_t s);
// G[pos0+j][l] = sum_c part[c][j][l] (+ sparse missing-value term), g32 = float(G rows)
struct SparseRows {    // missing entries of the window in CSR by position
  const int64_t* rowptr;  // nsnps+1 (global positions)
  const int32_t* sample;  // entry -> sample
  const double* value;    // entry -> value in the centred scale (EM fill)
  const double* scale;    // per SNP scale (1 when not standardised)
  const int32_t* perm;    // position -> SNP
  int active;
};
void launch_window_g_finish(const WindowArgs& a, const float* part, int nchunks, const SparseRows& sp,
                            const double* omg, double* G, float* g32, cudaStream_t s);
// hpart[c][i][l] = sum over SNPs of split c of x(i, pos0+j) * g32[j][l]
int window_h_splits(const WindowArgs& a);
void launch_window_h(const WindowArgs& a, const float* g32, float* hpart, int nsplit, cudaStream_t s);
// Hx[i][l] += sum_c hpart[c][i][l], rows < nsamples (the EM term is added by
// launch_h_buckets)
void launch_window_h_finish(const WindowArgs& a, const float* hpart, int nsplit, double* Hx, cudaStream_t s);

// dense FP64 helpers (dense64.cu); tall matrices are row-major with ld = LP
int cross_blocks(int64_t rows);
size_t cross_smem(int na, int nb, int sym);
// W[i][j] (ld ldw) = sum_r A[r][i] * B[r][j], i < na, j < nb; sym: B = A
// f64 (here and below): plain FP64 arithmetic instead of FP32 pairs (the
// FP64-grade form)
// only_if (here and below): a device flag; when given and 0 the kernels do
// nothing (work decided on the device without a host round trip)
void launch_cross(const double* A, int lda, int na, const double* B, int ldb, int nb, int64_t rows, int sym,
                  double* W, int ldw, double* part, int nblocks, cudaStream_t s, bool f64 = false,
                  const int* only_if = nullptr);
// Cholesky of W (leading L block) -> R (upper), Rinv; padding = identity.  A
// failure ORs 1 into *status; with retry_rows >= 0 a failed factor is retaken
// with the shift of shifted CholeskyQR3 for a tall matrix of that many rows,
// and *shifted (when given) records whether it was
void launch_chol_inv(const double* W, int L, int LP, double* R, double* Rinv, int* status, cudaStream_t s,
                     bool f64 = false, int64_t retry_rows = -1, int* shifted = nullptr, const int* only_if = nullptr);
// C (rows x n, ld ldc) = A (rows x LP) * B (LP x n, ld ldb); C may alias A
void launch_gemm_tall(const double* A, int64_t rows, int LP, const double* B, int ldb, int n, double* C, int ldc,
                      cudaStream_t s, bool f64 = false);
// A <- A * B in place for B upper triangular (LP x LP, LP a multiple of 8)
void launch_gemm_tall_upper(double* A, int64_t rows, int LP, const double* B, cudaStream_t s, bool f64 = false,
                            const int* only_if = nullptr);
// Q columns times the signs an Eigen / LAPACK Householder QR gives
void launch_house_signs(double* Q, int64_t rows, int L, int LP, double* sgn, cudaStream_t s);
int flip_blocks(int64_t rows);
void launch_flip_omg(double* omg2, double* omg, int64_t rows, int L, int LP, double* part, double* sgn,
                     cudaStream_t s);
void launch_add(const double* a, const double* b, double* c, int64_t n, cudaStream_t s);
// dst = src (n doubles) when *only_if != 0
void launch_copy_if(const double* src, double* dst, int64_t n, const int* only_if, cudaStream_t s);
void launch_to_f32(const double* a, float* b, int64_t n, cudaStream_t s);
void launch_mult_small(const double* A, const double* B, double* C, int LP, cudaStream_t s,
                       const int* only_if = nullptr);
void launch_usv_small(const double* Rinv, const double* Wh, int L, int LP, int k, double* UB, double* sigma,
                      double* T, double* tmp, int* status, cudaStream_t s);
// W = R^T R with R = Y_n - X_n (X_n^T Y_n), the leading n columns of the
// orthonormal blocks X, Y (rows x k, ld k): the largest eigenvalue of W is the
// squared sine of the largest principal angle between span(X_n) and
// span(Y_n).  M (n x n) and R (rows x n) are scratch; FP64 throughout.
void launch_subspace_change(const double* X, const double* Y, int64_t rows, int k, int n, double* M, double* R,
                            double* W, double* part, int nblocks, cudaStream_t s);
void launch_mev(const double* X, const double* Y, int64_t rows, int k, double* out, double* W, double* part,
                int nblocks, cudaStream_t s);
void launch_em_fill(const int32_t* epos, const int32_t* sample, double* value, int64_t nnz, const int32_t* perm,
                    const double* F, const double* U, const double* S, const double* V, int k, cudaStream_t s);
int matvec_splits(int64_t nsnps, int nsamples);
void launch_matvec(const BedView& v, const double* F, const double* scale, const double* x, double* t, double* y,
                   double* ypart, int nsplit, cudaStream_t s);

// misc (util.cu)
void launch_missing_list(const BedView& v, const int32_t* perm, const int64_t* rowptr, int32_t* epos,
                         int32_t* sample, cudaStream_t s);
// missing genotypes grouped by (window of wsize positions, sample): counts, then
// positions / samples at the exclusive-scan offsets ptr (nwin * N + 1)
void launch_bucket_count(const BedView& v, const int32_t* perm, int64_t wsize, int nwin, int32_t* cnt,
                         cudaStream_t s);
// exclusive prefix sum of n int32 counts: out[0..n], out[n] = total;
// tile_sums holds scan_tiles_needed(n) values of scratch
void launch_exclusive_scan(const int32_t* in, int64_t n, int64_t* out, long long* tile_sums, cudaStream_t s);
int64_t scan_tiles_needed(int64_t n);
void launch_bucket_fill(const BedView& v, const int32_t* perm, int64_t wsize, int nwin, const int64_t* ptr,
                        int32_t* bpos, int32_t* bsample, cudaStream_t s);
// Hx[i] += the FP32-form EM term of window win: sum over the sample's missing
// positions p of s_p v_e G32[p - rbase] (G32 = the window's FP32 G rows)
void launch_h_buckets(int64_t win, int N, int L, int LP, const int64_t* ptr, const int32_t* bpos, const double* bval,
                      const int32_t* perm, const double* scale, const float* Rf, int64_t rbase, double* Hx,
                      cudaStream_t s);
void launch_seg_gather(const SegGatherArgs& a, cudaStream_t s);
// synthetic continuous dosages of SNPs [snp0, snp0 + nsnps) into out (nsnps x nsamples float32)
void launch_synth_dense(float* out, int64_t snp0, int64_t nsnps, int nsamples, int npop, const double* freq,
                        const double* weights, double sd, uint64_t seed, cudaStream_t s);
// dense rows: float32 -> FP16 rows of npad values (bytes at dst) and the exact row means
void launch_dense_rows(const float* src, int64_t nrows, int N, int npad, uint8_t* dst, double* mean, cudaStream_t s);
// projection of samples onto a fit (project.cu)
int project_max_k();
void launch_project_rhs(const BedView& v, const double* lut64, const double* B, int k, int npad, double* part,
                        int nsplit, double* R, cudaStream_t s);
void launch_project_solve(const double* K, const double* B, int k, const int64_t* ptr, const int32_t* pos,
                          const double* R, int N, double* X, cudaStream_t s);
void launch_flip_uv(double* U, int64_t nrows_u, double* V, int64_t nrows_v, int k, int* flag, cudaStream_t s);
void launch_transpose_out(const double* A, int64_t rows, int lda, int cols, double* out, cudaStream_t s);

}  // namespace pcaone
