// Tensor-core (tcgen05) window products: argument blocks and launchers.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include "internal.cuh"

namespace pcaone {
namespace tc {

// G = X_w * W for one SNP window (see prod_tc.cu)
struct GArgs {
  int64_t pos0;           // first position of the window (row of the packed matrix)
  int64_t kofs;           // K elements before the first of this product in the operand's rows (0 for G;
                          // the window's column offset when the kernel runs an H product on the
                          // sample-major copy)
  int nsnp;               // SNPs in the window
  int LP;                 // padded sketch width (multiple of 16, <= 112)
  int nslice;             // BF16 slices of W (1..3)
  int chunk;              // samples per CTA (multiple of 64)
  int npad;               // padded sample count
  int nchunks;            // gridDim.y
  int nstages;            // pipeline depth
  int tmem_cols;          // TMEM columns allocated per CTA
  const double* wscale;   // S x LP units of the W slices (dense input)
  void* part;             // [nchunks][nsnp][LP]: int64 slice combinations (genotypes; FP64 beyond
                          // kIntSlices slices) or FP32 sums (dense)
  int* err;               // set to 1 when a bounded wait gave up
  int dense;              // 1: FP16 values (FileBinary input) instead of packed codes
  long long wait_cycles;  // limit of the pipeline waits in SM cycles (0: about 2 s)
  int fp8;                // 1: E4M3 operands (128 samples per pipeline stage)
  int persist;            // 1: as many CTAs as stay resident, each taking (tile, chunk) items in
                          // turn; 0: one CTA per item.  The partial sums are the same.
};

// Sample-major copy of the packed rows for the H products (k_tc_g then runs
// H on it): block w of every sample row holds window w's codes, ldw positions
// per block (a multiple of 128), tpitch bytes per sample row.
void launch_transpose_codes(const uint8_t* bed, int64_t stride, int64_t M, int64_t ws, int64_t ldw, int nwin,
                            int npad, uint8_t* bt, int64_t tpitch, cudaStream_t s);

// H += X_w^T * Gh for one SNP window (dosage part; k_tc_h_finish adds the
// missing-entry sums gathered by k_seg_gather)
struct HArgs {
  int64_t pos0;
  int nsnp;
  int L;
  int LP;
  int nslice;
  int per_split;          // SNPs per CTA along K (multiple of 64)
  int nsplit;             // gridDim.y
  int npad;               // gridDim.x * 128
  int nstages;
  int tmem_cols;
  const double* hscale;   // S x LP units of the Gh slices (dense input)
  void* hpart;            // [nsplit][npad][LP]: as GArgs::part
  int* err;
  int dense;              // 1: FP16 values instead of packed codes
  long long wait_cycles;  // as GArgs::wait_cycles
  int fp8;                // 1: E4M3 operands (128 SNPs per pipeline stage)
};

// H rows of one window: Hx += sum of the split partials + missing-entry terms - c
struct HFinishArgs {
  int nsamples, npad, L, LP, nsplit, dense;
  int nslice;
  const void* hpart;          // as HArgs::hpart
  const double* c;            // LP centring terms
  double* Hx;
  const double* hunit_m;      // per column unit of the Gh integers of the sparse terms
  const double* hunit_p;      // per column unit of the partials (the last slice unit)
  unsigned long long* hisum;  // npad x LP int64 sums of Gm over missing entries (nullptr: none), cleared
  unsigned long long* hesum;  // npad x LP int64 EM product sums (nullptr: no EM), cleared
};

struct GFinishArgs {
  double vfac;                   // 1/2 for dosages (x = s (d/2 - f)), 1 for dense values (x = v - mu)
  int64_t pos0;
  int nsnp;
  int L, LP, nslice, nchunks;
  int fmt, digit_bits;           // operand format of the slices (kFmt*) and their digit width
  int ldg;                       // columns of the Gh operand (window length rounded up to 64)
  const void* part;              // chunk partials of D W (int64 for genotypes; FP64 with more than
                                 // kIntSlices slices; FP32 for dense input)
  const double* colsum;          // column sums of the sliced W
  const double* F;
  const double* scale;
  const int32_t* perm;
  const double* wunit_m;         // per column unit of the integer W of the sparse terms
  const double* wunit_p;         // per column unit of the partials (the last slice unit)
  unsigned long long* gisum;     // nsnp x LP int64 sums over missing entries (nullptr: none), cleared
  unsigned long long* gesum;     // nsnp x LP int64 EM product sums (nullptr: no EM), cleared
  double* G;                     // nsnps x LP (FP64)
  double* gh;                    // nsnp x LP (FP64): Gh of the window
  int32_t* ghint;                // nsnp x LP: Gh as represented by its slices, as integers
  int32_t* gmint;                // nsnp x LP: Gm = 2 f Gh represented as integers
  void* gt;                      // (nslice*LP) x ldg, K-major B operand of the H product (format fmt)
  double* cpart;                 // nsnp x LP partial terms of c
};

constexpr int kMapU8 = 0, kMapBF16 = 1, kMapF16 = 2;  // (E4M3 digits use kMapU8)
void make_map_2d(CUtensorMap* map, const void* base, int dtype, uint64_t inner, uint64_t outer, uint64_t pitch_bytes,
                 uint32_t box_inner, uint32_t box_outer, bool swizzle128);
// A tile bytes per pipeline stage of the G and H products
inline int g_tile_bytes(bool dense, bool fp8 = false) { return dense ? 128 * 128 : fp8 ? 128 * 32 : 128 * 16; }
inline int h_tile_bytes(bool dense, bool fp8 = false) { return dense ? 64 * 256 : fp8 ? 128 * 32 : 64 * 32; }
// pipeline stages within shared memory (B slices + packed tile per stage) and
// TMEM (nslice * LP accumulator columns + 32 A columns per stage)
int stages_for(int LP, int nslice, int pbytes, bool dense);
int tmem_cols_for(int ncols);
int tmem_cols_needed(int LP, int nslice, int nstages, bool dense);
// Slice digits: balanced base-512 integers, |w| <= 256, exact in BF16 and FP16.
// Three slices (27 bits) in the tensor-core form, six (54 bits, at least the
// FP64 significand relative to each column's maximum) in the FP64-grade form;
// the integers of the sparse missing-entry terms always carry kIntSlices
// slices (27 bits).
constexpr int kDigitBits = 9;
constexpr int kMaxSlices = 6;
constexpr int kIntSlices = 3;
// The FP8 form's slices: balanced base-16 digits, |w| <= 8, exact in E4M3
// (two slices: an 8-bit integer representation of each column).
constexpr int kDigitBits8 = 4;
// operand formats of the slice digits
constexpr int kFmtBF16 = 0, kFmtF16 = 1, kFmtE4M3 = 2;
inline __host__ __device__ int digit_bits_of(int fmt) { return fmt == kFmtE4M3 ? kDigitBits8 : kDigitBits; }
// Exact accumulation: a product d*w of a genotype dosage (<= 2) and a slice
// digit is at most 512 in magnitude, so a CTA that sums at most 2^14 K elements
// keeps every FP32 accumulator an exactly represented integer (|v| <= 2^23).
// Dense FP16 input rounds in FP32; its K per CTA stays at 4096.
constexpr int kMaxKExact = 16384;
constexpr int kMaxKDense = 4096;
// CTAs that run at once: two per SM when the TMEM plan pairs, else one
int cta_slots(int LP, int nslice, bool dense);
// number of parts to cut a K extent into (tiles CTAs per part): the fewest
// waves of `slots` CTAs times the per-CTA length plus a fixed cost, each part
// at most kmax long and a multiple of 64
int k_parts(int tiles, int K, int kmax, int slots);
void launch_g(const CUtensorMap& map_bed, const CUtensorMap& map_w, const GArgs& a, cudaStream_t s);
void launch_h(const CUtensorMap& map_bed, const CUtensorMap& map_g, const HArgs& a, cudaStream_t s);
// scratch of the multi-block column reductions: kColRedBlocks x LP partials and
// a completion counter that is zero between launches
constexpr int kColRedBlocks = 304;
struct ColRedScratch {
  double* part;
  unsigned* cnt;
};
void launch_omega_slices(const double* omg, int npad, int N, int LP, int S, void* w, double* wunit,
                         double* colsum, int* E, double* rep, int32_t* wint, int fmt, const ColRedScratch& cr,
                         cudaStream_t s);
// G finish, Gh slices and their units (hunit), Gm integers with their units
// (gmunit: S x LP, the last slice row is the unit of gmint), c
void launch_g_finish(const GFinishArgs& a, int* Eh, double* hunit, double* gmunit, double* c_out,
                     const ColRedScratch& cr, cudaStream_t s);
void launch_h_finish(const HFinishArgs& a, cudaStream_t s);
void launch_gather_rows(const uint8_t* src, uint8_t* dst, int64_t stride, const int32_t* perm, int64_t nrows,
                        cudaStream_t s);

}  // namespace tc
}  // namespace pcaone
