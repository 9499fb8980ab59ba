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
  int nsnp;               // SNPs in the window
  int LP;                 // padded sketch width (multiple of 16, <= 112)
  int nslice;             // BF16 slices of W (1..3)
  int chunk;              // samples per CTA (multiple of 64)
  int npad;               // padded sample count
  int nchunks;            // gridDim.y
  int mask;               // form the missing-mask product too
  int nstages;            // pipeline depth
  int tmem_cols;          // TMEM columns allocated per CTA
  const double* wscale;   // S x LP units of the W slices
  const int32_t* counts;  // per SNP (n00, n01, n10, n11)
  const int32_t* perm;    // position -> SNP (counts lookup); nullptr = identity
  float* part_d;          // [nchunks][nsnp][LP]
  float* part_m;          // [nchunks][nsnp][LP] (mask)
  int* err;               // set to 1 when a bounded wait gave up
};

// H += X_w^T * Gh (+ M^T * Gm) for one SNP window
struct HArgs {
  int64_t pos0;
  int nsnp;
  int LP;
  int nslice;
  int per_split;          // SNPs per CTA along K (multiple of 64)
  int nsplit;             // gridDim.y
  int npad;               // gridDim.x * 128
  int mask;
  int nstages;
  int tmem_cols;
  const double* hscale;   // (mask ? 2 : 1) * S x LP units of the Gh / Gm slices
  float* hpart;           // [nsplit][npad][LP]
  int* err;
};

struct GFinishArgs {
  int64_t pos0;
  int nsnp;
  int L, LP, nslice, nchunks, mask;
  int ldg;                       // columns of the Gh/Gm operand (window length rounded up to 64)
  const float* part_d;
  const float* part_m;           // nullptr when no mask product
  const double* colsum;          // column sums of the sliced W
  const double* F;
  const double* scale;
  const int32_t* perm;
  const double* omg;             // FP64 Omega (EM sparse term)
  SparseRows sp;
  double* G;                     // nsnps x LP (FP64)
  double* gh;                    // nsnp x LP (FP64) Gh of the window
  __nv_bfloat16* gt;             // (2*nslice*LP) x ldg, K-major B operand of the H product
  double* cpart;                 // nsnp x LP partial terms of c
};

void make_map_2d(CUtensorMap* map, const void* base, bool bf16, uint64_t inner, uint64_t outer, uint64_t pitch_bytes,
                 uint32_t box_inner, uint32_t box_outer, bool swizzle128);
// pipeline stages: shared memory holds bparts B slice groups, TMEM acc_parts accumulator groups
int stages_for(int LP, int nslice, int bparts, int acc_parts, bool mask, int pbytes);
int tmem_cols_for(int ncols);
int tmem_cols_needed(int LP, int nslice, int bparts, bool mask, int nstages);
void launch_g(const CUtensorMap& map_bed, const CUtensorMap& map_w, const GArgs& a, cudaStream_t s);
void launch_h(const CUtensorMap& map_bed, const CUtensorMap& map_g, const HArgs& a, cudaStream_t s);
void launch_omega_slices(const double* omg, int npad, int N, int LP, int S, __nv_bfloat16* w, double* wunit,
                         double* colsum, int* E, double* rep, cudaStream_t s);
void launch_g_finish(const GFinishArgs& a, int* Eh, double* hunit, double* c_out, cudaStream_t s);
void launch_h_finish(int nsamples, int npad, int L, int LP, const float* hpart, int nsplit, const double* c,
                     double* Hx, cudaStream_t s);
void launch_gather_rows(const uint8_t* src, uint8_t* dst, int64_t stride, const int32_t* perm, int64_t nrows,
                        cudaStream_t s);

}  // namespace tc
}  // namespace pcaone
