/*
 * pcaone_gpu.h -- C-ABI of the GB300 randomized-SVD hot path.
 *
 * The library replaces, for the PLINK path (in core, or out of core with the
 * rows in host memory) and FileBinary input, the reference's
 * RSVD operator interface (class RsvdOpData, src/Halko.hpp:6-42) and the data
 * it reads (class Data / FileBed, src/Data.hpp:9-59, src/FilePlink.hpp:7-47).
 * Every entry point takes plain pointers and sizes, returns 0 on success or a
 * negative PCAONE_E* code, and keeps the message of the last failure for
 * pcaone_gpu_last_error().  Matrices crossing the boundary are column-major
 * doubles, the layout of the reference's Eigen Mat2D.
 *
 * One context drives one GPU from one host thread; contexts are not
 * thread-safe.  All device memory belongs to the context.
 */
#ifndef PCAONE_GPU_H_
#define PCAONE_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PCAONE_GPU_ABI_VERSION 1

/* status codes */
#define PCAONE_OK 0
#define PCAONE_E_ARG -1       /* invalid argument or call order */
#define PCAONE_E_CUDA -2      /* CUDA runtime error */
#define PCAONE_E_NOMEM -3     /* device allocation failed */
#define PCAONE_E_FORMAT -4    /* malformed input (e.g. bad .bed magic) */
#define PCAONE_E_NUMERIC -5   /* numerical breakdown (non-SPD Gram, NaN) */
#define PCAONE_E_LIMIT -6     /* size beyond a documented limit */

/* precision of the block products G = X*Omega and H = X^T*G */
#define PCAONE_PREC_FP32 0    /* FP32 SIMT products, FP64 window sums */
#define PCAONE_PREC_BF16 1    /* tcgen05 tensor-core products: exact BF16 dosages; the test
                                 matrix and G split per column into three integer BF16 slices
                                 (27 bits), exact integer accumulation in TMEM, slices combined
                                 exactly in int64, FP64 epilogue; missing genotypes as an exact
                                 sparse term */
#define PCAONE_PREC_FP8 2     /* FP8 form: the range-finding epochs run tcgen05 kind::f8f6f4 products on
                                 E4M3 operands (exact dosages; the test matrix and G as two base-16
                                 integer digits, an 8-bit integer per entry, exact integer
                                 accumulation); the final epochs run the 27-bit BF16 form: at least two,
                                 and more (up to 16 beyond maxp) until the leading PCs separated by a
                                 relative eigen-gap above 5% move by less than 1e-7 (sine of the largest
                                 principal angle) between two exact epochs.  PLINK input;
                                 computeGandH alone runs E4M3 epochs */
#define PCAONE_PREC_BF16X3 3  /* same as PCAONE_PREC_BF16 */
#define PCAONE_PREC_FP64 4    /* FP64-grade form for checking the other forms (no counterpart in the
                                 reference): the tensor-core form with six slices (54 bits per column:
                                 at least the FP64 significand relative to each column's maximum),
                                 slices combined in FP64, CholeskyQR and the small SVD in plain FP64;
                                 the missing-genotype terms keep 27-bit integers.  PLINK input,
                                 k + oversamples <= 80 */

/* SVD method (Param::svd_t, src/Cmd.hpp:14) */
#define PCAONE_SVD_SINGLE 1   /* NormalRsvdOpData: single-pass RSVD, -d 1 */
#define PCAONE_SVD_WINDOW 2   /* FancyRsvdOpData: window-based winSVD, -d 2 */

/* Largest supported sketch width k + oversamples. */
#define PCAONE_MAX_L 112

typedef struct pcaone_gpu_ctx pcaone_gpu_ctx;

typedef struct {
  int device;   /* CUDA device ordinal */
  int verbose;  /* 0 silent, 1 per-epoch lines on stderr like the reference's log */
} pcaone_gpu_desc;

/* The subset of Param (src/Cmd.hpp:16-98) the RSVD path reads.  Callers apply
 * the CLI's derived settings themselves, as Param::Param does
 * (src/Cmd.cpp:216 oversamples >= k, :228-232 maxiter, :238 perm). */
typedef struct {
  int svd;          /* PCAONE_SVD_SINGLE or PCAONE_SVD_WINDOW */
  int k;            /* number of PCs */
  int oversamples;  /* p; sketch width L = k + p <= PCAONE_MAX_L */
  int maxp;         /* maximum power iterations (epochs - 1) */
  int bands;        /* winSVD windows, power of two >= 4 (-w) */
  int seed;         /* random-matrix seed (--seed) */
  int rand;         /* 1 Gaussian, 0 uniform(-1,1) test matrix (--rand) */
  int perm;         /* shuffle SNP columns before winSVD (true for -d 2 without -S) */
  int emu;          /* EM imputation of missing genotypes (--emu) */
  int maxiter;      /* EM iterations (--maxiter) */
  double tol;       /* RSVD tolerance (--tol-rsvd) */
  double tolem;     /* EM tolerance (--tol-em) */
  int ploidy;       /* 2 for diploid (standardisation sqrt(ploidy)/sd) */
  int standardize;  /* 1: per-SNP genetic standardisation (scale == -9) */
  int precision;    /* PCAONE_PREC_* */
} pcaone_gpu_params;

/* Learned warm start of the EM imputation (no reference counterpart; it
 * replaces only the mean-fill start of run_pca_with_halko's EM loop,
 * src/Halko.cpp:290-320).  After the first, mean-imputed computeUSV a small
 * MLP (64 -> 256 -> 256 -> 1, BF16 weights, FP32 accumulation, Adam) is
 * trained on the GPU on randomly drawn observed genotypes and fills every
 * missing genotype; EM then iterates from that fill exactly as without it.
 * Inputs of entry (SNP s, sample i): the 32 flanking SNP dosages of sample i
 * in file order, the sample's top-q scores, the SNP's top-q loadings, its
 * allele frequency and the sample's and SNP's missing fractions
 * (q = min(k, 14)). */
typedef struct {
  int enable;           /* 1: use the learned start when emu is set */
  int train_entries;    /* observed genotypes drawn for training */
  int holdout_entries;  /* further observed genotypes for the held-out error */
  int epochs;           /* passes over the training genotypes */
  int batch;            /* minibatch size */
  float lr;             /* Adam step size */
  uint64_t seed;        /* draws and initial weights */
} pcaone_gpu_mlp_params;

/* Number of FP32 parameters of the network (W1 64x256, b1, W2 256x256, b2,
 * w3 256, b3 in this order; W row = input). */
#define PCAONE_MLP_PARAMS 82689
#define PCAONE_MLP_INPUTS 64

/* Fills p with the defaults (enabled, 524288 training and 65536 held-out
 * genotypes, 4 epochs, batch 4096, lr 1e-3). */
void pcaone_gpu_mlp_default_params(pcaone_gpu_mlp_params* p);

/* Fills p with the reference's defaults (src/Cmd.hpp:29-95). */
void pcaone_gpu_default_params(pcaone_gpu_params* p);

/* ---- host-side random streams (no GPU, no context) ----------------------
 * The initial test matrix of RsvdOpData::initOmg (src/Halko.cpp:15-23,
 * StandardNormalRandom / UniformRandom of src/RSVD.hpp:20-59): rows x cols,
 * column-major, N(0,1) when gaussian (--rand 1) else U(-1,1), drawn with
 * std::default_random_engine seeded with `seed` -- the matrix pcaone_gpu_op_init
 * uses unless pcaone_gpu_set_omega replaced it. */
int pcaone_gpu_random_omega(int seed, int gaussian, uint64_t rows, uint32_t cols, double* out);
/* The in-core SNP shuffle of PCAone::permute_matrix (src/RSVD.hpp:61-70):
 * perm[i] = original SNP of working column i (std::shuffle of 0..n-1 with a
 * default-constructed engine), as pcaone_gpu_get_perm returns it. */
int pcaone_gpu_shuffle_order(uint64_t n, int32_t* perm);

/* ---- context ------------------------------------------------------------ */
int pcaone_gpu_open(const pcaone_gpu_desc* desc, pcaone_gpu_ctx** out);
int pcaone_gpu_close(pcaone_gpu_ctx* ctx);
const char* pcaone_gpu_last_error(const pcaone_gpu_ctx* ctx);
int pcaone_gpu_abi_version(void);
/* wall-clock split of the last run_halko/compute_usv call, seconds:
 * t[0] total, t[1] block products, t[2] QR/SVD, t[3] EM fill */
int pcaone_gpu_timings(const pcaone_gpu_ctx* ctx, double t[4]);

/* Instrumentation with no counterpart in the reference.  set_profiling(1)
 * records CUDA events on the context's stream around every launch of the
 * window-product kernels (class 0: G = X_w * Omega, class 1: H += X_w^T * G,
 * in the exact forms; classes 2 and 3: the same in the FP8 form's E4M3 epochs)
 * and resets the totals; kernel_stats returns per class the summed device
 * milliseconds, algorithmic flops (2 * N * SNPs * L per launch) and launches.
 * launch_count is the number of kernels the library has launched so far in
 * this process. */
int pcaone_gpu_set_profiling(pcaone_gpu_ctx* ctx, int on);
int pcaone_gpu_kernel_stats(pcaone_gpu_ctx* ctx, double ms[4], double flops[4], long long launches[4]);
unsigned long long pcaone_gpu_launch_count(void);
/* Test hook with no counterpart in the reference: the limit, in SM clock
 * cycles, of every pipeline wait in the tensor-core product kernels (0, the
 * default: about two seconds).  A wait that runs out makes its tile give up:
 * the tile waits (bounded) for its own copies and MMAs in flight, frees its
 * tensor memory and flags the error, and the call returns PCAONE_E_CUDA; the
 * context stays usable. */
int pcaone_gpu_set_wait_limit(pcaone_gpu_ctx* ctx, long long cycles);
/* No counterpart in the reference: how the G-shaped tensor-core products
 * (X_w * Omega, and X_w^T * G on the sample-major copy of the rows) are
 * launched.  0: one CTA per (row tile, K chunk) item; 1: only as many CTAs as
 * stay resident (two per SM where the plan pairs), each taking items in turn;
 * 2 (the default): 1 for the exact forms' products, 0 in the FP8 form's E4M3
 * epochs (the faster of the two for each on 200,000-sample windows).  Each
 * item accumulates the same MMAs in the same order in every form, so results
 * are identical bit for bit. */
int pcaone_gpu_set_product_form(pcaone_gpu_ctx* ctx, int form);

/* ---- data: replaces FileBed::read_all (src/FilePlink.cpp:26-120) --------- */
/* packed: the .bed body after the 3 magic bytes, nsnps rows of (nsamples+3)/4
 * bytes in SNP-major order (host memory; copied to HBM). */
int pcaone_gpu_load_bed(pcaone_gpu_ctx* ctx, const uint8_t* packed, uint64_t nsnps, uint32_t nsamples);
/* Same, from a whole .bed file image including its 3 magic bytes; checks the
 * magic like src/FilePlink.hpp:24-27 and the size like FilePlink.cpp:125-126. */
int pcaone_gpu_load_bed_file_image(pcaone_gpu_ctx* ctx, const uint8_t* image, uint64_t image_bytes,
                                   uint64_t nsnps, uint32_t nsamples);
/* Dense input: the FileBinary matrix (FileBin, src/FileBinary.hpp:7-40,
 * src/FileBinary.cpp:54-64): values of nsnps rows x nsamples (host float32,
 * row by SNP), held on the device as FP16 (the storage of imputed dosages;
 * values that are not FP16 numbers are rounded to the nearest one) and
 * centred per SNP by the mean of the stored values.  The reference runs this
 * input with -C 0 (no standardisation).  Dense input runs in the tensor-core
 * form, without EM; pcaone_gpu_counts, pcaone_gpu_get_bed and the matvec
 * return PCAONE_E_ARG for it. */
int pcaone_gpu_load_dense(pcaone_gpu_ctx* ctx, const float* values, uint64_t nsnps, uint32_t nsamples);
/* Same from the bytes of a FileBinary file: uint32 SNPs, uint32 samples, then
 * the float32 rows (values 4-byte aligned in memory). */
int pcaone_gpu_load_binary_file_image(pcaone_gpu_ctx* ctx, const uint8_t* image, uint64_t image_bytes);
/* Test and benchmark input: continuous dosages (allele count plus N(0, sd^2)
 * noise, clipped to [0, 2], as FP16) of the seeded model of
 * pcaone_gb300/synthetic.py (sample_dosages), generated on the device (host
 * arrays freq nsnps x npop, weights nsamples x npop). */
int pcaone_gpu_load_synthetic_dense(pcaone_gpu_ctx* ctx, uint64_t nsnps, uint32_t nsamples, int npop,
                                    const double* freq, const double* weights, double sd, uint64_t seed);
/* Same, from device memory already holding the packed rows (row pitch
 * src_pitch bytes). */
int pcaone_gpu_load_bed_device(pcaone_gpu_ctx* ctx, const void* dev_packed, uint64_t src_pitch,
                               uint64_t nsnps, uint32_t nsamples);
/* Per-SNP genotype counts (nsnps x 4 int32, row-major: n00 two A1 copies,
 * n01 missing, n10 heterozygous, n11 no A1 copy) and allele frequency F
 * (FilePlink.cpp:37-55, bit-exact).  Either pointer may be NULL. */
int pcaone_gpu_counts(pcaone_gpu_ctx* ctx, int32_t* counts, double* F);

/* Test and benchmark utility with no counterpart in the reference: fills the
 * context's genotype matrix on the device from the seeded Balding-Nichols
 * model of pcaone_gb300/synthetic.py (host arrays: freq nsnps x npop and
 * weights nsamples x npop row-major, miss_sample nsamples, miss_snp nsnps),
 * then counts like the load functions.  Bytes equal the numpy generator's. */
int pcaone_gpu_load_synthetic(pcaone_gpu_ctx* ctx, uint64_t nsnps, uint32_t nsamples, int npop,
                              const double* freq, const double* weights, const double* miss_sample,
                              const double* miss_snp, uint64_t seed);
/* Copies the resident packed genotypes back (nsnps rows of (nsamples+3)/4
 * bytes, the .bed body). */
int pcaone_gpu_get_bed(pcaone_gpu_ctx* ctx, uint8_t* packed);
/* --maf: Data::filter_snps_resize_F (src/Data.cpp:88-105), called by
 * FileBed / FilePgen::read_all (src/FilePlink.cpp:61, src/FilePgen.cpp:53).
 * Keeps the SNPs whose minor allele frequency min(F, 1 - F) exceeds maf, in
 * file order; the context then holds only those rows (counts, F, the shuffle
 * and the products see the filtered matrix; pcaone_gpu_op_init again before
 * a run).  0 < maf < 0.5 (src/Cmd.cpp:222); genotype input held in HBM only
 * (the reference has no filter out of core, src/Cmd.cpp:223, nor for
 * FileBinary input).  No SNP left: PCAONE_E_ARG.  nkept (may be NULL): the
 * new SNP count. */
int pcaone_gpu_filter_maf(pcaone_gpu_ctx* ctx, double maf, uint64_t* nkept);
/* Data::keepSNPs (src/Data.hpp:56): for each resident SNP its row in the
 * loaded file, composed over repeated filters (idx: nsnps entries); the
 * identity when no filter was applied since the load. */
int pcaone_gpu_kept_snps(pcaone_gpu_ctx* ctx, int64_t* idx);

/* ---- PLINK2 input: replaces FilePgen (src/FilePgen.hpp, FilePgen.cpp:27-86) -
 * Hard calls only: ALT allele counts 0/1/2 (3 = missing), the values FilePgen
 * takes from pgenlib's ReadHardcalls, dosage v / 2 (FilePgen.cpp:16-21); they
 * become PLINK 1 codes with A1 = ALT on the device, so counts, allele
 * frequencies and every product equal those of the same genotypes in a .bed.
 * The reference uses .pgen dosages when the file has them unless --hardcall
 * is given; this library reads hard calls in both cases.
 *
 * genovecs: nsnps rows of hard calls, 2 bits per sample (the layout of
 * pgenlib's genovec, sample i in bits 2(i%4) of byte i/4), row_pitch bytes
 * apart (>= ceil(nsamples/4); 0 = packed). */
int pcaone_gpu_load_pgen_genovecs(pcaone_gpu_ctx* ctx, const uint8_t* genovecs, uint64_t row_pitch, uint64_t nsnps,
                                  uint32_t nsamples);
/* A whole .pgen file image in a storage mode this library reads itself:
 * 0x01 (PLINK 1 variant-major rows; nsamples from the .psam), or the
 * fixed-width 0x02 / 0x03 / 0x04 (12-byte header with the variant and sample
 * counts, nsamples from the .psam checked against it when nonzero).
 * Variable-width (compressed) files return PCAONE_E_FORMAT: pgenlib decodes
 * those on the host, for pcaone_gpu_load_pgen_genovecs. */
int pcaone_gpu_load_pgen_file_image(pcaone_gpu_ctx* ctx, const uint8_t* image, uint64_t image_bytes,
                                    uint32_t nsamples);
/* The layout pcaone_gpu_load_pgen_file_image reads (no GPU needed): storage
 * mode, counts, offset of the first record and bytes per record. */
int pcaone_gpu_pgen_layout(const uint8_t* image, uint64_t image_bytes, uint32_t nsamples, int* mode, uint64_t* nsnps,
                           uint32_t* nsamples_out, uint64_t* offset, uint64_t* record_bytes);

/* ---- out-of-core: replaces the -m/--memory path ---------------------------
 * FileBed::read_block_initial (src/FilePlink.cpp:122-218) with the block plan
 * of Data::prepare (src/Data.cpp:40-84) and the block loops of computeGandH
 * (src/Halko.cpp:130-153, 227-268).  The packed rows stay in host memory: the
 * library keeps a pinned copy in its device row layout (nsnps x
 * ceil(nsamples/128)*32 bytes), and each SNP block the window products need is
 * copied into one of two device slots while the previous block's products run
 * (in the shuffled order of the window method, a kernel gathers the block's
 * rows over the host link).  device_budget bounds the two slots in bytes (0:
 * no bound).  Without the window method's shuffle, results are bit-identical
 * to those of the in-core load with the same parameters (the single-pass
 * method's blocks are the in-core ones unless the budget asks for smaller).  Everything else reads the host copy directly
 * (counts, missing-entry index, FP32 form, matvec, warm start).  Arguments and
 * checks as pcaone_gpu_load_bed / _file_image.
 * The window method's shuffle takes, as the reference's out-of-core mode
 * does (src/Main.cpp:120-130), the order in which permute_plink rewrites the
 * .bed (src/FilePlink.cpp:303-408; pcaone_gpu_ooc_order) instead of the
 * in-core std::shuffle order; buffer_gb is its --buffer (0: 2, the
 * reference's default); a kernel then gathers each window's rows over the
 * host link, where unshuffled windows are one host-to-device copy each. */
int pcaone_gpu_load_bed_stream(pcaone_gpu_ctx* ctx, const uint8_t* packed, uint64_t nsnps, uint32_t nsamples,
                               uint64_t device_budget, uint32_t buffer_gb);
int pcaone_gpu_load_bed_file_image_stream(pcaone_gpu_ctx* ctx, const uint8_t* image, uint64_t image_bytes,
                                          uint64_t nsnps, uint32_t nsamples, uint64_t device_budget,
                                          uint32_t buffer_gb);
/* The out-of-core SNP order alone (no GPU needed): order[p] is the .bed row at
 * working position p after permute_plink with --buffer buffer_gb (0: 2) and
 * bands windows.  PCAONE_E_ARG when a buffer holds fewer SNPs than windows. */
int pcaone_gpu_ooc_order(uint64_t nsnps, uint32_t nsamples, int bands, uint32_t buffer_gb, int32_t* order);
/* The block plan alone (no GPU needed): SNPs per streamed block and the number
 * of blocks for svd (PCAONE_SVD_*) and bands.  The window method streams its
 * windows of ceil(nsnps/bands) SNPs, which two slots must hold (the reference
 * cuts a window into bandFactor blocks instead, Data.cpp:66-77); the
 * single-pass method uses blocks of at most 16384 SNPs, fewer when the budget
 * asks, balanced.  PCAONE_E_LIMIT when the budget holds fewer than two blocks. */
int pcaone_gpu_stream_plan(uint64_t nsnps, uint32_t nsamples, int svd, int bands, uint64_t device_budget,
                           uint64_t* block_snps, uint64_t* nblocks);
/* Whether the loaded rows are streamed, and the bytes copied into the device
 * slots since the previous call (which resets the count). */
int pcaone_gpu_stream_info(pcaone_gpu_ctx* ctx, int* streamed, double* bytes_fetched);

/* ---- operator: replaces RsvdOpData and subclasses (src/Halko.hpp) ------- */
/* Constructor of Normal/FancyRsvdOpData: draws Omega (initOmg, Halko.cpp:15-23). */
int pcaone_gpu_op_init(pcaone_gpu_ctx* ctx, const pcaone_gpu_params* params);
/* Replace the initial random matrix (N x L column-major) by the caller's own
 * draw; this and every later op_init / initOmg use it until the data is
 * reloaded or omega is NULL (which restores the library's draw).  May be
 * called before or after pcaone_gpu_op_init. */
int pcaone_gpu_set_omega(pcaone_gpu_ctx* ctx, const double* omega, uint32_t rows, uint32_t cols);
/* RsvdOpData::setFlags (Halko.hpp:32-35). */
int pcaone_gpu_set_flags(pcaone_gpu_ctx* ctx, int update, int standardize);
/* computeGandH (Halko.cpp:99-269, in-core branches): one epoch pi.  G (M x L)
 * and H (N x L) are copied out when non-NULL. */
int pcaone_gpu_compute_g_and_h(pcaone_gpu_ctx* ctx, int pi, double* G, double* H);
/* RsvdOpData::computeUSV (Halko.cpp:46-97): epochs until convergence.
 * U (N x k), S (k), V (M x k, rows in the working SNP order) when non-NULL. */
int pcaone_gpu_compute_usv(pcaone_gpu_ctx* ctx, int p, double tol, double* U, double* S, double* V,
                           int* epochs);
/* run_pca_with_halko (Halko.cpp:271-320, non-LD PLINK path) including the EM
 * loop; outputs like compute_usv, em_iters may be NULL. */
int pcaone_gpu_run_halko(pcaone_gpu_ctx* ctx, const pcaone_gpu_params* params, double* U, double* S,
                         double* V, int* em_iters);
/* The working SNP order: perm[i] = original SNP of column i (Data::perm,
 * src/Data.hpp:49); identity when no shuffle was applied. */
int pcaone_gpu_get_perm(pcaone_gpu_ctx* ctx, int32_t* perm);

/* Projection of the loaded samples (a PLINK fileset with the fit's SNPs) onto
 * a fit: run_projection --project 1 / 2 (src/Projection.cpp:236-247,
 * solve_projection_scores :159-178).  The genotypes are decoded, centred and
 * standardised (ploidy 2) with the fit's allele frequencies F (nsnps; the
 * reference reads them from the .mbim, src/Data.cpp:17-32); V is the fit's
 * loadings (nsnps x k, column-major, file order, as in .loadings) and S its
 * singular values.  mode 1: U = X V S^-1 (missing genotypes at the mean);
 * mode 2: per sample the least-squares solution of (V S) x = g over its
 * observed SNPs (NaN for a sample whose system is singular).  U: nsamples x k
 * column-major.  k <= 32. */
int pcaone_gpu_project(pcaone_gpu_ctx* ctx, const double* F, const double* V, const double* S, int k, int mode,
                       double* U);

/* Learned warm start for the next pcaone_gpu_run_halko calls with emu set
 * (NULL or enable = 0: plain mean-fill EM). */
int pcaone_gpu_set_warm_start(pcaone_gpu_ctx* ctx, const pcaone_gpu_mlp_params* p);
/* Statistics of the last learned start: [0] mean squared error of the last
 * training epoch, [1] held-out mean squared error of the MLP, [2] held-out
 * mean squared error of the mean fill, [3] training seconds, [4] seconds to
 * fill the missing genotypes, [5] missing genotypes filled (both orderings).
 * Errors are on the centred scale d/2 - f. */
int pcaone_gpu_mlp_stats(pcaone_gpu_ctx* ctx, double out[6]);
/* One forward and backward pass of the network on caller data, for checks:
 * X (B x 64, row-major), y (B) targets, params (PCAONE_MLP_PARAMS FP32
 * values; the forward pass uses their BF16 rounding).  Writes out (B), the
 * mean squared error *loss and grads (PCAONE_MLP_PARAMS, the gradient of the
 * loss with respect to the rounded weights and the biases). */
int pcaone_gpu_mlp_forward_backward(int device, const float* X, const float* y, int B, const float* params,
                                    float* out, float* loss, float* grads);

/* ---- Arnoldi matvec: replaces ArnoldiOpData::perform_op (Arnoldi.cpp:18-46) */
/* y = X X^T x over the loaded genotypes (X samples x SNPs, centred, scaled by
 * sqrt(ploidy)/sd when standardize != 0, the ploidy of the last
 * pcaone_gpu_op_init or 2), x and y of length N. */
int pcaone_gpu_matvec(pcaone_gpu_ctx* ctx, const double* x, double* y, int standardize);

/* ---- matvec without device allocation (no counterpart in the reference) --
 * y = X X^T x like pcaone_gpu_matvec, for callers that cannot call cudaMalloc
 * (a host whose own allocator or memory arena owns all device memory, or a
 * loop that cannot afford an allocation's implicit synchronisation).  All
 * pointers are device pointers the caller owns: d_packed holds nsnps rows of
 * row_pitch bytes (the .bed body, row_pitch >= (nsamples+3)/4), d_F the allele
 * frequencies (pcaone_gpu_counts), d_x and d_y nsamples doubles; the work is
 * queued on `stream` (a cudaStream_t, NULL for the default stream) and is
 * complete when that stream is.  The intermediate X^T x lives in a static
 * device array of 2^21 doubles (16 MiB, held by every GPU that loads the
 * library until the process exits), so nsnps is limited to 2,097,152:
 * larger inputs return PCAONE_E_LIMIT.  The first call on a device resolves
 * the array's device address (cudaGetSymbolAddress); make that first call
 * before any stream capture.  Calls share the array: calls whose work overlaps
 * on the GPU race and must be serialised by the caller.  The scale is the
 * diploid one, sqrt(2)/sd (standardize != 0).  The cached address belongs to
 * the device's primary context: callers on another driver context, or after a
 * cudaDeviceReset, are not supported. */
int pcaone_gpu_matvec_static(const uint8_t* d_packed, uint64_t row_pitch, uint64_t nsnps, uint32_t nsamples,
                             const double* d_F, int standardize, const double* d_x, double* d_y, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PCAONE_GPU_H_ */
