// Host side of the RSVD operator: the GPU counterparts of RsvdOpData,
// NormalRsvdOpData and FancyRsvdOpData (reference src/Halko.hpp, src/Halko.cpp)
// and of the Data/FileBed state they read, plus the C-ABI of include/pcaone_gpu.h.
//
// Layout in HBM (one context):
//   bed      nsnps x stride bytes, stride = npad/4 (npad = N rounded up to 128)
//   F        nsnps doubles, counts nsnps x 4 int32
//   Omega    npad x LP doubles (+ FP32 copy), rows >= N and columns >= L zero
//   H, H1, H2  npad x LP doubles;  G  nsnps x LP doubles (rows in working order)
//   U        npad x k, V nsnps x k (row-major), S k
// where L = k + oversamples and LP = L rounded up to 8.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/pcaone_gpu.h"
#include "internal.cuh"
#include "mlp.cuh"
#include "prod_tc.cuh"

namespace pcaone {

unsigned long long g_kernel_launches = 0;

void host_random_omega(int seed, int gaussian, int64_t rows, int64_t cols, double* out_colmajor);
void host_shuffle_columns(int64_t n, int32_t* out);

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  // (re)allocates when the size changes; contents are zeroed when `zero`
  void ensure(size_t count, cudaStream_t s, bool zero = true) {
    if (count == 0) count = 1;
    if (count != n) {
      release();
      PCAONE_CUDA(cudaMalloc(&p, count * sizeof(T)));
      n = count;
    }
    if (zero) PCAONE_CUDA(cudaMemsetAsync(p, 0, count * sizeof(T), s));
  }
};

using clk = std::chrono::steady_clock;
static double secs(clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); }

struct Context {
  int device = 0;
  int verbose = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  double t_total = 0, t_prod = 0, t_qr = 0, t_em = 0;

  // ---- data (Data / FileBed) ----
  int N = 0;
  int npad = 0;
  int64_t M = 0;
  int64_t stride = 0;
  bool have_data = false;
  // dense input (FileBinary values as FP16, rows of npad values): `bed` holds the
  // FP16 rows (stride = 2 npad bytes), F the per-SNP means
  bool dense = false;
  DBuf<uint8_t> bed;
  DBuf<int32_t> counts;
  DBuf<double> F;
  std::vector<int32_t> counts_host;  // filled lazily
  long long counts_total_missing = -1;

  // missing entries in working order (EM)
  int64_t nnz = -1;
  DBuf<int64_t> miss_rowptr;
  std::vector<int64_t> miss_rowptr_host;
  DBuf<int32_t> miss_pos, miss_sample;
  DBuf<double> miss_value;
  bool miss_valid = false;
  // the same entries grouped by (window, sample): bucket w*N + i lists, in
  // position order, the positions of window w (bk_wsize positions each) where
  // sample i is missing; bk_value holds their EM fill values
  int64_t bk_wsize = 0;
  int bk_nwin = 0;
  bool bk_valid = false;
  DBuf<int64_t> bk_ptr;
  std::vector<int64_t> bk_ptr_host;  // offsets at the window boundaries: bucket w*N for w = 0..nwin
  DBuf<int32_t> bk_cnt, bk_pos, bk_sample;
  DBuf<long long> bk_scan;  // tile sums of the offsets' prefix sum
  DBuf<double> bk_value;
  bool bk_stale = true;  // bk_value does not yet hold the current fill values

  // learned warm start of the EM imputation (mlp.cu)
  pcaone_gpu_mlp_params warm{};
  bool prefilled = false;  // the fill values come from the warm start; skip the next EM fit
  double warm_stats[6] = {0, 0, 0, 0, 0, 0};
  std::unique_ptr<mlp::Net> net;
  DBuf<int32_t> wpos, wsmp;
  DBuf<float> wX, wy, smiss;

  // ---- operator (RsvdOpData) ----
  bool have_op = false;
  pcaone_gpu_params P{};
  int L = 0, LP = 0, k = 0;
  bool update = false, standardize = false, scaled = false, fitted = false;
  std::vector<double> omega0;  // N x L column-major (host)
  std::vector<double> omega_user;  // caller-supplied initial matrix (pcaone_gpu_set_omega)
  int omega_user_rows = 0, omega_user_cols = 0;
  DBuf<double> Omg0, Omg, Omg2;
  DBuf<float> Omg32;
  DBuf<double> H, H1, H2, G;
  DBuf<float4> lut32;
  DBuf<double> scale;
  DBuf<int32_t> perm;
  bool permuted = false;
  std::vector<int32_t> perm_host;
  // file row of each resident SNP after a MAF filter (Data::keepSNPs,
  // src/Data.hpp:56); empty: no filter applied since the load
  std::vector<int64_t> kept;
  int bandsize = 1;
  int64_t blocksize = 0;
  // window scratch
  DBuf<float> part, hpart, g32;
  // tensor-core form: chunk and split partials (int64 slice combinations for
  // genotypes, FP32 for dense input)
  DBuf<long long> tpart, thpart;
  // small matrices and reductions
  DBuf<double> W, R1, R1i, R2, R2i, R3, R3i, Rt, Rti, UB, sigma, T, tmp, sgn, red, mevv;
  DBuf<int> status, flag;
  DBuf<double> U, Upre, V, Vpre;
  DBuf<double> rres;  // FP8 form: residual of the leading-PC change
  bool have_usv = false;
  DBuf<double> outbuf;
  DBuf<double> mv_t, mv_ypart, mv_x, mv_y, mv_scale;

  // tensor-core form (prod_tc.cu)
  bool tc = false;
  DBuf<uint8_t> bedp;                 // packed rows in working order (shuffled window method)
  // sample-major copy of the working-order rows, one block of bt_ldw
  // positions per window (tc::launch_transpose_codes): the H products run the
  // G kernel on it, whose tiles decode without transposes
  DBuf<uint8_t> bedT;
  bool bt_valid = false, bt_off = false;
  int64_t bt_ws = 0, bt_ldw = 0, bt_pitch = 0;
  CUtensorMap map_bt{}, map_bt8{};
  const uint8_t* bed_work = nullptr;  // packed rows the tensor-core kernels read
  DBuf<__nv_bfloat16> wsl, gt;        // W slices (3*LP x npad), Gh slices (3*LP x ldg)
  DBuf<double> colsum, cpart, cvec, wunit, hunit, ghbuf, wrep;
  DBuf<int32_t> wint, ghint, gmint;   // represented W, Gh and Gm = 2 f Gh as integers (times a column unit)
  DBuf<double> gmunit;                // units of the Gm integers (last of S rows)
  // int64 sums of the missing-entry terms (k_seg_gather), cleared by the finish kernels
  DBuf<unsigned long long> gisum, gesum, hisum, hesum;
  DBuf<int> wexp, hexp;
  DBuf<int> err;
  DBuf<double> cr_part;    // column-reduction partials (tc::kColRedBlocks x LP)
  DBuf<unsigned> cr_cnt;   // its completion counter, zero between launches
  CUtensorMap map_bed_g{}, map_bed_h{}, map_w{}, map_gt{};
  // the FP8 form's operands: 128-sample / 128-SNP packed tiles, E4M3 digit slices
  CUtensorMap map_bed_g8{}, map_bed_h8{}, map_w8{}, map_gt8{};
  int ldg = 0, win_max = 0;
  int nslice_cur = 1, w_slices = 0;
  int max_slices = 3;  // slices of the chosen form: 3, or 6 in the FP64-grade form
  bool fp8_form = false;  // PCAONE_PREC_FP8: E4M3 range-finding epochs, exact final epochs
  bool fp8_now = false;   // the current epoch runs the E4M3 products
  int w_mode = -1;        // slices and format of the W slices now held (S * 4 + format)
  long long wait_cycles = 0;  // limit of the tensor-core pipeline waits (0: the kernels' default)
  // launch form of the G-shaped products (pcaone_gpu_set_product_form):
  // 0 one CTA per (tile, chunk) item, 1 resident CTAs taking items in turn,
  // 2 resident CTAs except in the E4M3 epochs
  int product_form = 2;
  bool fp64 = false;   // FP64-grade form: the QR and small-SVD kernels in plain FP64 too

  // optional per-kernel CUDA-event timing of the window products
  // (pcaone_gpu_set_profiling): class 0 = G product, 1 = H product
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<int, size_t>> ev_marks;  // (class, index of the start event)
  std::vector<std::pair<int, double>> ev_work;   // (class, flops of the launch)
  // classes: 0 G product, 1 H product (exact forms), 2 G, 3 H (E4M3 epochs)
  double prof_ms[4] = {0, 0, 0, 0}, prof_flops[4] = {0, 0, 0, 0};
  long long prof_launches[4] = {0, 0, 0, 0};

  // Out-of-core streaming (load_bed_stream; FileBed::read_block_initial,
  // src/FilePlink.cpp:122-218): the packed rows stay in pinned host memory in
  // the device row layout, mapped into the device address space, where the
  // kernels that read the matrix once per call (counts, missing-entry index,
  // matvec, projection, the FP32 form's products) read them over the host
  // link.  The tensor-core window products read each SNP block from one of two
  // device slots, filled on fetch_stream while the previous block's products
  // run (block plan: stream_block_size).
  struct Slot {
    DBuf<uint8_t> buf;
    int64_t pos0 = -1, n = 0, rows = 0;  // block held (working positions), capacity in rows
    cudaEvent_t ready = nullptr;         // the fill of the block has landed
    cudaEvent_t idle = nullptr;          // the last product reading the slot has run
    CUtensorMap g{}, h{}, g8{}, h8{};
  };
  bool streamed = false;
  int sm_count = 152;
  uint8_t* hbed = nullptr;      // pinned host rows, M x stride bytes
  uint8_t* hbed_dev = nullptr;  // their device address
  size_t hbed_bytes = 0;
  uint64_t stream_budget = 0;   // device bytes for the two slots (0: no bound)
  unsigned stream_buffer_gb = 2;  // --buffer of the out-of-core shuffle (src/Cmd.hpp:52)
  Slot slots[2];
  int slot_cur = -1;
  cudaStream_t fetch_stream = nullptr;
  double stream_bytes = 0;      // bytes fetched into the slots since the last query
  const uint8_t* rows_ptr() const { return streamed ? hbed_dev : bed.p; }
  uint8_t* rows_mut() { return streamed ? hbed_dev : bed.p; }
  BedView view() const { return BedView{rows_ptr(), stride, M, N}; }
  void invalidate_slots() {
    for (auto& s : slots) s.pos0 = -1, s.n = 0;
    slot_cur = -1;
  }
  void free_host_rows() {
    if (fetch_stream) cudaStreamSynchronize(fetch_stream);
    if (hbed) cudaFreeHost(hbed);
    hbed = hbed_dev = nullptr;
    hbed_bytes = 0;
    for (auto& s : slots) s.buf.release();
    invalidate_slots();
  }

  // host loads (load_bed_host): a copy stream, two staging buffers and their
  // events; ev_free[2] marks where the context's stream stood when a load began
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_free[3] = {nullptr, nullptr, nullptr};
  DBuf<uint8_t> stage;
  // out-of-core loads: padded chunks go back to the pinned host copy on a
  // third stream (ev_ready: chunk prepared; ev_back: chunk copied back)
  cudaStream_t back_stream = nullptr;
  cudaEvent_t ev_ready[2] = {nullptr, nullptr}, ev_back[2] = {nullptr, nullptr};
  DBuf<uint8_t> stage2;
  void ensure_copy_stream() {
    if (!copy_stream) {
      PCAONE_CUDA(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
      PCAONE_CUDA(cudaStreamCreateWithFlags(&back_stream, cudaStreamNonBlocking));
      for (auto* e : {&ev_copied[0], &ev_copied[1], &ev_free[0], &ev_free[1], &ev_free[2], &ev_ready[0],
                      &ev_ready[1], &ev_back[0], &ev_back[1]})
        PCAONE_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    PCAONE_CUDA(cudaEventRecord(ev_free[2], stream));
  }

  cudaEvent_t next_event() {
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e;
      PCAONE_CUDA(cudaEventCreate(&e));
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }
  // folds recorded event pairs into the per-class totals (stream synchronised)
  void collect_events() {
    for (size_t q = 0; q < ev_marks.size(); ++q) {
      float ms = 0.f;
      PCAONE_CUDA(cudaEventElapsedTime(&ms, ev_pool[ev_marks[q].second], ev_pool[ev_marks[q].second + 1]));
      prof_ms[ev_marks[q].first] += ms;
      prof_flops[ev_work[q].first] += ev_work[q].second;
      prof_launches[ev_marks[q].first] += 1;
    }
    ev_marks.clear();
    ev_work.clear();
    ev_used = 0;
  }
  ~Context() {
    free_host_rows();
    for (auto& s : slots)
      for (auto e : {s.ready, s.idle})
        if (e) cudaEventDestroy(e);
    if (fetch_stream) cudaStreamDestroy(fetch_stream);
    for (auto e : ev_pool) cudaEventDestroy(e);
    if (copy_stream) {
      cudaStreamSynchronize(copy_stream);
      cudaStreamSynchronize(back_stream);
      cudaStreamDestroy(copy_stream);
      cudaStreamDestroy(back_stream);
      for (auto e : {ev_copied[0], ev_copied[1], ev_free[0], ev_free[1], ev_free[2], ev_ready[0], ev_ready[1],
                     ev_back[0], ev_back[1]})
        cudaEventDestroy(e);
    }
  }
};

// ------------------------------------------------------------------------
// data
// ------------------------------------------------------------------------
// bytes of one staging buffer of the host loads
constexpr size_t kStageBytes = (size_t)512 << 20;

static void load_common(Context& c, uint64_t nsnps, uint32_t nsamples, bool dense = false, bool stream = false) {
  if (nsamples == 0 || nsnps == 0) throw Error(PCAONE_E_ARG, "empty genotype matrix");
  if (nsnps > 0x7fffffffull) throw Error(PCAONE_E_LIMIT, "more than 2^31-1 SNPs");
  if (nsamples > 0x7fffff00u) throw Error(PCAONE_E_LIMIT, "too many samples");
  c.N = (int)nsamples;
  c.M = (int64_t)nsnps;
  c.npad = round_up(c.N, 128);
  c.dense = dense;
  c.stride = dense ? (int64_t)c.npad * 2 : c.npad / 4;
  c.invalidate_slots();
  c.stream_bytes = 0;
  c.bt_valid = false;
  if (stream) {
    // the rows go to pinned, mapped host memory; no device copy of the matrix
    c.bed.release();
    c.bedp.release();
    const size_t bytes = (size_t)c.M * c.stride;
    if (bytes != c.hbed_bytes) {
      c.free_host_rows();
      void* h = nullptr;
      if (cudaHostAlloc(&h, bytes, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) {
        cudaGetLastError();
        throw Error(PCAONE_E_NOMEM, "out-of-core load: cannot pin " + std::to_string(bytes) + " bytes of host memory");
      }
      c.hbed = static_cast<uint8_t*>(h);
      c.hbed_bytes = bytes;
      void* d = nullptr;
      PCAONE_CUDA(cudaHostGetDevicePointer(&d, h, 0));
      c.hbed_dev = static_cast<uint8_t*>(d);
    }
    c.streamed = true;
  } else {
    c.free_host_rows();
    c.streamed = false;
    c.bed.ensure((size_t)c.M * c.stride, c.stream, true);
  }
  c.counts.ensure((size_t)c.M * 4, c.stream, false);
  c.F.ensure((size_t)c.M, c.stream, false);
  c.have_data = false;
  c.have_op = false;
  c.omega_user.clear();
  c.miss_valid = false;
  c.bk_valid = false;
  c.nnz = -1;
  c.counts_host.clear();
  c.kept.clear();
  c.permuted = false;  // the rows are in file order until the next op_init shuffles them
}

static void finish_load(Context& c) {
  launch_sanitize_padding(c.rows_mut(), c.stride, c.M, c.N, c.stream);
  launch_counts(c.view(), c.counts.p, c.F.p, c.stream);
  c.counts_total_missing = -1;
  c.have_data = true;
}

static void ensure_missing_total(Context& c) {
  if (c.counts_total_missing >= 0) return;
  c.counts_host.resize((size_t)c.M * 4);
  PCAONE_CUDA(cudaMemcpyAsync(c.counts_host.data(), c.counts.p, c.counts_host.size() * sizeof(int32_t),
                              cudaMemcpyDeviceToHost, c.stream));
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  long long t = 0;
  for (int64_t j = 0; j < c.M; ++j) t += c.counts_host[(size_t)j * 4 + 1];
  c.counts_total_missing = t;
}

// The .bed body from host memory: contiguous chunks of whole rows are copied
// into two staging buffers on a second stream (large linear copies run at the
// host link's rate, where one pitched copy of short rows does not) while the
// context's stream re-pitches the previous chunk into the padded rows.
//
// Out-of-core (stream): the same pipeline with the re-pitch writing the padded
// rows into the pinned host copy through its device address.
static void load_rows_to_host_copy(Context& c, const uint8_t* packed, int64_t bps);

//
// PLINK 2 hard calls (hardcalls: rows of 2-bit ALT allele counts, 3 =
// missing, src_pitch bytes apart) are translated to PLINK 1 codes on the
// device before the re-pitch.
static void load_bed_host(Context& c, const uint8_t* packed, uint64_t nsnps, uint32_t nsamples, bool stream = false,
                          bool hardcalls = false, int64_t src_pitch = 0) {
  load_common(c, nsnps, nsamples, false, stream);
  const int64_t bps = ((int64_t)nsamples + 3) / 4;
  if (src_pitch == 0) src_pitch = bps;
  if (src_pitch < bps) throw Error(PCAONE_E_ARG, "row pitch shorter than a row");
  if (stream) {
    if (hardcalls || src_pitch != bps) throw Error(PCAONE_E_ARG, "the out-of-core load takes PLINK 1 rows");
    load_rows_to_host_copy(c, packed, bps);
    return;
  }
  if (bps == c.stride && src_pitch == bps) {
    PCAONE_CUDA(cudaMemcpyAsync(c.bed.p, packed, (size_t)c.M * bps, cudaMemcpyHostToDevice, c.stream));
    if (hardcalls) launch_genovec_to_bed(c.bed.p, c.M * bps, c.stream);
    finish_load(c);
    return;
  }
  c.ensure_copy_stream();
  const int64_t rows = std::max<int64_t>(1, std::min<int64_t>(c.M, (int64_t)(kStageBytes / bps)));
  c.stage.ensure((size_t)(2 * rows * bps), c.stream, false);
  for (int64_t j0 = 0, q = 0; j0 < c.M; j0 += rows, ++q) {
    const int b = (int)(q & 1);
    const int64_t n = std::min<int64_t>(rows, c.M - j0);
    uint8_t* buf = c.stage.p + (size_t)b * rows * bps;
    // the buffer is free once the re-pitch that last read it has run (for the
    // first two chunks: once the context's stream reached this load)
    PCAONE_CUDA(cudaStreamWaitEvent(c.copy_stream, q >= 2 ? c.ev_free[b] : c.ev_free[2], 0));
    if (src_pitch == bps)
      PCAONE_CUDA(cudaMemcpyAsync(buf, packed + (size_t)j0 * bps, (size_t)n * bps, cudaMemcpyHostToDevice,
                                  c.copy_stream));
    else
      PCAONE_CUDA(cudaMemcpy2DAsync(buf, (size_t)bps, packed + (size_t)j0 * src_pitch, (size_t)src_pitch, (size_t)bps,
                                    (size_t)n, cudaMemcpyHostToDevice, c.copy_stream));
    PCAONE_CUDA(cudaEventRecord(c.ev_copied[b], c.copy_stream));
    PCAONE_CUDA(cudaStreamWaitEvent(c.stream, c.ev_copied[b], 0));
    if (hardcalls) launch_genovec_to_bed(buf, n * bps, c.stream);
    launch_repitch(buf, bps, c.rows_mut() + (size_t)j0 * c.stride, c.stride, n, bps, c.stream);
    PCAONE_CUDA(cudaEventRecord(c.ev_free[b], c.stream));
  }
  finish_load(c);
}

// Out-of-core load: chunks of whole rows pass through the device (copied in,
// re-pitched into padded rows, padding bits cleared, counted) and go back to
// the pinned host copy; both copies run on copy engines, in opposite
// directions, while the context's stream prepares the previous chunk.
static void load_rows_to_host_copy(Context& c, const uint8_t* packed, int64_t bps) {
  c.ensure_copy_stream();
  const int64_t rows = std::max<int64_t>(1, std::min<int64_t>(c.M, (int64_t)(kStageBytes / c.stride)));
  c.stage.ensure((size_t)(2 * rows * bps), c.stream, false);
  c.stage2.ensure((size_t)(2 * rows * c.stride), c.stream, false);
  for (int64_t j0 = 0, q = 0; j0 < c.M; j0 += rows, ++q) {
    const int b = (int)(q & 1);
    const int64_t n = std::min<int64_t>(rows, c.M - j0);
    uint8_t* in = c.stage.p + (size_t)b * rows * bps;
    uint8_t* out = c.stage2.p + (size_t)b * rows * c.stride;
    // `in` is free once the chunk two back was re-pitched; `out` once it was copied back
    PCAONE_CUDA(cudaStreamWaitEvent(c.copy_stream, q >= 2 ? c.ev_ready[b] : c.ev_free[2], 0));
    PCAONE_CUDA(cudaMemcpyAsync(in, packed + (size_t)j0 * bps, (size_t)n * bps, cudaMemcpyHostToDevice,
                                c.copy_stream));
    PCAONE_CUDA(cudaEventRecord(c.ev_copied[b], c.copy_stream));
    PCAONE_CUDA(cudaStreamWaitEvent(c.stream, c.ev_copied[b], 0));
    if (q >= 2) PCAONE_CUDA(cudaStreamWaitEvent(c.stream, c.ev_back[b], 0));
    launch_repitch(in, bps, out, c.stride, n, bps, c.stream);
    launch_sanitize_padding(out, c.stride, n, c.N, c.stream);
    launch_counts(BedView{out, c.stride, n, c.N}, c.counts.p + (size_t)j0 * 4, c.F.p + j0, c.stream);
    PCAONE_CUDA(cudaEventRecord(c.ev_ready[b], c.stream));
    PCAONE_CUDA(cudaStreamWaitEvent(c.back_stream, c.ev_ready[b], 0));
    PCAONE_CUDA(cudaMemcpyAsync(c.hbed + (size_t)j0 * c.stride, out, (size_t)n * c.stride, cudaMemcpyDeviceToHost,
                                c.back_stream));
    PCAONE_CUDA(cudaEventRecord(c.ev_back[b], c.back_stream));
  }
  // readers of the host copy (the context's stream) start after the last copy back
  for (int b = 0; b < 2; ++b) PCAONE_CUDA(cudaStreamWaitEvent(c.stream, c.ev_back[b], 0));
  c.counts_total_missing = -1;
  c.have_data = true;
}

static void load_bed_device(Context& c, const void* src, uint64_t pitch, uint64_t nsnps, uint32_t nsamples) {
  load_common(c, nsnps, nsamples);
  const size_t bps = ((size_t)nsamples + 3) / 4;
  PCAONE_CUDA(cudaMemcpy2DAsync(c.bed.p, c.stride, src, pitch, bps, nsnps, cudaMemcpyDeviceToDevice, c.stream));
  finish_load(c);
}

// Data::filter_snps_resize_F (src/Data.cpp:88-105, MAF of src/Common.hpp:26):
// keep the SNPs whose minor allele frequency exceeds maf, in file order.  The
// kept rows are gathered into a new buffer and loaded from there, so that
// counts, F (the same bits, from the same rows), the missing-entry index and
// every later step see the filtered matrix, as in the reference, whose
// FileBed::read_all decodes only the kept SNPs (src/FilePlink.cpp:61-72).
static int64_t filter_maf(Context& c, double maf) {
  if (!(maf > 0 && maf < 0.5)) throw Error(PCAONE_E_ARG, "--maf has to be between (0, 0.5)");
  if (c.dense) throw Error(PCAONE_E_ARG, "no MAF filter for dense (FileBinary) input");
  if (c.streamed) throw Error(PCAONE_E_ARG, "does not support --maf filters for out-of-core mode");
  std::vector<double> F((size_t)c.M);
  PCAONE_CUDA(cudaMemcpyAsync(F.data(), c.F.p, F.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  std::vector<int32_t> keep;
  keep.reserve(F.size());
  for (int64_t j = 0; j < c.M; ++j) {
    const double f = F[(size_t)j];
    if ((f > 0.5 ? 1 - f : f) > maf) keep.push_back((int32_t)j);
  }
  const int64_t nk = (int64_t)keep.size();
  if (nk < 1) throw Error(PCAONE_E_ARG, "no SNPs left after filtering");
  std::vector<int64_t> prev = c.kept;
  std::vector<int64_t> kept((size_t)nk);
  for (int64_t i = 0; i < nk; ++i) kept[(size_t)i] = prev.empty() ? keep[(size_t)i] : prev[(size_t)keep[(size_t)i]];
  if (nk < c.M) {
    DBuf<uint8_t> rows;
    DBuf<int32_t> idx;
    rows.ensure((size_t)nk * c.stride, c.stream, false);
    idx.ensure((size_t)nk, c.stream, false);
    PCAONE_CUDA(cudaMemcpyAsync(idx.p, keep.data(), (size_t)nk * sizeof(int32_t), cudaMemcpyHostToDevice, c.stream));
    tc::launch_gather_rows(c.bed.p, rows.p, c.stride, idx.p, nk, c.stream);
    load_bed_device(c, rows.p, (uint64_t)c.stride, (uint64_t)nk, (uint32_t)c.N);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  }
  c.kept = std::move(kept);
  return nk;
}

static void load_synthetic(Context& c, uint64_t nsnps, uint32_t nsamples, int npop, const double* freq,
                           const double* weights, const double* miss_sample, const double* miss_snp,
                           uint64_t seed) {
  if (npop <= 0 || !freq || !weights || !miss_sample || !miss_snp) throw Error(PCAONE_E_ARG, "bad model arrays");
  load_common(c, nsnps, nsamples);
  DBuf<double> dw, dms, dfreq, dmsnp;
  dw.ensure((size_t)nsamples * npop, c.stream, false);
  dms.ensure(nsamples, c.stream, false);
  PCAONE_CUDA(cudaMemcpyAsync(dw.p, weights, (size_t)nsamples * npop * 8, cudaMemcpyHostToDevice, c.stream));
  PCAONE_CUDA(cudaMemcpyAsync(dms.p, miss_sample, (size_t)nsamples * 8, cudaMemcpyHostToDevice, c.stream));
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>((int64_t)nsnps, (1 << 26) / npop));
  dfreq.ensure((size_t)chunk * npop, c.stream, false);
  dmsnp.ensure((size_t)chunk, c.stream, false);
  for (int64_t j0 = 0; j0 < (int64_t)nsnps; j0 += chunk) {
    const int64_t n = std::min<int64_t>(chunk, (int64_t)nsnps - j0);
    PCAONE_CUDA(cudaMemcpyAsync(dfreq.p, freq + j0 * npop, (size_t)n * npop * 8, cudaMemcpyHostToDevice, c.stream));
    PCAONE_CUDA(cudaMemcpyAsync(dmsnp.p, miss_snp + j0, (size_t)n * 8, cudaMemcpyHostToDevice, c.stream));
    launch_synth(c.bed.p + j0 * c.stride, c.stride, j0, n, (int)nsamples, npop, dfreq.p, dw.p, dms.p, dmsnp.p,
                 seed, c.stream);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  }
  finish_load(c);
}

// FileBinary values (src/FileBinary.cpp:54-64): float32 SNP rows, held as FP16
// (the storage of imputed dosages); each SNP is centred by the mean of its
// stored values, computed exactly (int64 sums of value * 2^24).
static void load_dense(Context& c, const float* values, uint64_t nsnps, uint32_t nsamples) {
  if (!values) throw Error(PCAONE_E_ARG, "null values");
  load_common(c, nsnps, nsamples, true);
  c.counts_host.assign((size_t)c.M * 4, 0);
  c.counts_total_missing = 0;
  const int64_t rows_per = std::max<int64_t>(1, (int64_t)(64u << 20) / ((int64_t)nsamples * 4));
  DBuf<float> stage;
  stage.ensure((size_t)std::min<int64_t>(rows_per, c.M) * nsamples, c.stream, false);
  for (int64_t j0 = 0; j0 < c.M; j0 += rows_per) {
    const int64_t n = std::min<int64_t>(rows_per, c.M - j0);
    PCAONE_CUDA(cudaMemcpyAsync(stage.p, values + (size_t)j0 * nsamples, (size_t)n * nsamples * sizeof(float),
                                cudaMemcpyHostToDevice, c.stream));
    launch_dense_rows(stage.p, n, (int)nsamples, c.npad, c.bed.p + j0 * c.stride, c.F.p + j0, c.stream);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  }
  c.have_data = true;
}

// synthetic continuous dosages of the seeded model (pcaone_gb300/synthetic.py
// sample_dosages), generated on the device and held like load_dense
static void load_synthetic_dense(Context& c, uint64_t nsnps, uint32_t nsamples, int npop, const double* freq,
                                 const double* weights, double sd, uint64_t seed) {
  if (npop <= 0 || !freq || !weights || !(sd >= 0.0)) throw Error(PCAONE_E_ARG, "bad model arrays");
  load_common(c, nsnps, nsamples, true);
  c.counts_host.assign((size_t)c.M * 4, 0);
  c.counts_total_missing = 0;
  DBuf<double> dw, dfreq;
  DBuf<float> stage;
  dw.ensure((size_t)nsamples * npop, c.stream, false);
  PCAONE_CUDA(cudaMemcpyAsync(dw.p, weights, (size_t)nsamples * npop * 8, cudaMemcpyHostToDevice, c.stream));
  const int64_t chunk = std::max<int64_t>(1, (int64_t)(256u << 20) / ((int64_t)nsamples * 4));
  const int64_t rows = std::min<int64_t>(chunk, (int64_t)nsnps);
  dfreq.ensure((size_t)rows * npop, c.stream, false);
  stage.ensure((size_t)rows * nsamples, c.stream, false);
  for (int64_t j0 = 0; j0 < (int64_t)nsnps; j0 += chunk) {
    const int64_t n = std::min<int64_t>(chunk, (int64_t)nsnps - j0);
    PCAONE_CUDA(cudaMemcpyAsync(dfreq.p, freq + j0 * npop, (size_t)n * npop * 8, cudaMemcpyHostToDevice, c.stream));
    launch_synth_dense(stage.p, j0, n, (int)nsamples, npop, dfreq.p, dw.p, sd, seed, c.stream);
    launch_dense_rows(stage.p, n, (int)nsamples, c.npad, c.bed.p + j0 * c.stride, c.F.p + j0, c.stream);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  }
  c.have_data = true;
}

static void need_data(const Context& c) {
  if (!c.have_data) throw Error(PCAONE_E_ARG, "no genotype data loaded");
}
static void need_plink(const Context& c) {
  need_data(c);
  if (c.dense) throw Error(PCAONE_E_ARG, "not available for dense (FileBinary) input");
}
static void need_op(const Context& c) {
  need_data(c);
  if (!c.have_op) throw Error(PCAONE_E_ARG, "operator not initialised (pcaone_gpu_op_init)");
}

// ------------------------------------------------------------------------
// operator set-up (RsvdOpData ctor + initOmg, Halko.cpp:15-23)
// ------------------------------------------------------------------------
static void upload_omega0(Context& c) {
  std::vector<double> rowmajor((size_t)c.npad * c.LP, 0.0);
  for (int j = 0; j < c.L; ++j)
    for (int i = 0; i < c.N; ++i) rowmajor[(size_t)i * c.LP + j] = c.omega0[(size_t)j * c.N + i];
  PCAONE_CUDA(cudaMemcpyAsync(c.Omg0.p, rowmajor.data(), rowmajor.size() * sizeof(double), cudaMemcpyHostToDevice,
                              c.stream));
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
}

// TMA descriptors of the packed rows (or FP16 rows) the tensor-core products
// read: `rows` rows from `base` (the whole matrix, or a streaming slot)
static void make_bed_maps(const Context& c, const uint8_t* base, int64_t rows, CUtensorMap& g, CUtensorMap& h,
                          CUtensorMap& g8, CUtensorMap& h8) {
  if (c.dense) {
    // FP16 rows: G tiles of 64 samples x 128 SNPs (128-byte swizzle), H tiles
    // of 128 samples x 64 SNPs
    tc::make_map_2d(&g, base, tc::kMapF16, (uint64_t)c.npad, (uint64_t)rows, (uint64_t)c.stride, 64, 128, true);
    tc::make_map_2d(&h, base, tc::kMapF16, (uint64_t)c.npad, (uint64_t)rows, (uint64_t)c.stride, 128, 64, false);
    return;
  }
  tc::make_map_2d(&g, base, tc::kMapU8, (uint64_t)c.stride, (uint64_t)rows, (uint64_t)c.stride, 16, 128, false);
  tc::make_map_2d(&h, base, tc::kMapU8, (uint64_t)c.stride, (uint64_t)rows, (uint64_t)c.stride, 32, 64, false);
  // E4M3 form: 128 samples (32 bytes) per G stage, 128 SNP rows per H stage
  tc::make_map_2d(&g8, base, tc::kMapU8, (uint64_t)c.stride, (uint64_t)rows, (uint64_t)c.stride, 32, 128, false);
  tc::make_map_2d(&h8, base, tc::kMapU8, (uint64_t)c.stride, (uint64_t)rows, (uint64_t)c.stride, 32, 128, false);
}

static void tc_make_bed_maps(Context& c) {
  make_bed_maps(c, c.bed_work, c.M, c.map_bed_g, c.map_bed_h, c.map_bed_g8, c.map_bed_h8);
}

// launch shapes of one window's tensor-core products: G tiles of 128 SNPs x
// chunks of samples, H tiles of 128 samples x splits of the window's SNPs.
// Genotypes (exact integer accumulation, K per CTA <= kMaxKExact): the fewest
// waves of long CTAs (tc::k_parts).  Dense FP16 input accumulates in FP32, so
// its error grows with K per CTA: at least 304 CTAs of at most 4096.
static void tc_shapes(const Context& c, int win, int S, bool fp8, int& chunk, int& nchunks, int& per_split,
                      int& nsplit) {
  const int gran = fp8 ? 128 : 64;  // K elements per pipeline stage
  if (c.dense) {
    const int xt = ceil_div(win, 128), xh = c.npad / 128;
    chunk = std::min(round_up(ceil_div(c.npad, std::max(1, ceil_div(304, xt))), 64), tc::kMaxKDense);
    per_split = std::min(round_up(ceil_div(win, std::max(1, ceil_div(304, xh))), 64), tc::kMaxKDense);
  } else {
    const int slots = tc::cta_slots(c.LP, S, false);
    const int nch = tc::k_parts(ceil_div(win, 128), c.npad, tc::kMaxKExact, slots);
    chunk = round_up(ceil_div(c.npad, nch), gran);
    const int nsp = tc::k_parts(c.npad / 128, win, tc::kMaxKExact, slots);
    per_split = round_up(ceil_div(win, nsp), gran);
  }
  nchunks = ceil_div(c.npad, chunk);
  nsplit = ceil_div(win, per_split);
}

// Out-of-core block plan (Data::prepare, src/Data.cpp:40-84): SNPs per block
// when two device slots of stride-byte rows share `budget` bytes (0: no
// bound).  The window method streams its own windows (ceil(M / bands) SNPs,
// the blocks the products use in core too), which two slots must hold: the
// reference instead cuts each window into bandFactor blocks (Data.cpp:66-77),
// which the products here do not need.  The single-pass method uses the in-core
// blocks of at most 16384 SNPs, smaller when the budget asks, balanced over
// the blocks.  Returns 0 when the budget cannot hold two blocks.
int64_t stream_block_size(int64_t M, int64_t stride, int svd, int bands, uint64_t budget) {
  if (M <= 0 || stride <= 0) return 0;
  const uint64_t per_slot = budget / 2;
  if (svd == PCAONE_SVD_WINDOW) {
    if (bands <= 0) return 0;
    const int64_t win = (M + bands - 1) / bands;
    return budget == 0 || (uint64_t)win * (uint64_t)stride <= per_slot ? win : 0;
  }
  int64_t cap = 16384;
  if (budget) cap = std::min<int64_t>(cap, (int64_t)(per_slot / (uint64_t)stride));
  if (cap <= 0) return 0;
  const int64_t nblk = (M + cap - 1) / cap;
  return (M + nblk - 1) / nblk;
}

// The SNP order of the reference's out-of-core window method, whose
// permute_plink (src/FilePlink.cpp:303-408) rewrites the .bed before the run:
// the file is read in buffers of per_buf consecutive SNPs (as many as
// buffer_gb GiB of rows hold, cut to a multiple of the bands), and band b takes
// from each buffer the SNPs at offsets b, b + bands, b + 2 bands, ...; in the
// rewritten file band b starts where ceil(M / bands)-SNP bands would (the
// first M mod bands bands) or hold one SNP fewer, and buffer i's share of a
// band sits at i * (per_buf / bands) within it.  A last, shorter buffer gives
// its first (count mod bands) bands one SNP more than the others.
// order[p] = the file row at working position p.  Returns false when a buffer
// holds fewer SNPs than there are bands.
bool host_ooc_order(int64_t M, int64_t bps, unsigned buffer_gb, int bands, int32_t* order) {
  int64_t per_buf = (int64_t)std::floor(1073741824.0 * (double)buffer_gb / (double)bps);
  per_buf = std::min(per_buf, M);
  const int64_t per_band0 = per_buf / bands;
  if (per_band0 == 0) return false;
  per_buf = per_band0 * bands;
  const int64_t big = (M + bands - 1) / bands, rem = M % bands;
  const int64_t nbuf = (M + per_buf - 1) / per_buf, tail = M % per_buf;
  for (int64_t i = 0; i < nbuf; ++i) {
    const bool short_buf = i == nbuf - 1 && tail != 0;
    const int64_t per_band = short_buf ? (tail + bands - 1) / bands : per_band0;
    const int64_t full_bands = short_buf ? tail % bands : 0;  // 0: every band takes per_band
    for (int64_t b = 0; b < bands; ++b) {
      const int64_t start = rem == 0 || b < rem ? b * big : rem * big + (big - 1) * (b - rem);
      const int64_t nj = full_bands != 0 && b >= full_bands ? per_band - 1 : per_band;
      for (int64_t j = 0; j < nj; ++j) order[start + i * per_band0 + j] = (int32_t)(i * per_buf + j * bands + b);
    }
  }
  return true;
}

// positions per SNP window of the current operator: the winSVD band blocks
// (src/Halko.cpp:169-172) or the sSVD blocks of at most 16384 SNPs (the
// out-of-core block plan when the rows are streamed)
static int64_t window_size(const Context& c) {
  if (c.streamed) return stream_block_size(c.M, c.stride, c.P.svd, c.P.bands, c.stream_budget);
  if (c.P.svd == PCAONE_SVD_WINDOW) return (c.M + c.P.bands - 1) / c.P.bands;
  const int64_t nwin = (c.M + 16383) / 16384;
  return (c.M + nwin - 1) / nwin;
}

// two device slots of `rows` packed rows, their events and TMA descriptors
static void setup_slots(Context& c, int64_t rows) {
  if (c.fetch_stream) PCAONE_CUDA(cudaStreamSynchronize(c.fetch_stream));  // no fill in flight into a slot
  if (!c.fetch_stream) {
    int lo = 0, hi = 0;
    PCAONE_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    PCAONE_CUDA(cudaStreamCreateWithPriority(&c.fetch_stream, cudaStreamNonBlocking, hi));
  }
  for (auto& sl : c.slots) {
    if (!sl.ready) PCAONE_CUDA(cudaEventCreateWithFlags(&sl.ready, cudaEventDisableTiming));
    if (!sl.idle) PCAONE_CUDA(cudaEventCreateWithFlags(&sl.idle, cudaEventDisableTiming));
    sl.buf.ensure((size_t)rows * c.stride, c.stream, false);
    sl.rows = rows;
    make_bed_maps(c, sl.buf.p, rows, sl.g, sl.h, sl.g8, sl.h8);
    PCAONE_CUDA(cudaEventRecord(sl.idle, c.stream));
  }
  c.invalidate_slots();
}

static void tc_setup(Context& c, int win, const std::vector<int64_t>& lens) {
  const int LP = c.LP;
  c.win_max = win;
  c.ldg = round_up(win, 64);
  size_t need_part = 1, need_hpart = 1;
  for (int64_t n : lens) {
    if (n <= 0) continue;
    for (int S = 1; S <= c.max_slices; ++S) {
      for (int f8 = 0; f8 < 2; ++f8) {
        int ch, nch, per, nsp;
        tc_shapes(c, (int)n, S, f8 != 0, ch, nch, per, nsp);
        need_part = std::max(need_part, (size_t)nch * n * LP);
        need_hpart = std::max(need_hpart, (size_t)nsp * c.npad * LP);
      }
    }
  }
  const int smax = c.max_slices;
  c.wsl.ensure((size_t)smax * LP * c.npad, c.stream);
  c.gt.ensure((size_t)smax * LP * c.ldg, c.stream);
  c.colsum.ensure(LP, c.stream);
  c.cvec.ensure(LP, c.stream);
  c.cpart.ensure((size_t)win * LP, c.stream, false);
  c.ghbuf.ensure((size_t)win * LP, c.stream, false);
  c.wrep.ensure((size_t)c.npad * LP, c.stream, false);
  c.wint.ensure((size_t)c.npad * LP, c.stream, false);
  c.ghint.ensure((size_t)win * LP, c.stream, false);
  c.gmint.ensure((size_t)win * LP, c.stream, false);
  c.gmunit.ensure((size_t)smax * LP, c.stream);
  c.gisum.ensure((size_t)win * LP, c.stream, true);
  c.gesum.ensure((size_t)win * LP, c.stream, true);
  c.hisum.ensure((size_t)c.npad * LP, c.stream, true);
  c.hesum.ensure((size_t)c.npad * LP, c.stream, true);
  c.wunit.ensure((size_t)smax * LP, c.stream);
  c.hunit.ensure((size_t)smax * LP, c.stream);
  c.wexp.ensure(LP, c.stream);
  c.hexp.ensure(LP, c.stream);
  c.err.ensure(1, c.stream);
  c.cr_part.ensure((size_t)tc::kColRedBlocks * LP, c.stream, false);
  c.cr_cnt.ensure(1, c.stream, true);
  c.tpart.ensure(need_part, c.stream, false);
  c.thpart.ensure(need_hpart, c.stream, false);
  if (c.streamed) {
    c.bed_work = nullptr;
    setup_slots(c, win);
  } else {
    c.bed_work = c.bed.p;
    tc_make_bed_maps(c);
  }
  const int sl = c.dense ? tc::kMapF16 : tc::kMapBF16;  // slice digits: FP16 for dense input, else BF16
  tc::make_map_2d(&c.map_w, c.wsl.p, sl, (uint64_t)c.npad, (uint64_t)smax * LP, (uint64_t)c.npad * 2, 64, LP, true);
  tc::make_map_2d(&c.map_gt, c.gt.p, sl, (uint64_t)c.ldg, (uint64_t)smax * LP, (uint64_t)c.ldg * 2, 64, LP, true);
  // the same buffers seen as rows of E4M3 digits (one byte per K element)
  tc::make_map_2d(&c.map_w8, c.wsl.p, tc::kMapU8, (uint64_t)c.npad, (uint64_t)smax * LP, (uint64_t)c.npad, 128, LP,
                  true);
  tc::make_map_2d(&c.map_gt8, c.gt.p, tc::kMapU8, (uint64_t)c.ldg, (uint64_t)smax * LP, (uint64_t)c.ldg, 128, LP, true);
  c.w_slices = 0;
  c.w_mode = -1;
}

static void op_init(Context& c, const pcaone_gpu_params& p) {
  need_data(c);
  if (p.k <= 0 || p.oversamples < 0) throw Error(PCAONE_E_ARG, "k must be positive and oversamples >= 0");
  const int L = p.k + p.oversamples;
  if (L > kMaxL) throw Error(PCAONE_E_LIMIT, "k + oversamples exceeds " + std::to_string(kMaxL));
  if (L > c.N) throw Error(PCAONE_E_ARG, "k + oversamples exceeds the number of samples");
  if (p.svd != PCAONE_SVD_SINGLE && p.svd != PCAONE_SVD_WINDOW) throw Error(PCAONE_E_ARG, "svd must be 1 or 2");
  if (p.svd == PCAONE_SVD_WINDOW && (p.bands < 4 || (p.bands & (p.bands - 1)) != 0))
    throw Error(PCAONE_E_ARG, "the -w/--batches must be a power of 2 and the minimun is 4.");
  if (p.precision != PCAONE_PREC_FP32 && p.precision != PCAONE_PREC_BF16 && p.precision != PCAONE_PREC_BF16X3 &&
      p.precision != PCAONE_PREC_FP64 && p.precision != PCAONE_PREC_FP8)
    throw Error(PCAONE_E_ARG, "unknown precision form");
  if (c.dense && p.precision == PCAONE_PREC_FP8)
    throw Error(PCAONE_E_ARG, "the FP8 form takes PLINK genotypes (dense FP16 values are not E4M3 numbers)");
  if (c.dense && p.precision == PCAONE_PREC_FP32)
    throw Error(PCAONE_E_ARG, "dense (FileBinary) input runs in the tensor-core form only");
  if (c.dense && p.precision == PCAONE_PREC_FP64)
    throw Error(PCAONE_E_ARG, "the FP64-grade form takes PLINK genotypes (its products are exact only for integer dosages)");
  if (c.dense && p.emu) throw Error(PCAONE_E_ARG, "EM imputation needs PLINK input (no missing genotypes in dense input)");
  c.P = p;
  c.k = p.k;
  c.L = L;
  c.tc = p.precision != PCAONE_PREC_FP32;
  c.max_slices = p.precision == PCAONE_PREC_FP64 ? tc::kMaxSlices : tc::kIntSlices;
  c.fp64 = p.precision == PCAONE_PREC_FP64;
  c.fp8_form = p.precision == PCAONE_PREC_FP8;
  c.fp8_now = c.fp8_form;
  c.LP = c.tc ? round_up(L, 16) : round_up(L, 8);
  c.update = c.standardize = c.scaled = c.fitted = false;
  c.have_usv = false;
  c.permuted = false;
  c.perm_host.clear();
  if (!c.omega_user.empty()) {
    if (c.omega_user_rows != c.N || c.omega_user_cols != L)
      throw Error(PCAONE_E_ARG, "the supplied omega is not N x (k + oversamples)");
    c.omega0 = c.omega_user;
  } else {
    c.omega0.assign((size_t)c.N * L, 0.0);
    host_random_omega(p.seed, p.rand ? 1 : 0, c.N, L, c.omega0.data());
  }
  const size_t nl = (size_t)c.npad * c.LP;
  c.Omg0.ensure(nl, c.stream);
  c.Omg.ensure(nl, c.stream);
  c.Omg2.ensure(nl, c.stream);
  c.Omg32.ensure(nl, c.stream);
  c.H.ensure(nl, c.stream);
  c.H1.ensure(nl, c.stream);
  c.H2.ensure(nl, c.stream);
  c.G.ensure((size_t)c.M * c.LP, c.stream);
  c.lut32.ensure((size_t)c.M, c.stream, false);
  c.scale.ensure((size_t)c.M, c.stream, false);
  c.perm.ensure((size_t)c.M, c.stream, false);
  const size_t ll = (size_t)c.LP * c.LP;
  for (DBuf<double>* b : {&c.W, &c.R1, &c.R1i, &c.R2, &c.R2i, &c.R3, &c.R3i, &c.Rt, &c.Rti, &c.UB, &c.tmp})
    b->ensure(ll, c.stream);
  c.sigma.ensure(c.LP, c.stream);
  c.sgn.ensure(c.LP, c.stream);
  c.T.ensure((size_t)c.LP * c.k, c.stream);
  c.mevv.ensure(4, c.stream);
  c.status.ensure(4, c.stream);
  c.flag.ensure(c.LP, c.stream);
  const int cb = std::max(cross_blocks(std::max<int64_t>(c.M, c.npad)), flip_blocks(c.npad));
  c.red.ensure((size_t)cb * std::max(c.LP * c.LP, 2 * c.LP), c.stream, false);
  c.U.ensure((size_t)c.npad * c.k, c.stream);
  c.Upre.ensure((size_t)c.npad * c.k, c.stream);
  c.V.ensure((size_t)c.M * c.k, c.stream);
  c.Vpre.ensure((size_t)c.M * c.k, c.stream);
  // window scratch: the largest need over the distinct window lengths of the schedule
  const int64_t win = window_size(c);
  if (win <= 0)
    throw Error(PCAONE_E_LIMIT, "out-of-core: the device budget of " + std::to_string(c.stream_budget) +
                                    " bytes does not hold two SNP blocks (raise it, or the number of windows)");
  std::vector<int64_t> lens = {win, c.M % std::max<int64_t>(1, win)};
  size_t need_part = 1, need_hpart = 1;
  for (int64_t n : lens) {
    if (n <= 0) continue;
    WindowArgs a{c.view(), nullptr, nullptr, 0, (int)n, c.LP, c.npad};
    need_part = std::max(need_part, (size_t)window_g_chunks(a) * n * c.LP);
    need_hpart = std::max(need_hpart, (size_t)window_h_splits(a) * c.npad * c.LP);
  }
  c.part.ensure(need_part, c.stream, false);
  c.hpart.ensure(need_hpart, c.stream, false);
  c.g32.ensure((size_t)std::max<int64_t>(1, win) * c.LP, c.stream, false);
  c.bk_valid = false;  // the window size may have changed
  if (c.tc) {
    ensure_missing_total(c);
    // TMEM per CTA: one accumulator per slice (3 x LP columns) plus at least
    // one 32-column stage of the A operand (LP <= 112 always fits)
    if (c.max_slices * c.LP + 32 > 512)
      throw Error(PCAONE_E_LIMIT, c.max_slices > 3 ? "FP64-grade form: k + oversamples above 80 do not fit in TMEM"
                                                   : "tensor-core form: k + oversamples too large for TMEM");
    tc_setup(c, (int)std::max<int64_t>(1, win), lens);
  }
  upload_omega0(c);
  c.have_op = true;
}

// a caller-supplied initial matrix replaces the library's draw in this and
// every later op_init (NULL clears it)
static void set_omega(Context& c, const double* omega, uint32_t rows, uint32_t cols) {
  need_data(c);
  if (!omega) {
    c.omega_user.clear();
    c.omega_user_rows = c.omega_user_cols = 0;
    return;
  }
  if ((int)rows != c.N || cols == 0 || cols > (uint32_t)kMaxL) throw Error(PCAONE_E_ARG, "omega must be N x L");
  c.omega_user.assign(omega, omega + (size_t)rows * cols);
  c.omega_user_rows = (int)rows;
  c.omega_user_cols = (int)cols;
  if (c.have_op) {
    if ((int)cols != c.L) throw Error(PCAONE_E_ARG, "omega must be N x (k + oversamples)");
    c.omega0 = c.omega_user;
    upload_omega0(c);
  }
}

// initOmg: Omega = Omega2 = the initial draw
static void init_omg(Context& c) {
  const size_t nl = (size_t)c.npad * c.LP;
  PCAONE_CUDA(cudaMemcpyAsync(c.Omg.p, c.Omg0.p, nl * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  PCAONE_CUDA(cudaMemcpyAsync(c.Omg2.p, c.Omg0.p, nl * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  launch_to_f32(c.Omg.p, c.Omg32.p, (int64_t)nl, c.stream);
  c.w_slices = 0;
}

// a tensor-core tile that gave up a bounded wait leaves its partial sums
// unwritten: PCAONE_E_CUDA, reported before any numerical consequence
static void check_tc_err(Context& c) {
  if (!c.tc) return;
  int e = 0;
  PCAONE_CUDA(cudaMemcpyAsync(&e, c.err.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  if (e) throw Error(PCAONE_E_CUDA, "tensor-core pipeline: a bounded wait gave up (kernel aborted its tile)");
}

// Device status words: [0] CholeskyQR failures (OR of the factor kernels),
// [1] small-SVD convergence, [2] whether the first Gram of the last CholeskyQR
// needed the shift.  Read once per epoch (check_status), not per factor.
static void clear_status(Context& c) { PCAONE_CUDA(cudaMemsetAsync(c.status.p, 0, 2 * sizeof(int), c.stream)); }

static void check_status(Context& c) {
  int st[2] = {0, 0};
  PCAONE_CUDA(cudaMemcpyAsync(st, c.status.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  if (st[0]) {
    check_tc_err(c);  // a tile that gave up leaves partial sums unwritten: report that first
    throw Error(PCAONE_E_NUMERIC, "CholeskyQR: Gram matrix not positive definite, also after the shift");
  }
}

// Orthonormal factor of A (rows x LP, in place) by CholeskyQR2, or shifted
// CholeskyQR3 when the first Gram is not numerically positive definite
// (Fukaya, Kannan, Nakatsukasa, Yamamoto, Yanagisawa 2020): the first factor
// retries with the shift on the device and raises a device flag, which the
// third pass's kernels read, so no host round trip decides the path.  With
// need_r, Rt holds R (upper, A_in = Q R) and Rti its inverse on return; the
// updates of Omega only need Q.  Failures land in the device status word.
static void cholqr(Context& c, double* A, int64_t rows, bool need_r) {
  const int L = c.L, LP = c.LP;
  const int nb = cross_blocks(rows);
  int* failed = c.status.p;
  int* shifted = c.status.p + 2;
  launch_cross(A, LP, L, A, LP, L, rows, 1, c.W.p, LP, c.red.p, nb, c.stream, c.fp64);
  launch_chol_inv(c.W.p, L, LP, c.R1.p, c.R1i.p, failed, c.stream, c.fp64, rows, shifted);
  launch_gemm_tall_upper(A, rows, LP, c.R1i.p, c.stream, c.fp64);
  launch_cross(A, LP, L, A, LP, L, rows, 1, c.W.p, LP, c.red.p, nb, c.stream, c.fp64);
  launch_chol_inv(c.W.p, L, LP, c.R2.p, c.R2i.p, failed, c.stream, c.fp64);
  launch_gemm_tall_upper(A, rows, LP, c.R2i.p, c.stream, c.fp64);
  if (need_r) {
    launch_mult_small(c.R2.p, c.R1.p, c.Rt.p, LP, c.stream);     // R = R2 R1
    launch_mult_small(c.R1i.p, c.R2i.p, c.Rti.p, LP, c.stream);  // R^-1 = R1^-1 R2^-1
  }
  // the third pass of shifted CholeskyQR3, run by the device only when the
  // first factor needed the shift
  launch_cross(A, LP, L, A, LP, L, rows, 1, c.W.p, LP, c.red.p, nb, c.stream, c.fp64, shifted);
  launch_chol_inv(c.W.p, L, LP, c.R3.p, c.R3i.p, failed, c.stream, c.fp64, -1, nullptr, shifted);
  launch_gemm_tall_upper(A, rows, LP, c.R3i.p, c.stream, c.fp64, shifted);
  if (need_r) {
    launch_mult_small(c.R3.p, c.Rt.p, c.R1.p, LP, c.stream, shifted);    // R = R3 R2 R1
    launch_mult_small(c.Rti.p, c.R3i.p, c.R1i.p, LP, c.stream, shifted); // R^-1 = R1^-1 R2^-1 R3^-1
    launch_copy_if(c.R1.p, c.Rt.p, (int64_t)LP * LP, shifted, c.stream);
    launch_copy_if(c.R1i.p, c.Rti.p, (int64_t)LP * LP, shifted, c.stream);
  }
}

// Omega <- Q of a Householder QR of H (same column signs as Eigen's
// HouseholderQR::householderQ()), then PCAone::flipOmg(Omg2, Omg).
static void update_omega_from_h(Context& c) {
  const size_t nl = (size_t)c.npad * c.LP;
  PCAONE_CUDA(cudaMemcpyAsync(c.Omg.p, c.H.p, nl * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  cholqr(c, c.Omg.p, c.N, false);
  launch_house_signs(c.Omg.p, c.N, c.L, c.LP, c.sgn.p, c.stream);
  launch_flip_omg(c.Omg2.p, c.Omg.p, c.N, c.L, c.LP, c.red.p, c.sgn.p, c.stream);
  launch_to_f32(c.Omg.p, c.Omg32.p, (int64_t)nl, c.stream);
  c.w_slices = 0;
}

static void zero(DBuf<double>& b, cudaStream_t s) { PCAONE_CUDA(cudaMemsetAsync(b.p, 0, b.n * sizeof(double), s)); }

// missing-genotype list in working order (built once the order is final)
static void build_missing(Context& c) {
  if (c.miss_valid) return;
  if (c.counts_host.empty()) {
    c.counts_host.resize((size_t)c.M * 4);
    PCAONE_CUDA(cudaMemcpyAsync(c.counts_host.data(), c.counts.p, c.counts_host.size() * sizeof(int32_t),
                                cudaMemcpyDeviceToHost, c.stream));
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  }
  std::vector<int64_t> rowptr((size_t)c.M + 1, 0);
  for (int64_t p = 0; p < c.M; ++p) {
    const int64_t snp = c.permuted ? c.perm_host[p] : p;
    rowptr[p + 1] = rowptr[p] + c.counts_host[(size_t)snp * 4 + 1];
  }
  c.nnz = rowptr[c.M];
  if (c.nnz > 0x7fffffffLL) throw Error(PCAONE_E_LIMIT, "more than 2^31-1 missing genotypes");
  c.miss_rowptr.ensure(rowptr.size(), c.stream, false);
  PCAONE_CUDA(cudaMemcpyAsync(c.miss_rowptr.p, rowptr.data(), rowptr.size() * sizeof(int64_t),
                              cudaMemcpyHostToDevice, c.stream));
  c.miss_pos.ensure((size_t)c.nnz, c.stream, false);
  c.miss_sample.ensure((size_t)c.nnz, c.stream, false);
  c.miss_value.ensure((size_t)c.nnz, c.stream, true);
  launch_missing_list(c.view(), c.permuted ? c.perm.p : nullptr, c.miss_rowptr.p, c.miss_pos.p, c.miss_sample.p,
                      c.stream);
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  c.miss_rowptr_host.swap(rowptr);
  c.miss_valid = true;
}

// Data::fit_with_pi EMU branch (src/Data.cpp:318-348) on the missing list
static void fit_with_pi(Context& c) {
  if (!c.have_usv) throw Error(PCAONE_E_ARG, "EM update requested before a first computeUSV");
  const auto t0 = clk::now();
  build_missing(c);
  launch_em_fill(c.miss_pos.p, c.miss_sample.p, c.miss_value.p, c.nnz, c.permuted ? c.perm.p : nullptr, c.F.p,
                 c.U.p, c.sigma.p, c.V.p, c.k, c.stream);
  c.fitted = true;
  c.bk_stale = true;
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  c.t_em += secs(t0, clk::now());
}


// missing entries grouped by (window, sample), in working order: a count pass
// over the packed rows, an exclusive scan, and a fill pass
static void ensure_buckets(Context& c) {
  const int64_t ws = window_size(c);
  if (c.bk_valid && c.bk_wsize == ws) return;
  const int64_t nwin = (c.M + ws - 1) / ws;
  if (nwin > 65535) throw Error(PCAONE_E_LIMIT, "too many SNP windows for the missing-entry index");
  const size_t nb = (size_t)nwin * c.N;
  const int32_t* perm = c.permuted ? c.perm.p : nullptr;
  c.bk_cnt.ensure(nb, c.stream, false);
  launch_bucket_count(c.view(), perm, ws, (int)nwin, c.bk_cnt.p, c.stream);
  // offsets by a prefix sum on the device; the host keeps those at the window
  // boundaries (bucket w*N), one strided copy
  c.bk_ptr.ensure(nb + 1, c.stream, false);
  c.bk_scan.ensure((size_t)std::max<int64_t>(1, scan_tiles_needed((int64_t)nb)), c.stream, false);
  launch_exclusive_scan(c.bk_cnt.p, (int64_t)nb, c.bk_ptr.p, c.bk_scan.p, c.stream);
  std::vector<int64_t> ptr((size_t)nwin + 1);
  PCAONE_CUDA(cudaMemcpy2DAsync(ptr.data(), sizeof(int64_t), c.bk_ptr.p, (size_t)c.N * sizeof(int64_t),
                                sizeof(int64_t), (size_t)nwin + 1, cudaMemcpyDeviceToHost, c.stream));
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  const int64_t total = ptr[(size_t)nwin];
  if (total != (int64_t)c.counts_total_missing)
    throw Error(PCAONE_E_CUDA, "internal: missing-entry index disagrees with the genotype counts");
  c.bk_pos.ensure((size_t)std::max<int64_t>(1, total), c.stream, false);
  c.bk_sample.ensure((size_t)std::max<int64_t>(1, total), c.stream, false);
  launch_bucket_fill(c.view(), perm, ws, (int)nwin, c.bk_ptr.p, c.bk_pos.p, c.bk_sample.p, c.stream);
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  c.bk_ptr_host.swap(ptr);
  c.bk_wsize = ws;
  c.bk_nwin = (int)nwin;
  c.bk_valid = true;
  c.bk_stale = true;
}

// the missing-entry structures the window products read (the CSR list by
// position and its (window, sample) grouping, with the EM fill values once
// fitted): needed by the tensor-core form whenever a genotype is missing, and
// by the FP32 form for the EM term
static void prepare_missing(Context& c) {
  ensure_missing_total(c);
  const bool em = c.fitted && c.P.emu;
  if (c.counts_total_missing <= 0 || !(c.tc || em)) return;
  build_missing(c);
  ensure_buckets(c);
  if (em && c.bk_stale) {
    c.bk_value.ensure((size_t)std::max<int64_t>(1, c.nnz), c.stream, false);
    launch_em_fill(c.bk_pos.p, c.bk_sample.p, c.bk_value.p, c.nnz, c.permuted ? c.perm.p : nullptr, c.F.p, c.U.p,
                   c.sigma.p, c.V.p, c.k, c.stream);
    c.bk_stale = false;
  }
}

static void refresh_lut(Context& c) {
  launch_lut(c.F.p, c.M, c.scaled ? 1 : 0, c.P.ploidy, c.lut32.p, nullptr, c.scale.p, c.stream);
}

// the pi == 0 data preparation shared by both operators
static void prepare_epoch0(Context& c, bool window) {
  if (c.update && c.P.emu) {
    if (c.prefilled)
      c.prefilled = false;  // the learned start already holds the first fill
    else
      fit_with_pi(c);
  }
  // Data::standardize_E scales in place, once; FileBinary input runs with
  // -C 0, where standardize_E does nothing (src/Data.cpp:353)
  if (c.standardize && !c.dense) c.scaled = true;
  refresh_lut(c);
  if (window) {
    c.bandsize = 1;
    c.blocksize = (c.M + c.P.bands - 1) / c.P.bands;
    if (c.P.perm && !(c.update && c.P.emu) && !c.permuted) {
      // PCAone::permute_matrix (src/RSVD.hpp:61-70): column i <- column perm[i];
      // out of core, the order permute_plink gives the rewritten file
      // (src/Main.cpp:120-130)
      c.perm_host.resize((size_t)c.M);
      if (!c.streamed)
        host_shuffle_columns(c.M, c.perm_host.data());
      else if (!host_ooc_order(c.M, ((int64_t)c.N + 3) / 4, c.stream_buffer_gb, c.P.bands, c.perm_host.data()))
        throw Error(PCAONE_E_ARG, "out-of-core shuffle: a buffer of the --buffer size holds fewer SNPs than windows");
      PCAONE_CUDA(cudaMemcpyAsync(c.perm.p, c.perm_host.data(), c.M * sizeof(int32_t), cudaMemcpyHostToDevice,
                                  c.stream));
      PCAONE_CUDA(cudaStreamSynchronize(c.stream));
      c.permuted = true;
      c.miss_valid = false;
      c.bk_valid = false;
      c.invalidate_slots();  // streamed blocks are gathered through the order
      c.bt_valid = false;
      if (c.tc && !c.streamed) {
        c.bedp.ensure((size_t)c.M * c.stride, c.stream, false);
        tc::launch_gather_rows(c.bed.p, c.bedp.p, c.stride, c.perm.p, c.M, c.stream);
        c.bed_work = c.bedp.p;
        tc_make_bed_maps(c);
      }
    }
  }
  prepare_missing(c);
}

// ---- out-of-core streaming of SNP blocks (Halko.cpp:130-153, 227-268) ----

// the slot holding the block [pos0, pos0 + n) of the working order, or -1
static int find_slot(const Context& c, int64_t pos0, int64_t n) {
  for (int s = 0; s < 2; ++s)
    if (c.slots[s].pos0 == pos0 && c.slots[s].n == n) return s;
  return -1;
}

// fills slot s with the block [pos0, pos0 + n) on the fetch stream once the
// products that last read the slot have run: one host-to-device copy of the
// contiguous rows, or, in a shuffled order, a gather kernel that reads the
// rows through their device address
static void fetch_block(Context& c, int s, int64_t pos0, int64_t n) {
  Context::Slot& sl = c.slots[s];
  if (n > sl.rows) throw Error(PCAONE_E_ARG, "internal: streamed block larger than its slot");
  PCAONE_CUDA(cudaStreamWaitEvent(c.fetch_stream, sl.idle, 0));
  if (!c.permuted) {
    PCAONE_CUDA(cudaMemcpyAsync(sl.buf.p, c.hbed + (size_t)pos0 * c.stride, (size_t)n * c.stride,
                                cudaMemcpyHostToDevice, c.fetch_stream));
  } else {
    // shuffled windows: a gather kernel reads the block's rows through their
    // device address (scattered rows cross the host link at about 110 GB/s on
    // this system whether a kernel or pitched copies move them; contiguous
    // windows copy at about 170 GB/s)
    launch_gather_rows_deep(c.hbed_dev, sl.buf.p, c.stride, c.perm.p + pos0, n, 4 * c.sm_count, c.fetch_stream);
  }
  PCAONE_CUDA(cudaEventRecord(sl.ready, c.fetch_stream));
  sl.pos0 = pos0;
  sl.n = n;
  c.stream_bytes += (double)n * (double)c.stride;
}

// makes the block [pos0, pos0 + n) readable by the products on the context's
// stream and points the TMA descriptors at its slot, then prefetches the block
// that follows in schedule order (the next window, the first after the last)
// into the other slot.  Returns the first position the slot holds.
static int64_t acquire_block(Context& c, int64_t pos0, int64_t n) {
  int s = find_slot(c, pos0, n);
  if (s < 0) {
    s = c.slot_cur == 0 ? 1 : 0;
    fetch_block(c, s, pos0, n);
  }
  PCAONE_CUDA(cudaStreamWaitEvent(c.stream, c.slots[s].ready, 0));
  c.slot_cur = s;
  const Context::Slot& sl = c.slots[s];
  c.map_bed_g = sl.g;
  c.map_bed_h = sl.h;
  c.map_bed_g8 = sl.g8;
  c.map_bed_h8 = sl.h8;
  const int64_t next = pos0 + n < c.M ? pos0 + n : 0;
  const int64_t nn = std::min(window_size(c), c.M - next);
  if (nn > 0 && find_slot(c, next, nn) < 0) fetch_block(c, 1 - s, next, nn);
  return sl.pos0;
}

// the products of the current block are queued: its slot may be refilled after them
static void release_block(Context& c) { PCAONE_CUDA(cudaEventRecord(c.slots[c.slot_cur].idle, c.stream)); }

// The sample-major copy for the H products of genotype windows in HBM, built
// once per working order; false (and the transposing H kernel instead) for
// streamed rows, dense input, or when the copy does not fit in device memory.
static bool ensure_sample_major(Context& c) {
  if (c.dense || c.streamed || c.bt_off) return false;
  const int64_t ws = window_size(c);
  if (c.bt_valid && c.bt_ws == ws) return true;
  const int64_t ldw = (ws + 127) / 128 * 128;
  const int64_t nwin = (c.M + ws - 1) / ws;
  const int64_t pitch = nwin * (ldw / 4);
  try {
    c.bedT.ensure((size_t)c.npad * (size_t)pitch, c.stream, false);
  } catch (const Error&) {
    cudaGetLastError();
    c.bedT.release();
    c.bt_off = true;  // the H products keep the transposing kernel
    return false;
  }
  tc::launch_transpose_codes(c.bed_work, c.stride, c.M, ws, ldw, (int)nwin, c.npad, c.bedT.p, pitch, c.stream);
  tc::make_map_2d(&c.map_bt, c.bedT.p, tc::kMapU8, (uint64_t)pitch, (uint64_t)c.npad, (uint64_t)pitch, 16, 128,
                  false);
  tc::make_map_2d(&c.map_bt8, c.bedT.p, tc::kMapU8, (uint64_t)pitch, (uint64_t)c.npad, (uint64_t)pitch, 32, 128,
                  false);
  c.bt_ws = ws;
  c.bt_ldw = ldw;
  c.bt_pitch = pitch;
  c.bt_valid = true;
  return true;
}

// tensor-core form of one window (prod_tc.cu)
static void window_product_tc(Context& c, int64_t pos0, int64_t n, double* Hx) {
  const int LP = c.LP, S = c.nslice_cur;
  const bool fp8 = c.fp8_now;
  const int fmt = fp8 ? tc::kFmtE4M3 : c.dense ? tc::kFmtF16 : tc::kFmtBF16;
  if (c.w_slices != S || c.w_mode != S * 4 + fmt) {
    tc::launch_omega_slices(c.Omg.p, c.npad, c.N, LP, S, c.wsl.p, c.wunit.p, c.colsum.p, c.wexp.p, c.wrep.p,
                            c.wint.p, fmt, tc::ColRedScratch{c.cr_part.p, c.cr_cnt.p}, c.stream);
    c.w_slices = S;
    c.w_mode = S * 4 + fmt;
  }
  int chunk, nch, per, nsp;
  tc_shapes(c, (int)n, S, fp8, chunk, nch, per, nsp);
  if ((size_t)nch * n * LP > c.tpart.n || (size_t)nsp * c.npad * LP > c.thpart.n || n > c.win_max)
    throw Error(PCAONE_E_ARG, "internal: tensor-core window scratch too small");
  const bool any_miss = c.counts_total_missing > 0;
  const bool em = c.fitted && c.P.emu && c.nnz > 0;
  const int32_t* perm = c.permuted ? c.perm.p : nullptr;
  const int64_t win = any_miss && c.bk_wsize > 0 ? pos0 / c.bk_wsize : 0;
  if (any_miss && (!c.bk_valid || !c.miss_valid || pos0 != win * c.bk_wsize))
    throw Error(PCAONE_E_ARG, "internal: missing-entry index does not match the windows");
  const double flops = 2.0 * (double)c.N * (double)n * (double)c.L;
  auto mark = [&](int cls) {
    if (!c.profiling) return;
    const size_t i0 = c.ev_used;
    PCAONE_CUDA(cudaEventRecord(c.next_event(), c.stream));
    c.next_event();
    c.ev_marks.push_back({cls, i0});
    c.ev_work.push_back({cls, flops});
  };
  auto close_mark = [&]() {
    if (c.profiling) PCAONE_CUDA(cudaEventRecord(c.ev_pool[c.ev_marks.back().second + 1], c.stream));
  };
  // rows of the packed matrix the products read: the whole matrix in HBM, or
  // the streamed block's slot
  const int64_t row_base = c.streamed ? acquire_block(c, pos0, n) : 0;
  tc::GArgs ga{};
  ga.pos0 = pos0 - row_base;
  ga.nsnp = (int)n;
  ga.LP = LP;
  ga.nslice = S;
  ga.chunk = chunk;
  ga.npad = c.npad;
  ga.nchunks = nch;
  ga.nstages = tc::stages_for(LP, S, tc::g_tile_bytes(c.dense, fp8), c.dense);
  ga.tmem_cols = tc::tmem_cols_for(tc::tmem_cols_needed(LP, S, ga.nstages, c.dense));
  ga.wscale = c.wunit.p;
  ga.part = c.tpart.p;
  ga.err = c.err.p;
  ga.dense = c.dense ? 1 : 0;
  ga.wait_cycles = c.wait_cycles;
  ga.fp8 = fp8 ? 1 : 0;
  // resident CTAs: 3-8% faster on the 27-bit BF16 products of the
  // 200,000-sample windows, 3-4% slower on their E4M3 products
  ga.persist = c.product_form == 1 || (c.product_form == 2 && !fp8) ? 1 : 0;
  mark(fp8 ? 2 : 0);
  tc::launch_g(fp8 ? c.map_bed_g8 : c.map_bed_g, fp8 ? c.map_w8 : c.map_w, ga, c.stream);
  close_mark();
  if (any_miss) {
    // f sum_i W_i (and sum_i e_i W_i) over each SNP's missing samples
    SegGatherArgs sg{};
    sg.e0 = c.miss_rowptr_host[pos0];
    sg.e1 = c.miss_rowptr_host[pos0 + n];
    sg.key = c.miss_pos.p;
    sg.key_base = pos0;
    sg.src = c.miss_sample.p;
    sg.src_base = 0;
    sg.L = c.L;
    sg.LP = LP;
    sg.R = c.wint.p;
    sg.out = c.gisum.p;
    sg.val = em ? c.miss_value.p : nullptr;
    sg.R2 = c.wint.p;
    sg.out2 = c.gesum.p;
    launch_seg_gather(sg, c.stream);
  }
  tc::GFinishArgs fa{};
  fa.vfac = c.dense ? 1.0 : 0.5;
  fa.pos0 = pos0;
  fa.nsnp = (int)n;
  fa.L = c.L;
  fa.LP = LP;
  fa.nslice = S;
  fa.nchunks = nch;
  fa.fmt = fmt;
  fa.digit_bits = tc::digit_bits_of(fmt);
  // the B operand tensor map spans ldg columns; windows shorter than the
  // longest one leave the tail zeroed by the slicing kernel
  fa.ldg = c.ldg;
  fa.part = c.tpart.p;
  fa.colsum = c.colsum.p;
  fa.F = c.F.p;
  fa.scale = c.scale.p;
  fa.perm = perm;
  fa.wunit_m = c.wunit.p + (size_t)(std::min(S, tc::kIntSlices) - 1) * LP;
  fa.wunit_p = c.wunit.p + (size_t)(S - 1) * LP;
  fa.gisum = any_miss ? c.gisum.p : nullptr;
  fa.gesum = (any_miss && em) ? c.gesum.p : nullptr;
  fa.G = c.G.p;
  fa.gh = c.ghbuf.p;
  fa.ghint = c.ghint.p;
  fa.gmint = c.gmint.p;
  fa.gt = c.gt.p;
  fa.cpart = c.cpart.p;
  tc::launch_g_finish(fa, c.hexp.p, c.hunit.p, c.gmunit.p, c.cvec.p, tc::ColRedScratch{c.cr_part.p, c.cr_cnt.p},
                      c.stream);
  tc::HArgs ha{};
  ha.pos0 = pos0 - row_base;
  ha.nsnp = (int)n;
  ha.L = c.L;
  ha.LP = LP;
  ha.nslice = S;
  ha.per_split = per;
  ha.nsplit = nsp;
  ha.npad = c.npad;
  ha.nstages = tc::stages_for(LP, S, tc::h_tile_bytes(c.dense, fp8), c.dense);
  ha.tmem_cols = tc::tmem_cols_for(tc::tmem_cols_needed(LP, S, ha.nstages, c.dense));
  ha.hscale = c.hunit.p;
  ha.hpart = c.thpart.p;
  ha.err = c.err.p;
  ha.dense = c.dense ? 1 : 0;
  ha.wait_cycles = c.wait_cycles;
  ha.fp8 = fp8 ? 1 : 0;
  if (any_miss) {
    // sum_j Gm_j (and sum_j 2 e_j Gh_j) over each sample's missing SNPs of the window
    SegGatherArgs sg{};
    sg.e0 = c.bk_ptr_host[(size_t)win];
    sg.e1 = c.bk_ptr_host[(size_t)win + 1];
    sg.key = c.bk_sample.p;
    sg.key_base = 0;
    sg.src = c.bk_pos.p;
    sg.src_base = pos0;
    sg.L = c.L;
    sg.LP = LP;
    sg.R = c.gmint.p;
    sg.out = c.hisum.p;
    sg.val = em ? c.bk_value.p : nullptr;
    sg.R2 = c.ghint.p;
    sg.out2 = c.hesum.p;
    launch_seg_gather(sg, c.stream);
  }
  if (ensure_sample_major(c)) {
    // H = X_w^T Gh as a G product on the sample-major copy: rows = samples,
    // K = the window's positions (column block pos0 / ws), B = the Gh slices
    tc::GArgs ta{};
    ta.pos0 = 0;
    ta.kofs = pos0 / c.bt_ws * c.bt_ldw;
    ta.nsnp = c.npad;
    ta.LP = LP;
    ta.nslice = S;
    ta.chunk = per;
    ta.npad = (int)round_up64(n, fp8 ? 128 : 64);
    ta.nchunks = nsp;
    ta.nstages = tc::stages_for(LP, S, tc::g_tile_bytes(false, fp8), false);
    ta.tmem_cols = tc::tmem_cols_for(tc::tmem_cols_needed(LP, S, ta.nstages, false));
    ta.wscale = nullptr;
    ta.part = c.thpart.p;
    ta.err = c.err.p;
    ta.dense = 0;
    ta.wait_cycles = c.wait_cycles;
    ta.fp8 = fp8 ? 1 : 0;
    ta.persist = ga.persist;
    mark(fp8 ? 3 : 1);
    tc::launch_g(fp8 ? c.map_bt8 : c.map_bt, fp8 ? c.map_gt8 : c.map_gt, ta, c.stream);
    close_mark();
  } else {
    mark(fp8 ? 3 : 1);
    tc::launch_h(fp8 ? c.map_bed_h8 : c.map_bed_h, fp8 ? c.map_gt8 : c.map_gt, ha, c.stream);
    close_mark();
  }
  if (c.streamed) release_block(c);
  tc::HFinishArgs hf{};
  hf.nsamples = c.N;
  hf.npad = c.npad;
  hf.L = c.L;
  hf.LP = LP;
  hf.nsplit = nsp;
  hf.dense = c.dense ? 1 : 0;
  hf.hpart = c.thpart.p;
  hf.c = c.cvec.p;
  hf.Hx = Hx;
  hf.nslice = S;
  hf.hunit_m = c.hunit.p + (size_t)(std::min(S, tc::kIntSlices) - 1) * LP;
  hf.hunit_p = c.hunit.p + (size_t)(S - 1) * LP;
  hf.hisum = any_miss ? c.hisum.p : nullptr;
  hf.hesum = (any_miss && em) ? c.hesum.p : nullptr;
  tc::launch_h_finish(hf, c.stream);
}

// one window: G[pos0 .. pos0+n) = X_w Omega;  Hx += X_w^T G_w
static void window_product(Context& c, int64_t pos0, int64_t n, double* Hx) {
  if (n <= 0) return;
  if (c.tc) {
    window_product_tc(c, pos0, n, Hx);
    return;
  }
  WindowArgs a{c.view(), c.permuted ? c.perm.p : nullptr, c.lut32.p, pos0, (int)n, c.LP, c.npad};
  SparseRows sp{};
  if (c.fitted && c.P.emu && c.nnz > 0) {
    sp = SparseRows{c.miss_rowptr.p, c.miss_sample.p, c.miss_value.p, c.scale.p,
                    c.permuted ? c.perm.p : nullptr, 1};
  }
  const int nch = window_g_chunks(a);
  const int nsp = window_h_splits(a);
  if ((size_t)nch * n * c.LP > c.part.n || (size_t)nsp * c.npad * c.LP > c.hpart.n || (size_t)n * c.LP > c.g32.n)
    throw Error(PCAONE_E_ARG, "internal: window scratch too small");
  const double flops = 2.0 * (double)c.N * (double)n * (double)c.L;
  auto mark = [&](int cls) {
    if (!c.profiling) return;
    const size_t i0 = c.ev_used;
    PCAONE_CUDA(cudaEventRecord(c.next_event(), c.stream));
    c.next_event();
    c.ev_marks.push_back({cls, i0});
    c.ev_work.push_back({cls, flops});
  };
  auto close_mark = [&]() {
    if (c.profiling) PCAONE_CUDA(cudaEventRecord(c.ev_pool[c.ev_marks.back().second + 1], c.stream));
  };
  mark(0);
  launch_window_g(a, c.Omg32.p, c.part.p, nch, c.stream);
  close_mark();
  launch_window_g_finish(a, c.part.p, nch, sp, c.Omg.p, c.G.p, c.g32.p, c.stream);
  mark(1);
  launch_window_h(a, c.g32.p, c.hpart.p, nsp, c.stream);
  close_mark();
  launch_window_h_finish(a, c.hpart.p, nsp, Hx, c.stream);
  if (sp.active) {
    const int64_t win = c.bk_wsize > 0 ? pos0 / c.bk_wsize : 0;
    if (!c.bk_valid || pos0 != win * c.bk_wsize)
      throw Error(PCAONE_E_ARG, "internal: missing-entry index does not match the windows");
    launch_h_buckets(win, c.N, c.L, c.LP, c.bk_ptr.p, c.bk_pos.p, c.bk_value.p, sp.perm, c.scale.p, c.g32.p, pos0,
                     Hx, c.stream);
  }
}

// NormalRsvdOpData::computeGandH, in-core branch (src/Halko.cpp:99-128)
static void compute_g_and_h_single(Context& c, int pi) {
  if (pi == 0) init_omg(c);
  if (pi == 0) prepare_epoch0(c, false);
  if (pi > 0) update_omega_from_h(c);
  zero(c.H, c.stream);
  const int64_t w = window_size(c);
  for (int64_t pos = 0; pos < c.M; pos += w) window_product(c, pos, std::min(w, c.M - pos), c.H.p);
}

// FancyRsvdOpData::computeGandH, in-core branch (src/Halko.cpp:155-225)
static void compute_g_and_h_window(Context& c, int pi) {
  const int bands = c.P.bands;
  if (pi == 0) init_omg(c);
  if (std::ldexp(1.0, pi) >= bands) {
    zero(c.H1, c.stream);
    zero(c.H2, c.stream);
  }
  if (pi == 0) prepare_epoch0(c, true);
  c.bandsize = std::min(c.bandsize * 2, bands);
  const int64_t bs = c.blocksize;
  for (int b = 0, i = 1; b < bands; ++b, ++i) {
    const int64_t start = (int64_t)b * bs;
    const int64_t stop = (int64_t)(b + 1) * bs >= c.M ? c.M - 1 : (int64_t)(b + 1) * bs - 1;
    const int64_t n = stop - start + 1;  // <= 0 for windows past the last SNP (M < bands * blocksize)
    window_product(c, start, n, i <= c.bandsize / 2 ? c.H1.p : c.H2.p);
    const bool adjacent = pi > 0 && (b + 1) == (int)std::ldexp(1.0, pi - 1) && std::ldexp(1.0, pi) < bands;
    if ((b + 1) < c.bandsize && !adjacent) continue;
    if (!((i == c.bandsize) || (i == c.bandsize / 2) || adjacent)) continue;
    launch_add(c.H1.p, c.H2.p, c.H.p, (int64_t)c.npad * c.LP, c.stream);
    update_omega_from_h(c);
    if (i == c.bandsize) {
      zero(c.H1, c.stream);
      i = 0;
    } else {
      zero(c.H2, c.stream);
    }
  }
}

// integer slices of the tensor-core forms: three (27 bits per column), six
// (54 bits) in the FP64-grade form, and in the FP8 form's E4M3 epochs two
// base-16 digits (an 8-bit integer representation)
static int slices_for_epoch(const Context& c) { return c.fp8_now ? 2 : c.max_slices; }

// The FP8 form runs its range-finding epochs on E4M3 operands and at least
// kExactEpochs final epochs in the exact 27-bit form; after those it stops
// only once the leading PCs (those separated from the next by a relative
// eigen-gap above 5%) are within kFp8Settle of their limit: the change d
// between two exact epochs (sine of the largest principal angle) times
// r / (1 - r), with r = (sigma_L / sigma_n)^2 the per-epoch contraction of
// subspace iteration on the leading n of L columns (sigma_L bounds the first
// singular value outside the sketch); at most kFp8MaxExtra epochs beyond the
// schedule's own.
constexpr int kExactEpochs = 2;
constexpr double kFp8Settle = 1e-7;
constexpr int kFp8MaxExtra = 16;

// largest eigenvalue of a small symmetric matrix (row-major n x n), cyclic
// Jacobi rotations in FP64
static double sym_max_eig(std::vector<double> a, int n) {
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += a[p * n + q] * a[p * n + q];
    if (off < 1e-300) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[p * n + q];
        if (apq == 0.0) continue;
        const double theta = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int r = 0; r < n; ++r) {  // columns p, q
          const double arp = a[r * n + p], arq = a[r * n + q];
          a[r * n + p] = cs * arp - sn * arq;
          a[r * n + q] = sn * arp + cs * arq;
        }
        for (int r = 0; r < n; ++r) {  // rows p, q
          const double apr = a[p * n + r], aqr = a[q * n + r];
          a[p * n + r] = cs * apr - sn * aqr;
          a[q * n + r] = sn * apr + cs * aqr;
        }
      }
  }
  double m = 0.0;
  for (int i = 0; i < n; ++i) m = std::max(m, a[i * n + i]);
  return m;
}

// FP8 form: the predicted distance of the leading well-separated PCs of U
// (this epoch) from their limit, from their change against Upre (the
// previous epoch); 0 when no PC is separated from the next
static double fp8_leading_change(Context& c) {
  std::vector<double> sg((size_t)c.L);
  PCAONE_CUDA(cudaMemcpyAsync(sg.data(), c.sigma.p, c.L * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  int n = 0;
  for (int i = 0; i + 1 < c.k; ++i) {
    const double e0 = sg[i] * sg[i], e1 = sg[i + 1] * sg[i + 1];
    if (e0 > 0.0 && (e0 - e1) / e0 > 0.05) n = i + 1;
  }
  if (n == 0) return 0.0;
  const double q = sg[c.L - 1] / sg[n - 1];
  const double r = std::min(0.999, q * q);
  c.rres.ensure((size_t)c.npad * n, c.stream, false);
  launch_subspace_change(c.U.p, c.Upre.p, c.N, c.k, n, c.tmp.p, c.rres.p, c.W.p, c.red.p, cross_blocks(c.N),
                         c.stream);
  std::vector<double> w((size_t)n * n);
  PCAONE_CUDA(cudaMemcpyAsync(w.data(), c.W.p, w.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  return std::sqrt(std::max(0.0, sym_max_eig(w, n))) * r / (1.0 - r);
}


static void compute_g_and_h(Context& c, int pi) {
  c.nslice_cur = c.tc ? slices_for_epoch(c) : 1;
  if (c.P.svd == PCAONE_SVD_WINDOW)
    compute_g_and_h_window(c, pi);
  else
    compute_g_and_h_single(c, pi);
}

// RsvdOpData::computeUSV (src/Halko.cpp:46-97)
static int compute_usv(Context& c, int p, double tol) {
  const int64_t M = c.M;
  if (c.tc) PCAONE_CUDA(cudaMemsetAsync(c.err.p, 0, sizeof(int), c.stream));  // a fresh abort flag per call
  clear_status(c);
  const int N = c.N, L = c.L, LP = c.LP, k = c.k;
  int epochs = 0;
  bool done = false, ucur_in_upre = false;
  // FP8 form: E4M3 epochs while kExactEpochs epochs remain after them and the
  // range finder has not converged; then exact epochs, of which at least
  // kExactEpochs run before the convergence rule may stop the loop
  bool switched = false;
  int exact_done = 0;
  const int p_cap = p + kFp8MaxExtra;
  for (int pi = 0; pi <= p; ++pi) {
    auto t0 = clk::now();
    c.fp8_now = c.fp8_form && !switched && pi + kExactEpochs <= p;
    if (!c.fp8_now) ++exact_done;
    compute_g_and_h(c, pi);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
    check_tc_err(c);
    check_status(c);
    c.collect_events();
    auto t1 = clk::now();
    c.t_prod += secs(t0, t1);
    ++epochs;
    cholqr(c, c.G.p, M, true);  // G <- Q2, Rt = R2 R1
    launch_cross(c.H.p, LP, L, c.H.p, LP, L, N, 1, c.W.p, LP, c.red.p, cross_blocks(N), c.stream, c.fp64);
    launch_usv_small(c.Rti.p, c.W.p, L, LP, k, c.UB.p, c.sigma.p, c.T.p, c.tmp.p, c.status.p + 1, c.stream);
    // Ucur = H T (right singular vectors of B = R^{-T} H^T)
    launch_gemm_tall(c.H.p, N, LP, c.T.p, k, k, c.U.p, k, c.stream, c.fp64);
    // Upre <- Ucur only where the reference assigns it (Halko.cpp:84-94); the
    // winSVD minimum-epoch branch keeps the older Upre.
    bool set_upre = pi == 0;
    if (pi > 0) {
      launch_mev(c.U.p, c.Upre.p, N, k, c.mevv.p, c.tmp.p, c.red.p, cross_blocks(N), c.stream);
      double mv = 0;
      PCAONE_CUDA(cudaMemcpyAsync(&mv, c.mevv.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
      PCAONE_CUDA(cudaStreamSynchronize(c.stream));
      check_status(c);  // the QR of G
      const double diff = 1.0 - mv;
      if (c.verbose && !c.P.emu) std::fprintf(stderr, "running of epoch = %d, diff = %g\n", pi, diff);
      if (diff < tol || pi == p) {
        if (c.P.svd == PCAONE_SVD_WINDOW && std::ldexp(1.0, pi) < c.P.bands) {
          p = (int)std::log2((double)c.P.bands);
        } else if (c.fp8_form && (c.fp8_now || exact_done < kExactEpochs)) {
          // the E4M3 range finder has converged (or too few exact epochs ran):
          // continue with exact epochs
          switched = true;
          p = std::max(p, pi + kExactEpochs - (c.fp8_now ? 0 : exact_done));
          set_upre = true;
        } else if (c.fp8_form && pi < p_cap && fp8_leading_change(c) > kFp8Settle) {
          // the leading PCs still move after the E4M3 epochs: one more exact epoch
          p = std::max(p, pi + 1);
          set_upre = true;
        } else {
          launch_gemm_tall(c.G.p, M, LP, c.UB.p, LP, k, c.V.p, k, c.stream, c.fp64);  // V = Q2 U_B[:, :k]
          done = true;
        }
      } else {
        set_upre = true;
      }
    }
    ucur_in_upre = false;
    if (set_upre) {
      std::swap(c.U.p, c.Upre.p);
      ucur_in_upre = true;
    }
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
    c.t_qr += secs(t1, clk::now());
    if (done) break;
  }
  if (ucur_in_upre) std::swap(c.U.p, c.Upre.p);  // U = Ucur after the loop (Halko.cpp:96)
  check_status(c);
  c.have_usv = true;
  return epochs;
}

static void copy_out(Context& c, const double* dev, int64_t rows, int ld, int cols, double* host) {
  if (!host) return;
  c.outbuf.ensure((size_t)rows * cols, c.stream, false);
  launch_transpose_out(dev, rows, ld, cols, c.outbuf.p, c.stream);
  PCAONE_CUDA(cudaMemcpyAsync(host, c.outbuf.p, (size_t)rows * cols * sizeof(double), cudaMemcpyDeviceToHost,
                              c.stream));
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
}

static void outputs(Context& c, double* U, double* S, double* V) {
  copy_out(c, c.U.p, c.N, c.k, c.k, U);
  copy_out(c, c.V.p, c.M, c.k, c.k, V);
  if (S) {
    PCAONE_CUDA(cudaMemcpyAsync(S, c.sigma.p, c.k * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  }
}

static void flip_uv(Context& c) { launch_flip_uv(c.U.p, c.N, c.V.p, c.M, c.k, c.flag.p, c.stream); }

// run_pca_with_halko (src/Halko.cpp:271-320), PLINK input, no LD output
// Learned warm start (mlp.cu): train the network on observed genotypes drawn
// at random, measure it on further held-out ones, then fill every missing
// genotype (in both orderings of the missing-entry lists) with its clamped
// prediction; the next EM iteration starts from that fill.
static void warm_start(Context& c) {
  const auto t0 = clk::now();
  const pcaone_gpu_mlp_params& w = c.warm;
  if (w.train_entries <= 0 || w.batch <= 0 || w.epochs < 0 || w.holdout_entries < 0)
    throw Error(PCAONE_E_ARG, "invalid warm-start parameters");
  build_missing(c);
  ensure_buckets(c);
  if (!c.net) c.net.reset(new mlp::Net(c.stream));
  mlp::Net& net = *c.net;
  net.init(w.seed);
  const int32_t* perm = c.permuted ? c.perm.p : nullptr;
  c.smiss.ensure(c.N, c.stream, false);
  mlp::sample_missing(c.bk_ptr.p, c.bk_nwin, c.N, c.M, c.smiss.p, c.stream);
  mlp::FeatureArgs fa{c.rows_ptr(), c.stride, c.M, c.N, perm, c.F.p, c.U.p, c.V.p, c.smiss.p, c.counts.p, c.k,
                      std::min(c.k, 14), std::sqrt((double)c.N), std::sqrt((double)c.M)};
  const int T = (w.train_entries / w.batch) * w.batch, Hn = w.holdout_entries;
  if (T <= 0) throw Error(PCAONE_E_ARG, "warm start: fewer training genotypes than one batch");
  const int D = T + Hn;
  c.wpos.ensure(D, c.stream, false);
  c.wsmp.ensure(D, c.stream, false);
  c.wX.ensure((size_t)D * mlp::kIn, c.stream, false);
  c.wy.ensure(D, c.stream, false);
  mlp::draw_observed(c.view(), perm, w.seed ^ 0x5eedULL, D, c.wpos.p, c.wsmp.p, c.stream);
  mlp::features(fa, c.wpos.p, c.wsmp.p, D, c.wX.p, c.wy.p, c.stream);
  double last = 0.0;
  for (int e = 0; e < w.epochs; ++e) {
    double sum = 0.0;
    for (int b0 = 0; b0 < T; b0 += w.batch) {
      net.forward(c.wX.p + (size_t)b0 * mlp::kIn, w.batch, true);
      net.backward(c.wX.p + (size_t)b0 * mlp::kIn, c.wy.p + b0, w.batch);
      net.adam(w.lr);
      if (e + 1 == w.epochs) sum += net.loss_host();
    }
    last = sum / T;
  }
  // held-out error of the network and of the mean fill (prediction 0)
  double mse = 0.0, mse0 = 0.0;
  if (Hn > 0) {
    std::vector<float> out(Hn), y(Hn);
    for (int b0 = 0; b0 < Hn; b0 += w.batch) {
      const int nb = std::min(w.batch, Hn - b0);
      net.forward(c.wX.p + (size_t)(T + b0) * mlp::kIn, nb, false);
      PCAONE_CUDA(cudaMemcpyAsync(out.data() + b0, net.out(), nb * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
    }
    PCAONE_CUDA(cudaMemcpyAsync(y.data(), c.wy.p + T, Hn * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
    for (int r = 0; r < Hn; ++r) {
      mse += ((double)out[r] - y[r]) * ((double)out[r] - y[r]);
      mse0 += (double)y[r] * y[r];
    }
    mse /= Hn;
    mse0 /= Hn;
  }
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  const auto t1 = clk::now();
  // fill the missing genotypes: CSR by position (G side) and buckets (H side)
  c.bk_value.ensure((size_t)std::max<int64_t>(1, c.nnz), c.stream, false);
  const int chunk = 65536;
  c.wX.ensure(std::max((size_t)D * mlp::kIn, (size_t)chunk * mlp::kIn), c.stream, false);
  for (int pass = 0; pass < 2; ++pass) {
    const int32_t* ppos = pass == 0 ? c.miss_pos.p : c.bk_pos.p;
    const int32_t* psmp = pass == 0 ? c.miss_sample.p : c.bk_sample.p;
    double* val = pass == 0 ? c.miss_value.p : c.bk_value.p;
    for (int64_t e0 = 0; e0 < c.nnz; e0 += chunk) {
      const int nb = (int)std::min<int64_t>(chunk, c.nnz - e0);
      mlp::features(fa, ppos + e0, psmp + e0, nb, c.wX.p, nullptr, c.stream);
      net.forward(c.wX.p, nb, false);
      mlp::fill(net.out(), ppos + e0, perm, c.F.p, nb, val + e0, c.stream);
    }
  }
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  c.fitted = true;
  c.prefilled = true;
  c.bk_stale = false;
  c.warm_stats[0] = last;
  c.warm_stats[1] = mse;
  c.warm_stats[2] = mse0;
  c.warm_stats[3] = secs(t0, t1);
  c.warm_stats[4] = secs(t1, clk::now());
  c.warm_stats[5] = 2.0 * (double)c.nnz;
}

static int run_halko(Context& c, const pcaone_gpu_params& p) {
  op_init(c, p);
  int em_iters = 0;
  if (!p.emu) {
    c.update = false;
    c.standardize = p.standardize != 0;
    compute_usv(c, p.maxp, p.tol);
    return 0;
  }
  c.update = false;
  c.standardize = false;
  compute_usv(c, p.maxp, p.tol);
  flip_uv(c);
  c.prefilled = false;
  ensure_missing_total(c);
  if (c.warm.enable && c.counts_total_missing > 0 && p.maxiter > 0) warm_start(c);
  for (int it = 0; it < p.maxiter; ++it) {
    c.update = true;
    c.standardize = false;
    PCAONE_CUDA(cudaMemcpyAsync(c.Vpre.p, c.V.p, (size_t)c.M * c.k * sizeof(double), cudaMemcpyDeviceToDevice,
                                c.stream));
    compute_usv(c, p.maxp, p.tol);
    flip_uv(c);
    launch_mev(c.V.p, c.Vpre.p, c.M, c.k, c.mevv.p, c.tmp.p, c.red.p, cross_blocks(c.M), c.stream);
    double mv = 0;
    PCAONE_CUDA(cudaMemcpyAsync(&mv, c.mevv.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
    const double diff = 1.0 - mv;
    em_iters = it + 1;
    if (c.verbose) std::fprintf(stderr, "individual allele frequencies estimated iter = %d, diff = %g\n", it + 1, diff);
    if (diff < p.tolem) break;
  }
  c.update = true;
  c.standardize = true;
  compute_usv(c, p.maxp, p.tol);
  flip_uv(c);
  return em_iters;
}

// Projection of the loaded samples onto a fit (project.cu; run_projection,
// src/Projection.cpp:236-247).  F, V (M x k column-major, file order) and S
// come from the fit; U (N x k column-major) receives the scores.
static void project(Context& c, const double* F, const double* V, const double* S, int k, int mode, double* U) {
  need_plink(c);
  if (!F || !V || !S || !U) throw Error(PCAONE_E_ARG, "null projection argument");
  if (mode != 1 && mode != 2) throw Error(PCAONE_E_ARG, "projection mode must be 1 or 2");
  if (k <= 0 || k > project_max_k())
    throw Error(PCAONE_E_LIMIT, "projection takes 1 to " + std::to_string(project_max_k()) + " PCs");
  const int N = c.N;
  const int64_t M = c.M;
  std::vector<double> Bh((size_t)M * k);
  for (int q = 0; q < k; ++q) {
    if (!(S[q] > 0.0)) throw Error(PCAONE_E_ARG, "singular values must be positive");
    const double f = mode == 1 ? 1.0 / S[q] : S[q];
    for (int64_t j = 0; j < M; ++j) Bh[(size_t)j * k + q] = V[(size_t)q * M + j] * f;
  }
  DBuf<double> Fd, B, lut, sc, part, R, X, W, red;
  Fd.ensure((size_t)M, c.stream, false);
  B.ensure((size_t)M * k, c.stream, false);
  lut.ensure((size_t)M * 4, c.stream, false);
  sc.ensure((size_t)M, c.stream, false);
  PCAONE_CUDA(cudaMemcpyAsync(Fd.p, F, (size_t)M * 8, cudaMemcpyHostToDevice, c.stream));
  PCAONE_CUDA(cudaMemcpyAsync(B.p, Bh.data(), Bh.size() * 8, cudaMemcpyHostToDevice, c.stream));
  launch_lut(Fd.p, M, 1, 2, nullptr, lut.p, sc.p, c.stream);  // standardize_E with the fit's F, ploidy 2
  const int ctas = c.npad / 128;
  const int nsplit = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(608, ctas), (M + 31) / 32));
  part.ensure((size_t)nsplit * c.npad * k, c.stream, false);
  R.ensure((size_t)N * k, c.stream, false);
  launch_project_rhs(c.view(), lut.p, B.p, k, c.npad, part.p, nsplit, R.p, c.stream);
  const double* out = R.p;
  if (mode == 2) {
    // K = B^T B, then per sample minus its missing SNPs' outer products
    const int nb = cross_blocks(M);
    W.ensure((size_t)k * k, c.stream, false);
    red.ensure((size_t)nb * k * k, c.stream, false);
    launch_cross(B.p, k, k, B.p, k, k, M, 1, W.p, k, red.p, nb, c.stream);
    DBuf<int32_t> cnt, pos, smp;
    DBuf<int64_t> ptr;
    cnt.ensure(N, c.stream, false);
    launch_bucket_count(c.view(), nullptr, M, 1, cnt.p, c.stream);
    std::vector<int32_t> ch(N);
    PCAONE_CUDA(cudaMemcpyAsync(ch.data(), cnt.p, (size_t)N * 4, cudaMemcpyDeviceToHost, c.stream));
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<int64_t> ph((size_t)N + 1, 0);
    for (int i = 0; i < N; ++i) ph[i + 1] = ph[i] + ch[i];
    ptr.ensure((size_t)N + 1, c.stream, false);
    PCAONE_CUDA(cudaMemcpyAsync(ptr.p, ph.data(), ph.size() * 8, cudaMemcpyHostToDevice, c.stream));
    pos.ensure((size_t)std::max<int64_t>(1, ph[N]), c.stream, false);
    smp.ensure((size_t)std::max<int64_t>(1, ph[N]), c.stream, false);
    launch_bucket_fill(c.view(), nullptr, M, 1, ptr.p, pos.p, smp.p, c.stream);
    X.ensure((size_t)N * k, c.stream, false);
    launch_project_solve(W.p, B.p, k, ptr.p, pos.p, R.p, N, X.p, c.stream);
    out = X.p;
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));  // the local buffers are freed on return
  }
  copy_out(c, out, N, k, k, U);
}

static void matvec(Context& c, const double* x, double* y, int standardize) {
  need_plink(c);
  const int N = c.N;
  c.mv_x.ensure(N, c.stream, false);
  c.mv_y.ensure(N, c.stream, false);
  c.mv_t.ensure((size_t)c.M, c.stream, false);
  c.mv_scale.ensure((size_t)c.M, c.stream, false);
  const int nsplit = matvec_splits(c.M, N);
  c.mv_ypart.ensure((size_t)nsplit * N, c.stream, false);
  PCAONE_CUDA(cudaMemcpyAsync(c.mv_x.p, x, N * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  // the scale sqrt(ploidy)/sd of src/FilePlink.cpp:146, with the ploidy of the
  // operator's parameters (2 before any pcaone_gpu_op_init)
  launch_lut(c.F.p, c.M, standardize, c.have_op ? c.P.ploidy : 2, nullptr, nullptr, c.mv_scale.p, c.stream);
  launch_matvec(c.view(), c.F.p, c.mv_scale.p, c.mv_x.p, c.mv_t.p, c.mv_y.p, c.mv_ypart.p, nsplit, c.stream);
  PCAONE_CUDA(cudaMemcpyAsync(y, c.mv_y.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  PCAONE_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace pcaone

// ==========================================================================
// C-ABI
// ==========================================================================
using pcaone::Context;
using pcaone::Error;

struct pcaone_gpu_ctx {
  Context c;
};

template <class F>
static int guarded(pcaone_gpu_ctx* ctx, F&& fn) {
  if (!ctx) return PCAONE_E_ARG;
  try {
    PCAONE_CUDA(cudaSetDevice(ctx->c.device));
    fn(ctx->c);
    ctx->c.last_error.clear();
    return PCAONE_OK;
  } catch (const Error& e) {
    ctx->c.last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    ctx->c.last_error = "host allocation failed";
    return PCAONE_E_NOMEM;
  } catch (const std::exception& e) {
    ctx->c.last_error = e.what();
    return PCAONE_E_ARG;
  }
}

namespace pcaone {
// Layout of a .pgen image this library reads itself (FilePgen, src/FilePgen.hpp:13-40,
// reads every .pgen through pgenlib): PLINK 1 variant-major rows (storage mode
// 0x01: the 3 magic bytes, then ceil(N/4)-byte rows, the sample count from the
// caller's .psam), or the fixed-width PLINK 2 modes 0x02 (2-bit hard calls),
// 0x03 (hard calls, then 2 N bytes of dosages per record) and 0x04 (then 4 N
// bytes of dosages and phased dosages): magic, mode, variant and sample counts
// (little-endian uint32), and a control byte whose low six bits are zero and
// whose top two say where the non-reference flags are (3: one bit per variant
// right after the 12 header bytes).  Only the hard calls are read.
// Variable-width files (compressed records) are decoded by pgenlib on the host,
// whose hard calls pcaone_gpu_load_pgen_genovecs takes.
struct PgenLayout {
  int mode = 0;
  uint64_t nsnps = 0, offset = 0, pitch = 0;
  uint32_t nsamples = 0;
};

static uint32_t le32(const uint8_t* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

PgenLayout pgen_layout(const uint8_t* img, uint64_t bytes, uint32_t nsamples_psam) {
  if (!img || bytes < 3 || img[0] != 0x6c || img[1] != 0x1b) throw Error(PCAONE_E_FORMAT, "not a .pgen file (magic)");
  PgenLayout l;
  l.mode = img[2];
  if (l.mode == 0x01) {
    if (nsamples_psam == 0) throw Error(PCAONE_E_ARG, "a PLINK 1 mode .pgen needs the sample count of its .psam");
    l.nsamples = nsamples_psam;
    l.pitch = ((uint64_t)l.nsamples + 3) / 4;
    l.offset = 3;
    if ((bytes - 3) % l.pitch != 0) throw Error(PCAONE_E_FORMAT, "PLINK 1 mode .pgen: size is not a whole number of rows");
    l.nsnps = (bytes - 3) / l.pitch;
    return l;
  }
  if (l.mode == 0x00) throw Error(PCAONE_E_FORMAT, "sample-major PLINK 1 data");
  if (l.mode >= 0x10)
    throw Error(PCAONE_E_FORMAT, "variable-width .pgen (compressed records): decode the records with pgenlib and pass "
                                 "the hard calls to pcaone_gpu_load_pgen_genovecs");
  if (l.mode > 0x04) throw Error(PCAONE_E_FORMAT, "unknown .pgen storage mode");
  if (bytes < 12) throw Error(PCAONE_E_FORMAT, "truncated .pgen header");
  l.nsnps = le32(img + 3);
  l.nsamples = le32(img + 7);
  const uint8_t ctrl = img[11];
  if (ctrl & 63) throw Error(PCAONE_E_FORMAT, "fixed-width .pgen with a variable-width control byte");
  if (l.nsnps == 0 || l.nsamples == 0) throw Error(PCAONE_E_FORMAT, ".pgen with no variants or samples");
  if (nsamples_psam != 0 && nsamples_psam != l.nsamples)
    throw Error(PCAONE_E_ARG, ".pgen sample count differs from the .psam: " + std::to_string(l.nsamples) + " vs " +
                                  std::to_string(nsamples_psam));
  l.offset = 12 + ((ctrl >> 6) == 3 ? (l.nsnps + 7) / 8 : 0);
  l.pitch = ((uint64_t)l.nsamples + 3) / 4 + (l.mode == 0x03 ? 2ull : l.mode == 0x04 ? 4ull : 0ull) * l.nsamples;
  if (bytes != l.offset + l.nsnps * l.pitch)
    throw Error(PCAONE_E_FORMAT, ".pgen size " + std::to_string(bytes) + " bytes, expected " +
                                     std::to_string(l.offset + l.nsnps * l.pitch));
  return l;
}
}  // namespace pcaone

static void check_bed_image(const uint8_t* image, uint64_t image_bytes, uint64_t nsnps, uint32_t nsamples) {
  if (!image || image_bytes < 3) throw Error(PCAONE_E_FORMAT, "truncated .bed image");
  if (image[0] != 0x6c || image[1] != 0x1b || image[2] != 0x01)
    throw Error(PCAONE_E_FORMAT, "Incorrect magic number in plink bed file.");
  const uint64_t need = 3 + nsnps * (((uint64_t)nsamples + 3) / 4);
  if (image_bytes < need)
    throw Error(PCAONE_E_FORMAT, "truncated .bed: " + std::to_string(image_bytes) + " bytes, expected " +
                                     std::to_string(need));
}

extern "C" {

void pcaone_gpu_default_params(pcaone_gpu_params* p) {
  if (!p) return;
  p->svd = PCAONE_SVD_WINDOW;
  p->k = 10;
  p->oversamples = 10;
  p->maxp = 20;
  p->bands = 64;
  p->seed = 112;
  p->rand = 1;
  p->perm = 1;
  p->emu = 0;
  p->maxiter = 100;
  p->tol = 1e-4;
  p->tolem = 1e-5;
  p->ploidy = 2;
  p->standardize = 1;
  p->precision = PCAONE_PREC_FP32;
}

int pcaone_gpu_abi_version(void) { return PCAONE_GPU_ABI_VERSION; }

int pcaone_gpu_random_omega(int seed, int gaussian, uint64_t rows, uint32_t cols, double* out) {
  if (!out || rows == 0 || cols == 0) return PCAONE_E_ARG;
  try {
    pcaone::host_random_omega(seed, gaussian ? 1 : 0, (int64_t)rows, (int64_t)cols, out);
  } catch (const std::exception&) {
    return PCAONE_E_ARG;
  }
  return PCAONE_OK;
}

int pcaone_gpu_shuffle_order(uint64_t n, int32_t* perm) {
  if (!perm || n == 0 || n > 0x7fffffffull) return PCAONE_E_ARG;
  pcaone::host_shuffle_columns((int64_t)n, perm);
  return PCAONE_OK;
}

int pcaone_gpu_open(const pcaone_gpu_desc* desc, pcaone_gpu_ctx** out) {
  if (!out) return PCAONE_E_ARG;
  *out = nullptr;
  std::unique_ptr<pcaone_gpu_ctx> ctx(new (std::nothrow) pcaone_gpu_ctx());
  if (!ctx) return PCAONE_E_NOMEM;
  ctx->c.device = desc ? desc->device : 0;
  ctx->c.verbose = desc ? desc->verbose : 0;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PCAONE_E_CUDA;
  if (ctx->c.device < 0 || ctx->c.device >= ndev) return PCAONE_E_ARG;
  if (cudaSetDevice(ctx->c.device) != cudaSuccess) return PCAONE_E_CUDA;
  if (cudaDeviceGetAttribute(&ctx->c.sm_count, cudaDevAttrMultiProcessorCount, ctx->c.device) != cudaSuccess)
    return PCAONE_E_CUDA;
  if (cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking) != cudaSuccess) return PCAONE_E_CUDA;
  *out = ctx.release();
  return PCAONE_OK;
}

int pcaone_gpu_close(pcaone_gpu_ctx* ctx) {
  if (!ctx) return PCAONE_OK;
  cudaSetDevice(ctx->c.device);
  cudaStreamSynchronize(ctx->c.stream);
  cudaStream_t s = ctx->c.stream;
  delete ctx;  // frees device buffers
  cudaStreamDestroy(s);
  return PCAONE_OK;
}

const char* pcaone_gpu_last_error(const pcaone_gpu_ctx* ctx) {
  return ctx ? ctx->c.last_error.c_str() : "null context";
}

int pcaone_gpu_set_wait_limit(pcaone_gpu_ctx* ctx, long long cycles) {
  return guarded(ctx, [&](Context& c) {
    if (cycles < 0) throw Error(PCAONE_E_ARG, "negative wait limit");
    c.wait_cycles = cycles;
  });
}

int pcaone_gpu_set_product_form(pcaone_gpu_ctx* ctx, int form) {
  return guarded(ctx, [&](Context& c) {
    if (form < 0 || form > 2) throw Error(PCAONE_E_ARG, "product form must be 0, 1 or 2");
    c.product_form = form;
  });
}

int pcaone_gpu_set_profiling(pcaone_gpu_ctx* ctx, int on) {
  return guarded(ctx, [&](Context& c) {
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
    c.collect_events();
    c.profiling = on != 0;
    for (int i = 0; i < 4; ++i) {
      c.prof_ms[i] = 0;
      c.prof_flops[i] = 0;
      c.prof_launches[i] = 0;
    }
  });
}

int pcaone_gpu_kernel_stats(pcaone_gpu_ctx* ctx, double ms[4], double flops[4], long long launches[4]) {
  return guarded(ctx, [&](Context& c) {
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
    c.collect_events();
    for (int i = 0; i < 4; ++i) {
      if (ms) ms[i] = c.prof_ms[i];
      if (flops) flops[i] = c.prof_flops[i];
      if (launches) launches[i] = c.prof_launches[i];
    }
  });
}

unsigned long long pcaone_gpu_launch_count(void) { return pcaone::g_kernel_launches; }

int pcaone_gpu_timings(const pcaone_gpu_ctx* ctx, double t[4]) {
  if (!ctx || !t) return PCAONE_E_ARG;
  t[0] = ctx->c.t_total;
  t[1] = ctx->c.t_prod;
  t[2] = ctx->c.t_qr;
  t[3] = ctx->c.t_em;
  return PCAONE_OK;
}

int pcaone_gpu_load_bed(pcaone_gpu_ctx* ctx, const uint8_t* packed, uint64_t nsnps, uint32_t nsamples) {
  return guarded(ctx, [&](Context& c) {
    if (!packed) throw Error(PCAONE_E_ARG, "null genotype buffer");
    pcaone::load_bed_host(c, packed, nsnps, nsamples);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_load_bed_file_image(pcaone_gpu_ctx* ctx, const uint8_t* image, uint64_t image_bytes,
                                   uint64_t nsnps, uint32_t nsamples) {
  return guarded(ctx, [&](Context& c) {
    check_bed_image(image, image_bytes, nsnps, nsamples);
    pcaone::load_bed_host(c, image + 3, nsnps, nsamples);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_load_bed_stream(pcaone_gpu_ctx* ctx, const uint8_t* packed, uint64_t nsnps, uint32_t nsamples,
                               uint64_t device_budget, uint32_t buffer_gb) {
  return guarded(ctx, [&](Context& c) {
    if (!packed) throw Error(PCAONE_E_ARG, "null buffer");
    c.stream_budget = device_budget;
    c.stream_buffer_gb = buffer_gb ? buffer_gb : 2;
    pcaone::load_bed_host(c, packed, nsnps, nsamples, true);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_load_bed_file_image_stream(pcaone_gpu_ctx* ctx, const uint8_t* image, uint64_t image_bytes,
                                          uint64_t nsnps, uint32_t nsamples, uint64_t device_budget,
                                          uint32_t buffer_gb) {
  return guarded(ctx, [&](Context& c) {
    check_bed_image(image, image_bytes, nsnps, nsamples);
    c.stream_budget = device_budget;
    c.stream_buffer_gb = buffer_gb ? buffer_gb : 2;
    pcaone::load_bed_host(c, image + 3, nsnps, nsamples, true);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_stream_plan(uint64_t nsnps, uint32_t nsamples, int svd, int bands, uint64_t device_budget,
                           uint64_t* block_snps, uint64_t* nblocks) {
  if (nsnps == 0 || nsamples == 0 || nsnps > 0x7fffffffull || nsamples > 0x7fffff00u) return PCAONE_E_ARG;
  if (svd != PCAONE_SVD_SINGLE && svd != PCAONE_SVD_WINDOW) return PCAONE_E_ARG;
  if (svd == PCAONE_SVD_WINDOW && (bands < 4 || (bands & (bands - 1)) != 0)) return PCAONE_E_ARG;
  const int64_t stride = (((int64_t)nsamples + 127) / 128) * 32;
  const int64_t b = pcaone::stream_block_size((int64_t)nsnps, stride, svd, bands, device_budget);
  if (b <= 0) return PCAONE_E_LIMIT;
  if (block_snps) *block_snps = (uint64_t)b;
  if (nblocks) *nblocks = (nsnps + (uint64_t)b - 1) / (uint64_t)b;
  return PCAONE_OK;
}

int pcaone_gpu_ooc_order(uint64_t nsnps, uint32_t nsamples, int bands, uint32_t buffer_gb, int32_t* order) {
  if (!order || nsnps == 0 || nsamples == 0 || nsnps > 0x7fffffffull || nsamples > 0x7fffff00u) return PCAONE_E_ARG;
  if (bands < 4 || (bands & (bands - 1)) != 0) return PCAONE_E_ARG;
  return pcaone::host_ooc_order((int64_t)nsnps, ((int64_t)nsamples + 3) / 4, buffer_gb ? buffer_gb : 2, bands, order)
             ? PCAONE_OK
             : PCAONE_E_ARG;
}

int pcaone_gpu_stream_info(pcaone_gpu_ctx* ctx, int* streamed, double* bytes_fetched) {
  return guarded(ctx, [&](Context& c) {
    if (streamed) *streamed = c.streamed ? 1 : 0;
    if (bytes_fetched) *bytes_fetched = c.stream_bytes;
    c.stream_bytes = 0;
  });
}

int pcaone_gpu_pgen_layout(const uint8_t* image, uint64_t image_bytes, uint32_t nsamples, int* mode, uint64_t* nsnps,
                           uint32_t* nsamples_out, uint64_t* offset, uint64_t* record_bytes) {
  try {
    const pcaone::PgenLayout l = pcaone::pgen_layout(image, image_bytes, nsamples);
    if (mode) *mode = l.mode;
    if (nsnps) *nsnps = l.nsnps;
    if (nsamples_out) *nsamples_out = l.nsamples;
    if (offset) *offset = l.offset;
    if (record_bytes) *record_bytes = l.pitch;
    return PCAONE_OK;
  } catch (const Error& e) {
    return e.code;
  }
}

int pcaone_gpu_load_pgen_file_image(pcaone_gpu_ctx* ctx, const uint8_t* image, uint64_t image_bytes, uint32_t nsamples) {
  return guarded(ctx, [&](Context& c) {
    const pcaone::PgenLayout l = pcaone::pgen_layout(image, image_bytes, nsamples);
    pcaone::load_bed_host(c, image + l.offset, l.nsnps, l.nsamples, false, l.mode != 0x01, (int64_t)l.pitch);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_load_pgen_genovecs(pcaone_gpu_ctx* ctx, const uint8_t* genovecs, uint64_t row_pitch, uint64_t nsnps,
                                  uint32_t nsamples) {
  return guarded(ctx, [&](Context& c) {
    if (!genovecs) throw Error(PCAONE_E_ARG, "null buffer");
    pcaone::load_bed_host(c, genovecs, nsnps, nsamples, false, true, (int64_t)row_pitch);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_load_dense(pcaone_gpu_ctx* ctx, const float* values, uint64_t nsnps, uint32_t nsamples) {
  return guarded(ctx, [&](Context& c) {
    pcaone::load_dense(c, values, nsnps, nsamples);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_load_synthetic_dense(pcaone_gpu_ctx* ctx, uint64_t nsnps, uint32_t nsamples, int npop,
                                    const double* freq, const double* weights, double sd, uint64_t seed) {
  return guarded(ctx, [&](Context& c) {
    pcaone::load_synthetic_dense(c, nsnps, nsamples, npop, freq, weights, sd, seed);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_load_binary_file_image(pcaone_gpu_ctx* ctx, const uint8_t* image, uint64_t image_bytes) {
  return guarded(ctx, [&](Context& c) {
    // FileBin (src/FileBinary.hpp:17-18): uint32 SNPs, uint32 samples, float32 rows
    if (!image || image_bytes < 8) throw Error(PCAONE_E_FORMAT, "truncated binary image");
    uint32_t hdr[2];
    std::memcpy(hdr, image, 8);
    const uint64_t need = 8 + (uint64_t)hdr[0] * hdr[1] * 4;
    if (image_bytes < need)
      throw Error(PCAONE_E_FORMAT, "truncated binary file: " + std::to_string(image_bytes) + " bytes, expected " +
                                       std::to_string(need));
    if (((uintptr_t)(image + 8) & 3u) != 0) throw Error(PCAONE_E_ARG, "binary image values must be 4-byte aligned");
    pcaone::load_dense(c, reinterpret_cast<const float*>(image + 8), hdr[0], hdr[1]);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_load_bed_device(pcaone_gpu_ctx* ctx, const void* dev_packed, uint64_t src_pitch, uint64_t nsnps,
                               uint32_t nsamples) {
  return guarded(ctx, [&](Context& c) {
    if (!dev_packed) throw Error(PCAONE_E_ARG, "null genotype buffer");
    if (src_pitch < ((uint64_t)nsamples + 3) / 4) throw Error(PCAONE_E_ARG, "row pitch below (N+3)/4");
    pcaone::load_bed_device(c, dev_packed, src_pitch, nsnps, nsamples);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_filter_maf(pcaone_gpu_ctx* ctx, double maf, uint64_t* nkept) {
  return guarded(ctx, [&](Context& c) {
    pcaone::need_data(c);
    const int64_t nk = pcaone::filter_maf(c, maf);
    if (nkept) *nkept = (uint64_t)nk;
  });
}

int pcaone_gpu_kept_snps(pcaone_gpu_ctx* ctx, int64_t* idx) {
  return guarded(ctx, [&](Context& c) {
    pcaone::need_data(c);
    if (!idx) throw Error(PCAONE_E_ARG, "null index buffer");
    for (int64_t i = 0; i < c.M; ++i) idx[i] = c.kept.empty() ? i : c.kept[(size_t)i];
  });
}

int pcaone_gpu_load_synthetic(pcaone_gpu_ctx* ctx, uint64_t nsnps, uint32_t nsamples, int npop, const double* freq,
                              const double* weights, const double* miss_sample, const double* miss_snp,
                              uint64_t seed) {
  return guarded(ctx, [&](Context& c) {
    pcaone::load_synthetic(c, nsnps, nsamples, npop, freq, weights, miss_sample, miss_snp, seed);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_get_bed(pcaone_gpu_ctx* ctx, uint8_t* packed) {
  return guarded(ctx, [&](Context& c) {
    pcaone::need_plink(c);
    if (!packed) throw Error(PCAONE_E_ARG, "null buffer");
    const size_t bps = ((size_t)c.N + 3) / 4;
    PCAONE_CUDA(cudaMemcpy2DAsync(packed, bps, c.rows_ptr(), c.stride, bps, c.M, cudaMemcpyDefault, c.stream));
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_counts(pcaone_gpu_ctx* ctx, int32_t* counts, double* F) {
  return guarded(ctx, [&](Context& c) {
    pcaone::need_plink(c);
    if (counts)
      PCAONE_CUDA(cudaMemcpyAsync(counts, c.counts.p, (size_t)c.M * 4 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                  c.stream));
    if (F) PCAONE_CUDA(cudaMemcpyAsync(F, c.F.p, (size_t)c.M * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_op_init(pcaone_gpu_ctx* ctx, const pcaone_gpu_params* params) {
  return guarded(ctx, [&](Context& c) {
    if (!params) throw Error(PCAONE_E_ARG, "null params");
    pcaone::op_init(c, *params);
  });
}

int pcaone_gpu_set_omega(pcaone_gpu_ctx* ctx, const double* omega, uint32_t rows, uint32_t cols) {
  return guarded(ctx, [&](Context& c) {
    pcaone::set_omega(c, omega, rows, cols);
  });
}

int pcaone_gpu_set_flags(pcaone_gpu_ctx* ctx, int update, int standardize) {
  return guarded(ctx, [&](Context& c) {
    pcaone::need_op(c);
    c.update = update != 0;
    c.standardize = standardize != 0;
  });
}

int pcaone_gpu_compute_g_and_h(pcaone_gpu_ctx* ctx, int pi, double* G, double* H) {
  return guarded(ctx, [&](Context& c) {
    pcaone::need_op(c);
    if (pi < 0) throw Error(PCAONE_E_ARG, "negative epoch");
    pcaone::clear_status(c);
    pcaone::compute_g_and_h(c, pi);
    pcaone::check_status(c);
    pcaone::copy_out(c, c.G.p, c.M, c.LP, c.L, G);
    pcaone::copy_out(c, c.H.p, c.N, c.LP, c.L, H);
    PCAONE_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int pcaone_gpu_compute_usv(pcaone_gpu_ctx* ctx, int p, double tol, double* U, double* S, double* V, int* epochs) {
  return guarded(ctx, [&](Context& c) {
    pcaone::need_op(c);
    const auto t0 = pcaone::clk::now();
    c.t_prod = c.t_qr = c.t_em = 0;
    const int e = pcaone::compute_usv(c, p, tol);
    if (epochs) *epochs = e;
    pcaone::outputs(c, U, S, V);
    c.t_total = pcaone::secs(t0, pcaone::clk::now());
  });
}

int pcaone_gpu_run_halko(pcaone_gpu_ctx* ctx, const pcaone_gpu_params* params, double* U, double* S, double* V,
                         int* em_iters) {
  return guarded(ctx, [&](Context& c) {
    if (!params) throw Error(PCAONE_E_ARG, "null params");
    const auto t0 = pcaone::clk::now();
    c.t_prod = c.t_qr = c.t_em = 0;
    const int it = pcaone::run_halko(c, *params);
    if (em_iters) *em_iters = it;
    pcaone::outputs(c, U, S, V);
    c.t_total = pcaone::secs(t0, pcaone::clk::now());
  });
}

void pcaone_gpu_mlp_default_params(pcaone_gpu_mlp_params* p) {
  if (!p) return;
  p->enable = 1;
  p->train_entries = 524288;
  p->holdout_entries = 65536;
  p->epochs = 4;
  p->batch = 4096;
  p->lr = 1e-3f;
  p->seed = 20251;
}

int pcaone_gpu_set_warm_start(pcaone_gpu_ctx* ctx, const pcaone_gpu_mlp_params* p) {
  return guarded(ctx, [&](Context& c) {
    if (!p || !p->enable) {
      c.warm = pcaone_gpu_mlp_params{};
      return;
    }
    if (p->train_entries < p->batch || p->batch <= 0 || p->epochs < 0 || p->holdout_entries < 0 || !(p->lr > 0.f))
      throw Error(PCAONE_E_ARG, "invalid warm-start parameters");
    c.warm = *p;
  });
}

int pcaone_gpu_mlp_stats(pcaone_gpu_ctx* ctx, double out[6]) {
  return guarded(ctx, [&](Context& c) {
    if (!out) throw Error(PCAONE_E_ARG, "null output");
    for (int i = 0; i < 6; ++i) out[i] = c.warm_stats[i];
  });
}

int pcaone_gpu_mlp_forward_backward(int device, const float* X, const float* y, int B, const float* params,
                                    float* out, float* loss, float* grads) {
  if (!X || !y || !params || !out || !loss || !grads || B <= 0) return PCAONE_E_ARG;
  cudaStream_t s = nullptr;
  try {
    PCAONE_CUDA(cudaSetDevice(device));
    PCAONE_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    {
      pcaone::mlp::Net net(s);
      net.set_params(params);
      net.ensure_batch(B);
      PCAONE_CUDA(cudaMemcpyAsync(net.X(), X, (size_t)B * pcaone::mlp::kIn * sizeof(float), cudaMemcpyHostToDevice, s));
      PCAONE_CUDA(cudaMemcpyAsync(net.y(), y, (size_t)B * sizeof(float), cudaMemcpyHostToDevice, s));
      net.forward(net.X(), B, true);
      net.backward(net.X(), net.y(), B);
      PCAONE_CUDA(cudaMemcpyAsync(out, net.out(), (size_t)B * sizeof(float), cudaMemcpyDeviceToHost, s));
      PCAONE_CUDA(cudaMemcpyAsync(grads, net.grad(), (size_t)pcaone::mlp::kParams * sizeof(float),
                                  cudaMemcpyDeviceToHost, s));
      *loss = net.loss_host() / (float)B;
    }
    cudaStreamDestroy(s);
    return PCAONE_OK;
  } catch (const Error& e) {
    if (s) cudaStreamDestroy(s);
    return e.code;
  } catch (const std::exception&) {
    if (s) cudaStreamDestroy(s);
    return PCAONE_E_ARG;
  }
}

int pcaone_gpu_get_perm(pcaone_gpu_ctx* ctx, int32_t* perm) {
  return guarded(ctx, [&](Context& c) {
    pcaone::need_data(c);
    if (!perm) throw Error(PCAONE_E_ARG, "null perm");
    if (c.permuted)
      std::memcpy(perm, c.perm_host.data(), (size_t)c.M * sizeof(int32_t));
    else
      for (int64_t i = 0; i < c.M; ++i) perm[i] = (int32_t)i;
  });
}

int pcaone_gpu_project(pcaone_gpu_ctx* ctx, const double* F, const double* V, const double* S, int k, int mode,
                       double* U) {
  return guarded(ctx, [&](Context& c) { pcaone::project(c, F, V, S, k, mode, U); });
}

int pcaone_gpu_matvec(pcaone_gpu_ctx* ctx, const double* x, double* y, int standardize) {
  return guarded(ctx, [&](Context& c) {
    if (!x || !y) throw Error(PCAONE_E_ARG, "null vector");
    pcaone::matvec(c, x, y, standardize);
  });
}

}  // extern "C"
