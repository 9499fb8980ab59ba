// Test infrastructure only: a small driver linked against the reference's own
// sources (compiled by oracle/Makefile from the read-only reference tree).  It
// runs the reference's RSVD operators exactly as src/Halko.cpp:271-345 does,
// but writes U, S, V, F and the column permutation at full double precision
// (the reference's text writers keep 6 significant digits, src/Data.cpp:215).
//
// usage: ref_driver OUTDIR [driver options] <PCAone command-line options,
//        e.g. -b prefix -k 10 -d 2> (PLINK -b input, PLINK2 -p input read by the
//        reference's pgenlib, or FileBinary -B input with -C 0)
//
// Driver options:
//   --dump-g0             also write G0.npy (below)
//   --project-new PREFIX  also write P1.npy, P2.npy (below)
//   --force-oversamples P run with P oversamples although the CLI raises them to
//                         at least k (src/Cmd.cpp:216): the field of the parsed
//                         Param is set before the operator is built; the
//                         reference's code is unchanged
//   --eigs-files          also write the reference's text outputs through
//                         Data::write_eigs_files (src/Data.cpp:211-240) as
//                         src/Halko.cpp:339 does (needs -o PREFIX; -V for the
//                         .loadings)
//   --timing              write no arrays; print one JSON line with the wall
//                         time of prepare() (read, allele frequencies, decode)
//                         and of the RSVD (operator construction, shuffle and
//                         computeUSV), and the OpenMP thread count
//
// Outputs (numpy .npy, float64 column-major / int64):
//   F.npy         allele frequencies after the AF pass (src/FilePlink.cpp:33-62; PLINK only)
//   U.npy S.npy V.npy   final operator state (src/Halko.cpp:46-97)
//   perm.npy      the column permutation, if any: in core that of
//                 src/RSVD.hpp:61-78; out of core (-m with the window
//                 method's shuffle) that of permute_plink
//                 (src/FilePlink.cpp:303-408, as src/Main.cpp:120-130 runs it)
//   Omg0.npy      the initial random test matrix (src/Halko.cpp:15-23)
//   G0.npy        optional (--dump-g0 as first option): the decoded, centred
//                 matrix before standardisation (N x M), small inputs only
//   P1.npy P2.npy optional (--project-new PREFIX): scores of the samples of a
//                 second PLINK fileset (same SNPs) projected onto the fit, by
//                 --project 1 (U = G V S^-1) and 2 (per-sample least squares
//                 over observed SNPs, solve_projection_scores), with the new
//                 genotypes decoded and standardised with the fit's F as
//                 run_projection does (src/Projection.cpp:236-247,
//                 src/Data.cpp:17-32)
#define _DECLARE_TOOLBOX_HERE
#include <omp.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "FileBinary.hpp"
#include "FilePgen.hpp"
#include "FilePlink.hpp"
#include "Halko.hpp"
#include "Projection.hpp"
#include "Utils.hpp"

namespace {

void write_npy(const std::string& path, const char* descr, const void* data, size_t elem,
               std::vector<long long> shape, bool fortran) {
  std::string hdr = std::string("{'descr': '") + descr + "', 'fortran_order': " +
                    (fortran ? "True" : "False") + ", 'shape': (";
  for (size_t i = 0; i < shape.size(); ++i) hdr += std::to_string(shape[i]) + ", ";
  hdr += "), }";
  size_t total = 10 + hdr.size() + 1;
  size_t pad = (64 - total % 64) % 64;
  hdr.append(pad, ' ');
  hdr += '\n';
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  const char magic[] = "\x93NUMPY\x01\x00";
  std::fwrite(magic, 1, 8, f);
  uint16_t hl = (uint16_t)hdr.size();
  std::fwrite(&hl, 2, 1, f);
  std::fwrite(hdr.data(), 1, hdr.size(), f);
  size_t n = 1;
  for (auto s : shape) n *= (size_t)s;
  std::fwrite(data, elem, n, f);
  std::fclose(f);
}

void dump(const std::string& dir, const char* name, const Mat2D& m) {
  write_npy(dir + "/" + name + ".npy", "<f8", m.data(), 8, {(long long)m.rows(), (long long)m.cols()}, true);
}
void dump1(const std::string& dir, const char* name, const Mat1D& v) {
  write_npy(dir + "/" + name + ".npy", "<f8", v.data(), 8, {(long long)v.size()}, false);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s OUTDIR [--dump-g0] <PCAone options>\n", argv[0]);
    return 2;
  }
  std::string outdir = argv[1];
  bool dump_g0 = false, timing = false, eigs_files = false;
  int force_os = -1;
  std::string project_new;
  std::vector<char*> args;
  args.push_back(argv[0]);
  for (int i = 2; i < argc; ++i) {
    if (std::strcmp(argv[i], "--dump-g0") == 0) {
      dump_g0 = true;
      continue;
    }
    if (std::strcmp(argv[i], "--project-new") == 0 && i + 1 < argc) {
      project_new = argv[++i];
      continue;
    }
    if (std::strcmp(argv[i], "--force-oversamples") == 0 && i + 1 < argc) {
      force_os = std::atoi(argv[++i]);
      continue;
    }
    if (std::strcmp(argv[i], "--eigs-files") == 0) {
      eigs_files = true;
      continue;
    }
    if (std::strcmp(argv[i], "--timing") == 0) {
      timing = true;
      continue;
    }
    args.push_back(argv[i]);
  }
  Param params((int)args.size(), args.data());
  if (force_os >= 0) params.oversamples = force_os;
  cao.cao.open(outdir + "/ref.log");
  cao.is_screen = false;
  if (params.file_t != FileType::PLINK && params.file_t != FileType::BINARY && params.file_t != FileType::PGEN) {
    std::fprintf(stderr, "only PLINK, PGEN and binary input are driven here\n");
    return 2;
  }
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  // out-of-core (-m) with the window method's shuffle: the reference rewrites
  // the .bed in its structured order first and runs on that file
  // (src/Main.cpp:120-130); the rewritten files go to OUTDIR/ooc.perm.*
  const bool ooc_permutation = params.perm && params.out_of_core && params.file_t == FileType::PLINK;
  PermMat ooc_perm;
  if (ooc_permutation) ooc_perm = permute_plink(params.filein, outdir + "/ooc", params.buffer, params.bands);
  Data* data = params.file_t == FileType::PLINK  ? (Data*)new FileBed(params)
               : params.file_t == FileType::PGEN ? (Data*)new FilePgen(params)
                                                 : (Data*)new FileBin(params);
  if (ooc_permutation) data->perm = ooc_perm;
  data->prepare();
  const auto t1 = clk::now();
  if (timing) dump_g0 = false;
  if ((params.file_t == FileType::PLINK || params.file_t == FileType::PGEN) && !timing) dump1(outdir, "F", data->F);
  if (!data->keepSNPs.empty() && !timing) {
    // --maf: the file rows of the SNPs kept by Data::filter_snps_resize_F
    std::vector<long long> keep(data->keepSNPs.begin(), data->keepSNPs.end());
    write_npy(outdir + "/keep.npy", "<i8", keep.data(), 8, {(long long)keep.size()}, false);
  }
  if (dump_g0) dump(outdir, "G0", data->G);

  // operator selection and call sequence of run_pca_with_halko (src/Halko.cpp:271-320)
  RsvdOpData* rsvd;
  if (params.svd_t == SvdType::PCAoneAlg2)
    rsvd = new FancyRsvdOpData(data, params.k, params.oversamples);
  else
    rsvd = new NormalRsvdOpData(data, params.k, params.oversamples);
  if (!timing) dump(outdir, "Omg0", rsvd->Omg);
  int em_iters = 0;
  if (!params.missme) {
    rsvd->setFlags(false, params.ld ? false : true);
    rsvd->computeUSV(params.maxp, params.tol);
  } else {
    rsvd->setFlags(false, false);
    rsvd->computeUSV(params.maxp, params.tol);
    flip_UV(rsvd->U, rsvd->V, false);
    for (uint i = 0; i < params.maxiter; ++i) {
      rsvd->setFlags(true, false);
      Mat2D Vpre = rsvd->V;
      rsvd->computeUSV(params.maxp, params.tol);
      flip_UV(rsvd->U, rsvd->V, false);
      double diff = params.mev ? 1.0 - mev(rsvd->V, Vpre) : minSSE(rsvd->V, Vpre).sum() / Vpre.cols();
      em_iters = (int)i + 1;
      if (diff < params.tolem) break;
    }
    if (params.emu) {
      rsvd->setFlags(true, true);
      rsvd->computeUSV(params.maxp, params.tol);
      flip_UV(rsvd->U, rsvd->V, false);
    }
  }
  const auto t2 = clk::now();
  if (timing) {
    std::printf("{\"prepare_s\": %.6f, \"rsvd_s\": %.6f, \"total_s\": %.6f, \"threads\": %d, \"nsamples\": %lld, "
                "\"nsnps\": %lld, \"k\": %d, \"oversamples\": %d, \"em_iters\": %d, \"S0\": %.17g}\n",
                std::chrono::duration<double>(t1 - t0).count(), std::chrono::duration<double>(t2 - t1).count(),
                std::chrono::duration<double>(t2 - t0).count(), omp_get_max_threads(), (long long)data->nsamples,
                (long long)data->nsnps, (int)params.k, (int)params.oversamples, em_iters, (double)rsvd->S(0));
    delete rsvd;
    delete data;
    return 0;
  }
  if (eigs_files) data->write_eigs_files(rsvd->S.array().square() / data->nsnps, rsvd->S, rsvd->U, rsvd->V);
  dump(outdir, "U", rsvd->U);
  dump1(outdir, "S", rsvd->S);
  dump(outdir, "V", rsvd->V);
  if (data->perm.indices().size() > 0) {
    std::vector<long long> p(data->perm.indices().size());
    for (size_t i = 0; i < p.size(); ++i) p[i] = data->perm.indices()[i];
    write_npy(outdir + "/perm.npy", "<i8", p.data(), 8, {(long long)p.size()}, false);
  }
  if (!project_new.empty()) {
    // loadings in file order (the un-permutation of Data::write_eigs_files)
    Mat2D Vf = rsvd->V;
    if (params.perm && data->perm.indices().size() == (Eigen::Index)data->nsnps)
      for (Eigen::Index logical = 0; logical < (Eigen::Index)data->nsnps; ++logical)
        Vf.row(data->perm.indices()[logical]) = rsvd->V.row(logical);
    // the same options with the new fileset (Param is not copyable)
    std::vector<char*> args2(args);
    for (size_t i = 0; i + 1 < args2.size(); ++i)
      if (std::strcmp(args2[i], "-b") == 0) args2[i + 1] = const_cast<char*>(project_new.c_str());
    Param p2((int)args2.size(), args2.data());
    p2.dopca = false;
    p2.missme = true;
    FileBed* nd = new FileBed(p2);
    nd->F = data->F;  // the fit's allele frequencies (read from the .mbim in run_projection)
    nd->read_all();
    nd->standardize_E();
    const int K = (int)rsvd->S.size() < (int)params.k ? (int)rsvd->S.size() : (int)params.k;
    const Mat1D S = rsvd->S.head(K);
    const Mat2D V = Vf.leftCols(K);
    Mat2D P1 = nd->G * (V * S.array().inverse().matrix().asDiagonal());
    Mat2D P2(nd->nsamples, K);
    solve_projection_scores(V * S.asDiagonal(), nd->C, nd->G, P2);
    dump(outdir, "P1", P1);
    dump(outdir, "P2", P2);
    delete nd;
  }
  std::vector<long long> meta = {(long long)data->nsamples, (long long)data->nsnps, em_iters};
  write_npy(outdir + "/meta.npy", "<i8", meta.data(), 8, {3}, false);
  delete rsvd;
  delete data;
  return 0;
}
