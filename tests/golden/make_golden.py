"""Generate the golden fixtures of tests/golden/ from the reference itself.

Run in a container that has the reference tree (the fixtures are committed;
tests never run this):

    make -C oracle ref REF=<reference tree>   # builds oracle/_ref/ref_driver
    python tests/golden/make_golden.py         # all fixtures
    python tests/golden/make_golden.py --eigs-only   # only tests/golden/eigs/
    python tests/golden/make_golden.py --ooc-only    # only the out-of-core (-m) cases
    python tests/golden/make_golden.py --pgen-only   # only the PLINK2 .pgen cases
    python tests/golden/make_golden.py --maf-only    # only the --maf cases

Each case draws a seeded synthetic PLINK fileset (pcaone_gb300.synthetic),
runs the reference's RSVD operators through oracle/_ref/ref_driver with the
listed PCAone options, and stores the packed genotypes, the options and the
reference's full-precision outputs (F, U, S, V, the column permutation, the
initial random matrix, the EM iteration count and a SHA-256 of the decoded
centred matrix) in <case>.npz.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from pcaone_gb300 import synthetic  # noqa: E402
from tests.cases import pgen_image  # noqa: E402

DRIVER = os.path.join(REPO, "oracle", "_ref", "ref_driver")

# name -> (population model kwargs, PCAone options)
CASES = {
    # odd N (padding lanes carry garbage bits), winSVD with 16 windows
    "wsvd_n301": (dict(nsamples=301, nsnps=2400, npop=3, fst=0.1, seed=11, mcar=0.01, pad_garbage=True),
                  ["-d", "2", "-k", "4", "--maxp", "6", "-w", "16"]),
    # winSVD with the default 64 windows and k=10 (the CLI keeps p=10)
    "wsvd_n500_k10": (dict(nsamples=500, nsnps=4000, npop=3, fst=0.05, seed=12, mcar=0.01),
                      ["-d", "2", "-k", "10", "--maxp", "6"]),
    # winSVD without the column shuffle, uniform random test matrix, 5 PCs
    "wsvd_noshuffle_uniform": (dict(nsamples=256, nsnps=2048, npop=4, fst=0.08, seed=13, mcar=0.02),
                               ["-d", "2", "-S", "-k", "5", "--maxp", "8", "-w", "8", "--rand", "0"]),
    # single-pass RSVD with power iterations
    "ssvd_n203": (dict(nsamples=203, nsnps=1500, npop=3, fst=0.1, seed=5, mcar=0.05, pad_garbage=True),
                  ["-d", "1", "-k", "3", "--maxp", "4"]),
    # EMU on the window method without shuffle (the in-core shuffled EMU path
    # scales permuted columns with unpermuted frequencies, src/Data.cpp:328,355)
    "em_wsvd_noshuffle": (dict(nsamples=203, nsnps=1500, npop=3, fst=0.1, seed=5, mcar=0.05, pad_garbage=True),
                          ["-d", "2", "-S", "--emu", "--maxiter", "8", "--maxp", "6", "-k", "3", "-w", "16"]),
    # EMU on the single-pass method
    "em_ssvd": (dict(nsamples=160, nsnps=1200, npop=3, fst=0.1, seed=7, mcar=0.08),
                ["-d", "1", "--emu", "--maxiter", "5", "--maxp", "3", "-k", "2"]),
}

# --maf: Data::filter_snps_resize_F drops the SNPs with minor allele frequency
# at or below the bound before anything else (src/FilePlink.cpp:61); the
# fixture keeps every row of the file, and keep.npy lists the kept ones
MAF_CASES = {
    # ancestral frequencies from 0.02, so that about a fifth of the SNPs go
    "maf_wsvd_n301": (dict(nsamples=301, nsnps=2400, npop=3, fst=0.1, seed=51, mcar=0.01, anc_range=(0.02, 0.5),
                           pad_garbage=True),
                      ["-d", "2", "-k", "4", "--maxp", "6", "-w", "16", "--maf", "0.1"]),
    "maf_em_ssvd_n203": (dict(nsamples=203, nsnps=1500, npop=3, fst=0.1, seed=52, mcar=0.05, anc_range=(0.02, 0.5)),
                         ["-d", "1", "--emu", "--maxiter", "5", "--maxp", "4", "-k", "3", "--maf", "0.08"]),
}

# Out-of-core runs (-m GB): the reference streams blocks from the .bed file;
# with the window method's shuffle it first rewrites the file in the band
# interleave of permute_plink (src/FilePlink.cpp:303-408, --buffer 2 GB).  The
# budgets give 3 to 5 blocks, which Data::prepare then aligns with the windows.
OOC_CASES = {
    # M a multiple of the windows: each window is one band of the interleave
    "ooc_wsvd_n301": (dict(nsamples=301, nsnps=2400, npop=3, fst=0.1, seed=11, mcar=0.01, pad_garbage=True),
                      ["-d", "2", "-k", "4", "--maxp", "6", "-w", "16", "-m", "0.002"]),
    # M = 1500 over 16 windows: bands of 94 and 93 SNPs, windows of 94 (a last
    # window of 90), and a second buffer block of 12 SNPs in the interleave
    "ooc_em_wsvd_n203": (dict(nsamples=203, nsnps=1500, npop=3, fst=0.1, seed=5, mcar=0.05, pad_garbage=True),
                         ["-d", "2", "--emu", "--maxiter", "8", "--maxp", "6", "-k", "3", "-w", "16", "-m",
                          "0.0015"]),
    "ooc_ssvd_n203": (dict(nsamples=203, nsnps=1500, npop=3, fst=0.1, seed=5, mcar=0.05, pad_garbage=True),
                      ["-d", "1", "-k", "3", "--maxp", "4", "-m", "0.0015"]),
}


def run_ooc_case(name: str, model_kw: dict, opts: list) -> dict:
    kw = dict(model_kw)
    pad_garbage = kw.pop("pad_garbage", False)
    model = synthetic.draw_population_model(**kw)
    packed = synthetic.sample_packed_bed(model, pad_garbage=pad_garbage)
    with tempfile.TemporaryDirectory() as td:
        prefix = os.path.join(td, name)
        synthetic.write_plink(prefix, packed, model.nsamples)
        out = os.path.join(td, "out")
        os.makedirs(out)
        env = dict(os.environ, OMP_NUM_THREADS="1")
        subprocess.check_call([DRIVER, out, "-b", prefix] + opts, env=env)
        res = {k: np.load(os.path.join(out, k + ".npy")) for k in ("U", "S", "V", "Omg0", "meta")}
        if os.path.exists(os.path.join(out, "perm.npy")):
            res["perm"] = np.load(os.path.join(out, "perm.npy"))
    res["packed"] = packed
    res["options"] = np.array(json.dumps(opts))
    return res


# PLINK2 input (-p prefix), read by the reference's pgenlib: fixed-width
# .pgen files (storage mode 0x02: a 12-byte header -- magic, mode, variant
# count, sample count, control byte -- then one record of ceil(N/4) bytes per
# variant, 2-bit ALT allele counts, 3 = missing), with a .psam listing the samples
PGEN_CASES = {
    "pgen_wsvd_n301": (dict(nsamples=301, nsnps=2400, npop=3, fst=0.1, seed=31, mcar=0.01),
                       ["-d", "2", "-k", "4", "--maxp", "6", "-w", "16"]),
    "pgen_em_ssvd_n203": (dict(nsamples=203, nsnps=1500, npop=3, fst=0.1, seed=32, mcar=0.05),
                          ["-d", "1", "--emu", "--maxiter", "5", "--maxp", "4", "-k", "3"]),
}


def bed_to_genovec(packed: np.ndarray, nsamples: int) -> np.ndarray:
    """PLINK 1 codes -> PLINK 2 hard calls (ALT allele counts, A1 = ALT):
    00 -> 2, 10 -> 1, 11 -> 0, 01 (missing) -> 3; padding lanes zero."""
    p = np.asarray(packed, dtype=np.uint8)
    out = np.zeros_like(p)
    lut = np.array([2, 3, 1, 0], dtype=np.uint8)
    for s in range(4):
        out |= lut[(p >> (2 * s)) & 3] << (2 * s)
    nb = (nsamples + 3) // 4
    if nsamples % 4:
        out[:, nb - 1] &= np.uint8((1 << (2 * (nsamples % 4))) - 1)
    return out


def run_pgen_case(name: str, model_kw: dict, opts: list) -> dict:
    model = synthetic.draw_population_model(**model_kw)
    packed = synthetic.sample_packed_bed(model)
    genovec = bed_to_genovec(packed, model.nsamples)
    with tempfile.TemporaryDirectory() as td:
        prefix = os.path.join(td, name)
        with open(prefix + ".pgen", "wb") as f:
            f.write(pgen_image(genovec, model.nsamples))
        with open(prefix + ".psam", "w") as f:
            f.write("#IID\n" + "".join(f"s{i}\n" for i in range(model.nsamples)))
        out = os.path.join(td, "out")
        os.makedirs(out)
        env = dict(os.environ, OMP_NUM_THREADS="1")
        subprocess.check_call([DRIVER, out, "--dump-g0", "-p", prefix] + opts, env=env)
        res = {k: np.load(os.path.join(out, k + ".npy")) for k in ("F", "U", "S", "V", "Omg0", "meta")}
        g0 = np.load(os.path.join(out, "G0.npy"))
        res["G0_sha256"] = np.frombuffer(hashlib.sha256(np.asfortranarray(g0).tobytes(order="F")).digest(),
                                         dtype=np.uint8)
        if os.path.exists(os.path.join(out, "perm.npy")):
            res["perm"] = np.load(os.path.join(out, "perm.npy"))
    res["genovec"] = genovec
    res["options"] = np.array(json.dumps(opts))
    return res


# FileBinary input (-B; per-SNP mean centring only, -C 0): continuous dosages
# stored as float16 (synthetic.sample_dosages), written as the float32 matrix
BINARY_CASES = {
    "bin_wsvd_n301": (dict(nsamples=301, nsnps=2400, npop=3, fst=0.1, seed=21),
                      ["-d", "2", "-C", "0", "-k", "4", "--maxp", "6", "-w", "16"]),
    "bin_ssvd_n256": (dict(nsamples=256, nsnps=1800, npop=4, fst=0.08, seed=22),
                      ["-d", "1", "-C", "0", "-k", "3", "--maxp", "4"]),
}


def run_case(name: str, model_kw: dict, opts: list) -> dict:
    kw = dict(model_kw)
    pad_garbage = kw.pop("pad_garbage", False)
    model = synthetic.draw_population_model(**kw)
    packed = synthetic.sample_packed_bed(model, pad_garbage=pad_garbage)
    with tempfile.TemporaryDirectory() as td:
        prefix = os.path.join(td, name)
        synthetic.write_plink(prefix, packed, model.nsamples)
        out = os.path.join(td, "out")
        os.makedirs(out)
        env = dict(os.environ, OMP_NUM_THREADS="1")
        subprocess.check_call([DRIVER, out, "--dump-g0", "-b", prefix] + opts, env=env)
        res = {k: np.load(os.path.join(out, k + ".npy")) for k in ("F", "U", "S", "V", "Omg0", "meta")}
        g0 = np.load(os.path.join(out, "G0.npy"))
        res["G0_sha256"] = np.frombuffer(hashlib.sha256(np.asfortranarray(g0).tobytes(order="F")).digest(),
                                         dtype=np.uint8)
        if os.path.exists(os.path.join(out, "perm.npy")):
            res["perm"] = np.load(os.path.join(out, "perm.npy"))
        if os.path.exists(os.path.join(out, "keep.npy")):
            res["keep"] = np.load(os.path.join(out, "keep.npy"))
    res["packed"] = packed
    res["options"] = np.array(json.dumps(opts))
    return res


def run_binary_case(name: str, model_kw: dict, opts: list) -> dict:
    model = synthetic.draw_population_model(**model_kw)
    dense = synthetic.sample_dosages(model)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, name + ".bin")
        synthetic.write_binary(path, dense)
        out = os.path.join(td, "out")
        os.makedirs(out)
        env = dict(os.environ, OMP_NUM_THREADS="1")
        subprocess.check_call([DRIVER, out, "--dump-g0", "-B", path] + opts, env=env)
        res = {k: np.load(os.path.join(out, k + ".npy")) for k in ("U", "S", "V", "Omg0", "meta")}
        g0 = np.load(os.path.join(out, "G0.npy"))
        res["G0_sha256"] = np.frombuffer(hashlib.sha256(np.asfortranarray(g0).tobytes(order="F")).digest(),
                                         dtype=np.uint8)
        if os.path.exists(os.path.join(out, "perm.npy")):
            res["perm"] = np.load(os.path.join(out, "perm.npy"))
    res["dense"] = dense
    res["options"] = np.array(json.dumps(opts))
    return res


# projection of new samples (--project 1 and 2): the first n_base samples of
# one model are fitted, the rest are projected (same SNPs, 2% missing)
PROJECTION_CASES = {
    "proj_wsvd_n400": (dict(nsamples=520, nsnps=3000, npop=3, fst=0.1, seed=41, mcar=0.02), 400,
                       ["-d", "2", "-k", "4", "--maxp", "6", "-w", "16"]),
}


def run_projection_case(name: str, model_kw: dict, n_base: int, opts: list) -> dict:
    model = synthetic.draw_population_model(**model_kw)
    code = synthetic.sample_codes(model, 0, model.nsnps)
    packed = synthetic.pack_codes(code[:, :n_base])
    packed_new = synthetic.pack_codes(code[:, n_base:])
    with tempfile.TemporaryDirectory() as td:
        base, new = os.path.join(td, name), os.path.join(td, name + "_new")
        synthetic.write_plink(base, packed, n_base)
        synthetic.write_plink(new, packed_new, model.nsamples - n_base)
        out = os.path.join(td, "out")
        os.makedirs(out)
        env = dict(os.environ, OMP_NUM_THREADS="1")
        subprocess.check_call([DRIVER, out, "--dump-g0", "--project-new", new, "-b", base] + opts, env=env)
        res = {k: np.load(os.path.join(out, k + ".npy")) for k in ("F", "U", "S", "V", "Omg0", "meta", "P1", "P2")}
        g0 = np.load(os.path.join(out, "G0.npy"))
        res["G0_sha256"] = np.frombuffer(hashlib.sha256(np.asfortranarray(g0).tobytes(order="F")).digest(),
                                         dtype=np.uint8)
        if os.path.exists(os.path.join(out, "perm.npy")):
            res["perm"] = np.load(os.path.join(out, "perm.npy"))
    res["packed"] = packed
    res["packed_new"] = packed_new
    res["n_new"] = np.array(model.nsamples - n_base)
    res["options"] = np.array(json.dumps(opts))
    return res


# the reference's own text outputs (Data::write_eigs_files, src/Data.cpp:211-240:
# .sigvals, .eigvals = S^2/M, .eigvecs = U, .loadings = V in file SNP order,
# 6 significant digits) for two of the cases above: shuffled winSVD, and EM
# (whose outputs pass through flip_UV)
EIGS_CASES = ("wsvd_n301", "em_wsvd_noshuffle")
EIGS_DIR = os.path.join(HERE, "eigs")


def run_eigs_case(name: str) -> None:
    kw = dict(CASES[name][0])
    opts = CASES[name][1]
    pad_garbage = kw.pop("pad_garbage", False)
    model = synthetic.draw_population_model(**kw)
    packed = synthetic.sample_packed_bed(model, pad_garbage=pad_garbage)
    os.makedirs(EIGS_DIR, exist_ok=True)
    with tempfile.TemporaryDirectory() as td:
        prefix = os.path.join(td, name)
        synthetic.write_plink(prefix, packed, model.nsamples)
        out = os.path.join(td, "out")
        os.makedirs(out)
        env = dict(os.environ, OMP_NUM_THREADS="1")
        subprocess.check_call([DRIVER, out, "--eigs-files", "-b", prefix, "-o", os.path.join(out, name), "-V"] + opts,
                              env=env)
        for ext in ("sigvals", "eigvals", "eigvecs", "loadings"):
            with open(os.path.join(out, name + "." + ext)) as f, open(os.path.join(EIGS_DIR, name + "." + ext),
                                                                          "w") as g:
                g.write(f.read())
    print(name, "text outputs written to", EIGS_DIR)


def main() -> None:
    if not os.path.exists(DRIVER):
        sys.exit("build the reference driver first: make -C oracle ref")
    if "--eigs-only" in sys.argv:
        for name in EIGS_CASES:
            run_eigs_case(name)
        return
    if "--pgen-only" in sys.argv:
        for name, (mkw, opts) in PGEN_CASES.items():
            res = run_pgen_case(name, mkw, opts)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
            print(name, "N=%d M=%d" % (res["meta"][0], res["meta"][1]), "S=", res["S"])
        return
    if "--maf-only" in sys.argv:
        for name, (mkw, opts) in MAF_CASES.items():
            res = run_case(name, mkw, opts)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
            print(name, "N=%d M=%d" % (res["meta"][0], res["meta"][1]), "kept", len(res["keep"]), "S=", res["S"])
        return
    if "--ooc-only" in sys.argv:
        for name, (mkw, opts) in OOC_CASES.items():
            res = run_ooc_case(name, mkw, opts)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
            print(name, "N=%d M=%d" % (res["meta"][0], res["meta"][1]), "S=", res["S"])
        return
    for name, (mkw, opts) in CASES.items():
        res = run_case(name, mkw, opts)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print(name, "N=%d M=%d" % (res["meta"][0], res["meta"][1]), "S=", res["S"])
    for name, (mkw, opts) in BINARY_CASES.items():
        res = run_binary_case(name, mkw, opts)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print(name, "N=%d M=%d" % (res["meta"][0], res["meta"][1]), "S=", res["S"])
    for name, (mkw, nb, opts) in PROJECTION_CASES.items():
        res = run_projection_case(name, mkw, nb, opts)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print(name, "N=%d M=%d" % (res["meta"][0], res["meta"][1]), "S=", res["S"], "P2[0]=", res["P2"][0])
    for name, (mkw, opts) in PGEN_CASES.items():
        res = run_pgen_case(name, mkw, opts)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print(name, "N=%d M=%d" % (res["meta"][0], res["meta"][1]), "S=", res["S"])
    for name, (mkw, opts) in OOC_CASES.items():
        res = run_ooc_case(name, mkw, opts)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print(name, "N=%d M=%d" % (res["meta"][0], res["meta"][1]), "S=", res["S"])
    for name, (mkw, opts) in MAF_CASES.items():
        res = run_case(name, mkw, opts)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print(name, "N=%d M=%d" % (res["meta"][0], res["meta"][1]), "kept", len(res["keep"]), "S=", res["S"])
    for name in EIGS_CASES:
        run_eigs_case(name)


if __name__ == "__main__":
    main()
