"""Pin the oracle (CPU restatement) against the reference's own outputs.

The fixtures in tests/golden/ were produced by the reference compiled from
its sources (tests/golden/make_golden.py).  These tests need no GPU.
"""
import hashlib
import platform

import numpy as np
import pytest

from oracle import halko as H
from tests.cases import align_signs, golden_cases, pgen_cases

CASES = golden_cases()
IDS = [c.name for c in CASES]


def _oracle_run(case, omega0=None):
    o = case.opts
    d = H.OracleData(case.packed, case.nsamples, emu=o.emu, perm=o.perm, seed=o.seed,
                     bands=o.bands, rand=o.rand, svd_t=o.svd, omega0=omega0)
    op = H.run_pca_with_halko(d, o.k, o.oversamples, maxp=o.maxp, tol=o.tol,
                              maxiter=o.maxiter, tolem=o.tolem)
    return d, op


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_decode_and_allele_freq_bit_exact(case):
    counts = H.bed_counts(case.packed, case.nsamples)
    assert counts.sum(axis=1).tolist() == [case.nsamples] * case.nsnps
    F = H.allele_freq(counts)
    assert np.array_equal(F, case.ref["F"])          # bit-exact
    G0, _ = H.decode_centered(case.packed, case.nsamples, F)
    digest = hashlib.sha256(np.asfortranarray(G0).tobytes(order="F")).digest()
    assert digest == bytes(case.ref["G0_sha256"])    # bit-exact decode + centring


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_column_permutation(case):
    if not case.opts.perm:
        assert "perm" not in case.ref
        return
    assert np.array_equal(H.shuffle_columns(case.nsnps), case.ref["perm"])


@pytest.mark.skipif(platform.machine() != "x86_64",
                    reason="fixtures were drawn on x86-64, where -march=native contracts the "
                           "normal_distribution arithmetic differently than on Arm")
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_random_omega_bit_exact(case):
    o = case.opts
    Om = H.random_omega(o.seed, case.nsamples, o.L, gaussian=bool(o.rand))
    assert np.array_equal(Om, case.ref["Omg0"])


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_rsvd_matches_reference(case):
    """Same Omega, same schedule, FP64: the restatement agrees with the reference
    to rounding (1e-9 relative on eigenvalues and singular vectors)."""
    d, op = _oracle_run(case, omega0=case.ref["Omg0"])
    if case.opts.emu:
        assert op.em_iters == int(case.ref["meta"][2])
    S = case.ref["S"]
    assert np.max(np.abs(op.S ** 2 - S ** 2) / S ** 2) < 1e-9
    U = align_signs(op.U, case.ref["U"])
    V = align_signs(op.V, case.ref["V"])
    assert np.max(np.abs(U - case.ref["U"])) < 1e-8
    assert np.max(np.abs(V - case.ref["V"])) < 1e-8


def test_bed_counts_edge_cases():
    # all-missing SNP -> F = 0 (src/FilePlink.cpp:51-54); monomorphic SNPs; N=1
    code = np.array([[1, 1, 1, 1, 1], [0, 0, 0, 0, 0], [3, 3, 3, 3, 3], [2, 1, 0, 3, 1]], dtype=np.uint8)
    from pcaone_gb300.synthetic import pack_codes
    packed = pack_codes(code, pad_garbage=True, seed=3)
    cnt = H.bed_counts(packed, 5)
    assert cnt.tolist() == [[0, 5, 0, 0], [5, 0, 0, 0], [0, 0, 0, 5], [1, 2, 1, 1]]
    F = H.allele_freq(cnt)
    assert F.tolist() == [0.0, 1.0, 0.0, (1 + 0.5) / 3]
    one = pack_codes(np.array([[2]], dtype=np.uint8))
    assert H.allele_freq(H.bed_counts(one, 1)).tolist() == [0.5]


# ---- FileBinary input (-B, -C 0): the oracle against the reference ----
from tests.cases import binary_cases  # noqa: E402

BIN_CASES = binary_cases()
BIN_IDS = [c.name for c in BIN_CASES]


def _oracle_dense(case, omega0=None):
    o = case.opts
    assert o.scale == 0
    d = H.OracleData.from_dense(case.dense, perm=o.perm, seed=o.seed, bands=o.bands, rand=o.rand, svd_t=o.svd,
                                omega0=omega0)
    op = H.run_pca_with_halko(d, o.k, o.oversamples, maxp=o.maxp, tol=o.tol, maxiter=0)
    return d, op


@pytest.mark.parametrize("case", BIN_CASES, ids=BIN_IDS)
def test_binary_centring_bit_exact(case):
    """FileBin::read_all (src/FileBinary.cpp:54-64): float32 values, each SNP
    centred by its float64 mean."""
    d = H.OracleData.from_dense(case.dense)
    digest = hashlib.sha256(np.asfortranarray(d.G).tobytes(order="F")).digest()
    assert digest == bytes(case.ref["G0_sha256"])


@pytest.mark.parametrize("case", BIN_CASES, ids=BIN_IDS)
def test_binary_rsvd_matches_reference(case):
    d, op = _oracle_dense(case, omega0=case.ref["Omg0"])
    S = case.ref["S"]
    assert np.max(np.abs(op.S ** 2 - S ** 2) / S ** 2) < 1e-9
    assert np.max(np.abs(align_signs(op.U, case.ref["U"]) - case.ref["U"])) < 1e-8
    assert np.max(np.abs(align_signs(op.V, case.ref["V"]) - case.ref["V"])) < 1e-8
    if case.opts.perm:
        assert np.array_equal(H.shuffle_columns(case.nsnps), case.ref["perm"])


# ---- projection of new samples (--project 1 and 2) ----
PROJ_CASES = [c for c in CASES if "P2" in c.ref]


@pytest.mark.parametrize("case", PROJ_CASES, ids=[c.name for c in PROJ_CASES])
def test_projection_matches_reference(case):
    """run_projection with the fit's F, V (file order) and S: mode 1 and the
    per-sample least squares of mode 2 agree with the reference to rounding."""
    k = case.opts.k
    V = case.ref["V"][:, :k]
    if case.opts.perm:
        Vf = np.empty_like(V)
        Vf[case.ref["perm"]] = V
        V = Vf
    S = case.ref["S"][:k]
    n_new = int(case.ref["n_new"])
    for mode, key in ((1, "P1"), (2, "P2")):
        P = H.project(case.ref["packed_new"], n_new, case.ref["F"], V, S, mode)
        assert np.max(np.abs(P - case.ref[key])) <= 1e-10 * max(1.0, np.max(np.abs(case.ref[key]))), mode


# ---- out-of-core (-m) runs of the reference -------------------------------
OOC_CASES = golden_cases(out_of_core=True)
OOC_IDS = [c.name for c in OOC_CASES]


@pytest.mark.parametrize("case", OOC_CASES, ids=OOC_IDS)
def test_out_of_core_order(case):
    """The order permute_plink gives the rewritten .bed (src/FilePlink.cpp:303-408),
    restated by the oracle and by the library (pcaone_gpu_ooc_order), against the
    reference's own permutation; the single-pass method does not shuffle."""
    if not case.opts.perm:
        assert "perm" not in case.ref
        return
    order = H.permute_plink_order(case.nsnps, case.nsamples, case.opts.bands)
    assert np.array_equal(order, case.ref["perm"])
    from pcaone_gb300 import build as B
    from pcaone_gb300 import capi
    import os
    if not os.path.exists(capi.LIBPATH):
        B.build()
    assert np.array_equal(capi.ooc_order(case.nsnps, case.nsamples, case.opts.bands), case.ref["perm"])


@pytest.mark.parametrize("case", OOC_CASES, ids=OOC_IDS)
def test_out_of_core_rsvd_matches_reference(case):
    """The reference's out-of-core run equals the in-core computation on the
    rewritten matrix without the in-core shuffle: its windows are the in-core
    ones when Data::prepare aligns the blocks with them (bandFactor 1,
    src/Data.cpp:66-77), and the file's own allele frequencies keep the EM fill
    consistent.  The restatement on the rows in permute_plink order agrees to
    rounding."""
    o = case.opts
    packed = case.packed[case.ref["perm"]] if "perm" in case.ref else case.packed
    d = H.OracleData(packed, case.nsamples, emu=o.emu, perm=False, seed=o.seed, bands=o.bands, rand=o.rand,
                     svd_t=o.svd, omega0=case.ref["Omg0"])
    op = H.run_pca_with_halko(d, o.k, o.oversamples, maxp=o.maxp, tol=o.tol, maxiter=o.maxiter, tolem=o.tolem)
    if o.emu:
        assert op.em_iters == int(case.ref["meta"][2])
    S = case.ref["S"]
    assert np.max(np.abs(op.S ** 2 - S ** 2) / S ** 2) < 1e-9
    assert np.max(np.abs(align_signs(op.U, case.ref["U"]) - case.ref["U"])) < 1e-8
    assert np.max(np.abs(align_signs(op.V, case.ref["V"]) - case.ref["V"])) < 1e-8


# ---- PLINK2 .pgen input (the reference's FilePgen through its pgenlib) -----
PGEN = pgen_cases()


@pytest.mark.parametrize("case", PGEN, ids=[c.name for c in PGEN])
def test_pgen_hard_calls_as_plink1_codes(case):
    """The hard calls translated to PLINK 1 codes give the reference's PGEN
    allele frequencies and decoded, centred matrix bit for bit, and its PCs to
    rounding."""
    packed = H.genovec_to_bed(case.packed, case.nsamples)
    F = H.allele_freq(H.bed_counts(packed, case.nsamples))
    assert np.array_equal(F, case.ref["F"])
    G0, _ = H.decode_centered(packed, case.nsamples, F)
    assert hashlib.sha256(np.asfortranarray(G0).tobytes(order="F")).digest() == bytes(case.ref["G0_sha256"])
    o = case.opts
    d = H.OracleData(packed, case.nsamples, emu=o.emu, perm=o.perm, seed=o.seed, bands=o.bands, rand=o.rand,
                     svd_t=o.svd, omega0=case.ref["Omg0"])
    op = H.run_pca_with_halko(d, o.k, o.oversamples, maxp=o.maxp, tol=o.tol, maxiter=o.maxiter, tolem=o.tolem)
    if o.emu:
        assert op.em_iters == int(case.ref["meta"][2])
    S = case.ref["S"]
    assert np.max(np.abs(op.S ** 2 - S ** 2) / S ** 2) < 1e-9
    assert np.max(np.abs(align_signs(op.U, case.ref["U"]) - case.ref["U"])) < 1e-8
    assert np.max(np.abs(align_signs(op.V, case.ref["V"]) - case.ref["V"])) < 1e-8


# ---- --maf: Data::filter_snps_resize_F before the run ----
MAF = golden_cases(maf=True)


@pytest.mark.parametrize("case", MAF, ids=[c.name for c in MAF])
def test_maf_filter_matches_reference(case):
    """The kept rows (keepSNPs), their allele frequencies, decoded matrix,
    shuffle and PCs equal the reference's --maf run."""
    F_all = H.allele_freq(H.bed_counts(case.packed, case.nsamples))
    keep = H.maf_keep(F_all, case.opts.maf)
    assert np.array_equal(keep, case.ref["keep"])
    assert 0 < keep.size < case.nsnps and keep.size == int(case.ref["meta"][1])
    assert np.array_equal(F_all[keep], case.ref["F"])
    packed = case.packed[keep]
    G0, _ = H.decode_centered(packed, case.nsamples, case.ref["F"])
    assert hashlib.sha256(np.asfortranarray(G0).tobytes(order="F")).digest() == bytes(case.ref["G0_sha256"])
    o = case.opts
    if o.perm:
        assert np.array_equal(H.shuffle_columns(keep.size), case.ref["perm"])
    d = H.OracleData(packed, case.nsamples, emu=o.emu, perm=o.perm, seed=o.seed, bands=o.bands, rand=o.rand,
                     svd_t=o.svd, omega0=case.ref["Omg0"])
    op = H.run_pca_with_halko(d, o.k, o.oversamples, maxp=o.maxp, tol=o.tol, maxiter=o.maxiter, tolem=o.tolem)
    if o.emu:
        assert op.em_iters == int(case.ref["meta"][2])
    S = case.ref["S"]
    assert np.max(np.abs(op.S ** 2 - S ** 2) / S ** 2) < 1e-9
    assert np.max(np.abs(align_signs(op.U, case.ref["U"]) - case.ref["U"])) < 1e-8
    assert np.max(np.abs(align_signs(op.V, case.ref["V"]) - case.ref["V"])) < 1e-8


def test_maf_keep_boundaries():
    """MAF(F) = min(F, 1 - F) must exceed the bound strictly (Data.cpp:95)."""
    F = np.array([0.0, 0.1, 0.9, 0.10000000000000002, 0.5, 0.95, 1.0, 0.3])
    assert H.maf_keep(F, 0.1).tolist() == [3, 4, 7]
