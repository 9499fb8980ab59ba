"""Exactness of the decode and of the block products, through the C-ABI.

The genotype matrix is built so that every quantity of the first epoch is a
short dyadic rational, which FP64 holds exactly:

* every SNP has exactly 256 observed samples (and 44 missing ones), and its
  A1 count is a multiple of 64, so the allele frequency f = count / 512 is a
  multiple of 1/8 (FilePlink.cpp:37-55) and x = d/2 - f is a multiple of 1/8;
* the test matrix holds integers in [-3, 3];
* no standardisation (setFlags(false, false)), as in the first pass of the
  reference's EM path (src/Halko.cpp:293-294).

Then the oracle's FP64 G = X Omega and H = X^T G are exact, and so is the
tensor-core form: its dosages, slice digits and integer accumulation are
exact, every slice combination is an exact int64, and the centring and
missing-entry terms are exact dyadic numbers.  G must agree bit for bit in
both forms, H bit for bit in the tensor-core form (the FP32 CUDA-core form
rounds H's long sums, so it gets a relative tolerance).  Any error in the
2-bit decode, the missing-entry term or the epilogue shows up as a mismatch.
"""
import os

import numpy as np
import pytest

from oracle import halko as H
from pcaone_gb300 import build as B
from pcaone_gb300 import capi, synthetic

pytestmark = pytest.mark.gpu

# FP32 CUDA-core form: relative error of H (long FP32 sums); G is exact
FP32_H_TOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not os.path.exists(capi.LIBPATH):
        B.build()
    return capi.load()


def dyadic_bed(nsamples=300, nsnps=2000, nobs=256, seed=5):
    """Packed genotypes with nobs observed samples per SNP and an A1 count that
    is a multiple of 64 (f in {1/8, ..., 7/8}); PLINK codes 00 (two A1
    copies), 10 (one), 11 (none), 01 (missing), shuffled over samples."""
    rng = np.random.default_rng(seed)
    codes = np.empty((nsnps, nsamples), dtype=np.uint8)
    for j in range(nsnps):
        cnt = 64 * int(rng.integers(1, 8))
        n10 = 2 * int(rng.integers(0, min(cnt, 2 * nobs - cnt) // 2 + 1))
        n00 = (cnt - n10) // 2
        n11 = nobs - n00 - n10
        row = np.array([0] * n00 + [2] * n10 + [3] * n11 + [1] * (nsamples - nobs), dtype=np.uint8)
        codes[j] = row[rng.permutation(nsamples)]
    return synthetic.pack_codes(codes, pad_garbage=True, seed=seed)


@pytest.mark.parametrize("prec", ["bf16", "fp32"])
@pytest.mark.parametrize("k,os_", [(40, 10), (10, 10)], ids=["L50", "L20"])
def test_first_products_exact(prec, k, os_):
    N, M = 300, 2000
    packed = dyadic_bed(N, M)
    L = k + os_
    omega = np.random.default_rng(11).integers(-3, 4, size=(N, L)).astype(np.float64)
    d = H.OracleData(packed, N, omega0=omega, svd_t=1)
    assert np.all(d.F * 8 == np.round(d.F * 8))
    op = H.NormalRsvdOp(d, k, os_)
    op.set_flags(False, False)
    Gr, Hr = op.compute_g_and_h(0)
    p = capi.default_params(svd=1, k=k, oversamples=os_, precision={"bf16": capi.PREC_BF16,
                                                                    "fp32": capi.PREC_FP32}[prec])
    with capi.Context() as c:
        c.load_bed(packed, N)
        _, F = c.counts()
        assert np.array_equal(F, d.F)
        c.set_omega(omega)
        c.op_init(p)
        c.set_flags(False, False)
        G, Hg = c.compute_g_and_h(0)
    bad = np.argwhere(G != Gr)
    assert bad.size == 0, f"G differs at {bad[:5].tolist()}: {G[tuple(bad[0])]} vs {Gr[tuple(bad[0])]}"
    if prec == "bf16":
        bad = np.argwhere(Hg != Hr)
        assert bad.size == 0, f"H differs at {bad[:5].tolist()}: {Hg[tuple(bad[0])]} vs {Hr[tuple(bad[0])]}"
    else:
        eh = np.linalg.norm(Hg - Hr) / np.linalg.norm(Hr)
        print(f"fp32 form: H rel err {eh:.2e}")
        assert eh <= FP32_H_TOL


def test_window_products_exact_with_shuffle():
    """The window method with the shuffled SNP order: the G rows of the first
    two windows (computed before the first update of Omega) are exact."""
    N, M, k, os_, bands = 300, 4096, 10, 10, 64
    packed = dyadic_bed(N, M, seed=8)
    L = k + os_
    omega = np.random.default_rng(12).integers(-3, 4, size=(N, L)).astype(np.float64)
    d = H.OracleData(packed, N, omega0=omega, perm=True, bands=bands)
    op = H.FancyRsvdOp(d, k, os_)
    op.set_flags(False, False)
    Gr, _ = op.compute_g_and_h(0)
    w = M // bands
    with capi.Context() as c:
        c.load_bed(packed, N)
        c.set_omega(omega)
        c.op_init(capi.default_params(k=k, oversamples=os_, bands=bands, precision=capi.PREC_BF16))
        c.set_flags(False, False)
        G, _ = c.compute_g_and_h(0)
        assert np.array_equal(c.perm(), d.perm_idx)
    # epoch 0 updates Omega first after window 1 (band size 2), so windows 0
    # and 1 use the initial integer matrix
    assert np.array_equal(G[:2 * w], Gr[:2 * w])
