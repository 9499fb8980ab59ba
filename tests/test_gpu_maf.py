"""--maf on the GPU (pcaone_gpu_filter_maf, Data::filter_snps_resize_F of
src/Data.cpp:88-105): the kept rows, their allele frequencies and the PCs of
the filtered matrix against the reference's own --maf runs; the filter equals
loading the kept rows directly, bit for bit; repeated filters compose; the
reference's argument rules hold."""
import os

import numpy as np
import pytest

from oracle import halko as H
from pcaone_gb300 import build as B
from pcaone_gb300 import capi
from pcaone_gb300 import halko as HK
from tests.cases import golden_cases
from tests.test_gpu_parity import c_params, compare

pytestmark = pytest.mark.gpu

CASES = golden_cases(maf=True)
IDS = [c.name for c in CASES]
FORMS = {"bf16": (capi.PREC_BF16, 1e-6, 1e-8), "fp64": (capi.PREC_FP64, 2e-8, 2e-9)}


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not os.path.exists(capi.LIBPATH):
        B.build()
    return capi.load()


def _run(c, case, prec):
    c.set_omega(case.ref["Omg0"])
    return c.run_halko(c_params(case.opts, prec))


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_maf_vs_reference(case, form):
    prec, angle_tol, eig_tol = FORMS[form]
    with capi.Context() as c:
        c.load_bed(case.packed, case.nsamples)
        assert c.filter_maf(case.opts.maf) == case.ref["keep"].size
        assert np.array_equal(c.kept_snps(), case.ref["keep"])
        _, F = c.counts()
        assert np.array_equal(F, case.ref["F"])  # the reference's F of the kept SNPs, bit for bit
        U, S, V, it = _run(c, case, prec)
        if case.opts.perm:
            assert np.array_equal(c.perm(), case.ref["perm"])
    if case.opts.emu:
        assert abs(it - int(case.ref["meta"][2])) <= 1
    compare(U, S, V, case.ref["U"], case.ref["S"], case.ref["V"], f"{case.name}[{form}]", angle_tol=angle_tol,
            eig_tol=eig_tol)


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_maf_equals_loading_the_kept_rows(case):
    keep = case.ref["keep"]
    with capi.Context() as c:
        c.load_bed(case.packed, case.nsamples)
        c.filter_maf(case.opts.maf)
        bed_f = c.get_bed()
        cnt_f, F_f = c.counts()
        out_f = _run(c, case, capi.PREC_BF16)
    with capi.Context() as c:
        c.load_bed(np.ascontiguousarray(case.packed[keep]), case.nsamples)
        bed_k = c.get_bed()
        cnt_k, F_k = c.counts()
        out_k = _run(c, case, capi.PREC_BF16)
    bps = (case.nsamples + 3) // 4
    assert np.array_equal(bed_f[:, :bps], bed_k[:, :bps])
    assert np.array_equal(cnt_f, cnt_k) and np.array_equal(F_f, F_k)
    for a, b in zip(out_f, out_k):
        assert np.array_equal(np.asarray(a), np.asarray(b))


def test_maf_filters_compose_and_arguments_are_checked():
    case = CASES[0]
    F_all = H.allele_freq(H.bed_counts(case.packed, case.nsamples))
    with capi.Context() as c:
        c.load_bed(case.packed, case.nsamples)
        assert np.array_equal(c.kept_snps(), np.arange(case.nsnps))  # no filter: identity
        for bad in (0.0, -0.1, 0.5, 0.7, float("nan")):
            with pytest.raises(capi.PcaoneError) as e:
                c.filter_maf(bad)
            assert e.value.code == -1
        c.filter_maf(0.05)
        assert np.array_equal(c.kept_snps(), H.maf_keep(F_all, 0.05))
        c.filter_maf(case.opts.maf)  # a second filter on the filtered rows
        assert np.array_equal(c.kept_snps(), case.ref["keep"])
    # every SNP monomorphic: nothing is left
    with capi.Context() as c:
        c.load_bed(np.zeros((8, 4), dtype=np.uint8), 16)
        with pytest.raises(capi.PcaoneError) as e:
            c.filter_maf(0.01)
        assert e.value.code == -1
    # out of core (the reference has no filter there) and dense input
    with capi.Context() as c:
        c.load_bed_stream(case.packed, case.nsamples)
        with pytest.raises(capi.PcaoneError) as e:
            c.filter_maf(0.1)
        assert e.value.code == -1
    with capi.Context() as c:
        c.load_dense(np.ones((4, 8), dtype=np.float32))
        with pytest.raises(capi.PcaoneError) as e:
            c.filter_maf(0.1)
        assert e.value.code == -1


def test_mirror_file_bed_maf():
    case = CASES[0]
    o = case.opts
    fb = HK.FileBed(packed=case.packed, nsamples=case.nsamples, maf=o.maf)
    assert fb.nsnps == case.ref["keep"].size and np.array_equal(fb.keepSNPs, case.ref["keep"])
    assert np.array_equal(fb.F, case.ref["F"])
    p = HK.Param(svd=o.svd, k=o.k, oversamples=o.oversamples, maxp=o.maxp, bands=o.bands, seed=o.seed, rand=o.rand,
                 noshuffle=o.noshuffle, emu=o.emu, maxiter=o.maxiter, precision=capi.PREC_BF16).finalize()
    fb.ctx.set_omega(case.ref["Omg0"])
    U, S, V, _ = HK.run_pca_with_halko(fb, p)
    fb.close()
    compare(U, S, V, case.ref["U"], case.ref["S"], case.ref["V"], "mirror --maf")
