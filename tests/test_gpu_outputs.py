"""Outputs of the operator as the reference's callers see them, on the GPU:

* the library's own test matrix (no pcaone_gpu_set_omega): the host draw is the
  reference's Omg0 bit for bit, and a run from it matches the reference
  (initOmg, src/Halko.cpp:15-23);
* the signs of U and V after flip_UV (src/Utils.cpp:118-154, applied by the EM
  path at src/Halko.cpp:295,302,316), compared column by column without
  aligning signs;
* the text outputs (write_eigs_files, src/Data.cpp:211-240) through the
  reference-named mirror pcaone_gb300.halko (FileBed from a PLINK fileset,
  run_pca_with_halko): S^2/M eigenvalues and loadings in file SNP order
  against the reference's own files, to their 6 significant digits.
"""
import os

import numpy as np
import pytest

from oracle import halko as H
from pcaone_gb300 import build as B
from pcaone_gb300 import capi, synthetic
from pcaone_gb300 import halko as PH
from tests.cases import GOLDEN_DIR, golden_case, golden_cases
from tests.test_gpu_parity import ANGLE_TOL, EIG_TOL, c_params, compare

pytestmark = pytest.mark.gpu

EIGS_DIR = os.path.join(GOLDEN_DIR, "eigs")


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not os.path.exists(capi.LIBPATH):
        B.build()
    return capi.load()


def test_library_draw_is_the_reference_draw():
    for case in golden_cases():
        o = case.opts
        assert np.array_equal(capi.random_omega(o.seed, case.nsamples, o.L, gaussian=bool(o.rand)),
                              case.ref["Omg0"]), case.name
    case = golden_case("wsvd_n500_k10")
    with capi.Context() as c:
        c.load_bed(case.packed, case.nsamples)
        U, S, V, _ = c.run_halko(c_params(case.opts, capi.PREC_BF16))   # no set_omega
    compare(U, S, V, case.ref["U"], case.ref["S"], case.ref["V"], "library draw")


@pytest.mark.parametrize("name", ["em_ssvd", "em_wsvd_noshuffle"])
def test_flip_uv_signs(name):
    case = golden_case(name)
    with capi.Context() as c:
        c.load_bed(case.packed, case.nsamples)
        c.set_omega(case.ref["Omg0"])
        U, S, V, _ = c.run_halko(c_params(case.opts, capi.PREC_BF16))
    n = max(1, H.well_separated(case.ref["S"]))
    for A, R in ((U, case.ref["U"]), (V, case.ref["V"])):
        for col in range(n):
            err = np.max(np.abs(A[:, col] - R[:, col])) / np.max(np.abs(R[:, col]))
            assert err < 1e-5, (name, col, err)


def _read(path):
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines() if ln and not ln.startswith("#")]
    return np.array([[float(x) for x in ln.split("\t")] for ln in lines])


@pytest.mark.parametrize("name", ["wsvd_n301", "em_wsvd_noshuffle"])
def test_mirror_writes_the_reference_files(tmp_path, name):
    case = golden_case(name)
    o = case.opts
    prefix = str(tmp_path / name)
    synthetic.write_plink(prefix, case.packed, case.nsamples)
    data = PH.FileBed(prefix)
    assert np.array_equal(data.F, case.ref["F"])
    p = PH.Param(svd=o.svd, k=o.k, oversamples=o.oversamples, maxp=o.maxp, bands=o.bands, seed=o.seed,
                 rand=o.rand, emu=o.emu, maxiter=o.maxiter, tol=o.tol, tolem=o.tolem, noshuffle=o.noshuffle)
    U, S, V, _ = PH.run_pca_with_halko(data, p, fileout=prefix)
    data.close()
    n = max(1, H.well_separated(case.ref["S"]))
    with open(prefix + ".sigvals") as f, open(os.path.join(EIGS_DIR, name + ".sigvals")) as g:
        assert f.readline() == g.readline()  # "#N,M"
    for ext in ("sigvals", "eigvals"):
        got, ref = _read(prefix + "." + ext)[:n, 0], _read(os.path.join(EIGS_DIR, name + "." + ext))[:n, 0]
        assert np.allclose(got, ref, rtol=1e-5, atol=0), (ext, got, ref)
    for ext in ("eigvecs", "loadings"):
        got, ref = _read(prefix + "." + ext)[:, :n], _read(os.path.join(EIGS_DIR, name + "." + ext))[:, :n]
        assert got.shape == ref.shape
        got = got * np.sign(np.sum(got * ref, axis=0))[None, :]   # no-EM runs carry no sign convention
        assert np.max(np.abs(got - ref)) <= 1e-5 * np.max(np.abs(ref)) + 1e-6, ext


def test_mirror_operator_calls():
    """FancyRsvdOpData.computeUSV through the mirror, from the reference's Omg0."""
    case = golden_case("wsvd_n301")
    o = case.opts
    data = PH.FileBed(packed=case.packed, nsamples=case.nsamples)
    op = PH.FancyRsvdOpData(data, o.k, o.oversamples, omega=case.ref["Omg0"],
                            params=PH.Param(k=o.k, oversamples=o.oversamples, maxp=o.maxp, bands=o.bands))
    op.setFlags(False, True)
    op.computeUSV(o.maxp, o.tol)
    assert op.rows() == case.nsnps and op.cols() == case.nsamples and op.size() == o.L
    compare(op.U, op.S, op.V, case.ref["U"], case.ref["S"], case.ref["V"], "mirror computeUSV",
            angle_tol=ANGLE_TOL, eig_tol=EIG_TOL)
    data.close()
