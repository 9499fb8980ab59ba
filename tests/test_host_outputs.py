"""Host-side parts of the path, checked without a GPU against the reference's
own outputs (tests/golden/, written by the reference built from its sources):

* the initial random test matrix (initOmg, src/Halko.cpp:15-23) and the
  in-core SNP shuffle (src/RSVD.hpp:61-70) drawn by the library's host code:
  bit-exact;
* the text outputs of Data::write_eigs_files (src/Data.cpp:211-240) written by
  pcaone_gb300.halko from the reference's own U, S, V: byte-identical,
  including the S^2/M eigenvalues and the loadings back in file SNP order.
"""
import os

import numpy as np
import pytest

from pcaone_gb300 import build as B
from pcaone_gb300 import capi
from pcaone_gb300 import halko as PH
from tests.cases import GOLDEN_DIR, golden_case, golden_cases

EIGS_DIR = os.path.join(GOLDEN_DIR, "eigs")
EIGS_CASES = ("wsvd_n301", "em_wsvd_noshuffle")


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not os.path.exists(capi.LIBPATH):
        B.build()
    return capi.load()


@pytest.mark.parametrize("case", golden_cases(), ids=[c.name for c in golden_cases()])
def test_random_omega_bit_exact(case):
    o = case.opts
    om = capi.random_omega(o.seed, case.nsamples, o.L, gaussian=bool(o.rand))
    assert om.shape == case.ref["Omg0"].shape
    assert np.array_equal(om, case.ref["Omg0"])


@pytest.mark.parametrize("case", [c for c in golden_cases() if "perm" in c.ref], ids=lambda c: c.name)
def test_shuffle_order_bit_exact(case):
    assert np.array_equal(capi.shuffle_order(case.nsnps), case.ref["perm"])


@pytest.mark.parametrize("name", EIGS_CASES)
def test_eigs_files_byte_identical(tmp_path, name):
    case = golden_case(name)
    r = case.ref
    prefix = str(tmp_path / name)
    PH.write_eigs_files(prefix, r["S"], r["U"], r["V"], case.nsnps, r.get("perm"))
    for ext in ("sigvals", "eigvals", "eigvecs", "loadings"):
        with open(prefix + "." + ext) as f, open(os.path.join(EIGS_DIR, name + "." + ext)) as g:
            assert f.read() == g.read(), ext


def test_host_draw_errors():
    lib = capi.load()
    assert lib.pcaone_gpu_random_omega(1, 1, 0, 3, None) == -1
    assert lib.pcaone_gpu_shuffle_order(0, None) == -1
