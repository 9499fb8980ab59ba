"""The FP8 form (PCAONE_PREC_FP8): E4M3 tensor-core products (tcgen05
kind::f8f6f4) in the range-finding epochs, the exact 27-bit form in the final
ones.

* The E4M3 operands are exact: dosages 0/1/2, and the test matrix and G as two
  balanced base-16 digits |w| <= 8 (an 8-bit integer per entry, relative to the
  column maximum), with exact integer accumulation.  On the dyadic matrix of
  test_gpu_exact.py with integers in [-3, 3] as test matrix, the 8-bit
  representation is exact too, so G must equal the oracle's FP64 G bit for
  bit; H (from the 8-bit rounding of G) within the rounding's few percent.
* The E4M3 epochs follow another trajectory than the reference's FP64 epochs,
  so the FP8 form is held to the converged answer instead (the "converged
  oracle" measure): the top PCs of a dense FP64 SVD of the standardised
  matrix.  On the PCs separated from the next by a relative eigen-gap above
  5% it must meet the benchmark spec's bars: sin of the largest principal angle
  <= 1e-6 and relative eigenvalue error <= 1e-8.  (At the 200,000 x 1,000,000
  scale the bench also compares it with the FP64-grade form on the same
  schedule.)
"""
import os

import numpy as np
import pytest

from oracle import halko as H
from pcaone_gb300 import build as B
from pcaone_gb300 import capi, synthetic
from tests.cases import golden_cases
from tests.test_gpu_exact import dyadic_bed
from tests.test_gpu_parity import ANGLE_TOL, EIG_TOL, c_params, compare

pytestmark = pytest.mark.gpu

CASES = golden_cases()


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not os.path.exists(capi.LIBPATH):
        B.build()
    return capi.load()


@pytest.mark.parametrize("k,os_", [(40, 10), (10, 10)], ids=["L50", "L20"])
def test_fp8_first_products(k, os_):
    N, M = 300, 2000
    packed = dyadic_bed(N, M)
    L = k + os_
    omega = np.random.default_rng(11).integers(-3, 4, size=(N, L)).astype(np.float64)
    d = H.OracleData(packed, N, omega0=omega, svd_t=1)
    op = H.NormalRsvdOp(d, k, os_)
    op.set_flags(False, False)
    Gr, Hr = op.compute_g_and_h(0)
    with capi.Context() as c:
        c.load_bed(packed, N)
        c.set_omega(omega)
        c.op_init(capi.default_params(svd=1, k=k, oversamples=os_, precision=capi.PREC_FP8))
        c.set_flags(False, False)
        G, Hg = c.compute_g_and_h(0)
    bad = np.argwhere(G != Gr)
    assert bad.size == 0, f"G differs at {bad[:5].tolist()}: {G[tuple(bad[0])]} vs {Gr[tuple(bad[0])]}"
    eh = np.linalg.norm(Hg - Hr) / np.linalg.norm(Hr)
    print(f"fp8 epoch-0 H rel err {eh:.2e} (8-bit rounding of G)")
    assert 1e-6 < eh < 5e-2


def _dense_truth(packed, nsamples, k):
    """Top-k PCs of the standardised, mean-imputed matrix by a dense FP64 SVD
    (the converged answer), V in file SNP order."""
    d = H.OracleData(packed, nsamples)
    d.standardize_E()
    U, s, Vt = np.linalg.svd(d.G, full_matrices=False)
    return U[:, :k], s[:k], Vt[:k].T


def _fp8_vs_truth(packed, nsamples, k, os_, label, **kw):
    Ut, St, Vt = _dense_truth(packed, nsamples, k)
    p = capi.default_params(k=k, oversamples=os_, precision=capi.PREC_FP8, **kw)
    with capi.Context() as c:
        c.load_bed(packed, nsamples)
        U, S, V, _ = c.run_halko(p)
        perm = c.perm()
    Vf = np.empty_like(V)
    Vf[perm] = V
    return compare(U, S, Vf, Ut, St, Vt, label, angle_tol=ANGLE_TOL, eig_tol=EIG_TOL)


def test_fp8_converged_three_populations():
    """2,000 x 20,000, three populations (Fst 0.05), k=10, p=10, 64 windows."""
    model = synthetic.model_for("c1", seed=1)
    n, *_ = _fp8_vs_truth(synthetic.sample_packed_bed(model), model.nsamples, 10, 10, "c1[fp8 vs dense]",
                          maxp=6, bands=64)
    assert n >= 2


def test_fp8_converged_precision_form_shape():
    """k=40, p=10, eight populations plus admixed samples, 0.5% missing."""
    model = synthetic.model_for("c3", seed=3, nsamples=3001, nsnps=19200, mcar=0.005)
    n, *_ = _fp8_vs_truth(synthetic.sample_packed_bed(model), model.nsamples, 40, 10, "c3-shape[fp8 vs dense]",
                          maxp=6, bands=64)
    assert n >= 7


def test_fp8_converged_single_pass():
    case = next(c for c in CASES if c.name == "ssvd_n203")
    o = case.opts
    _fp8_vs_truth(case.packed, case.nsamples, o.k, o.oversamples, "ssvd_n203[fp8 vs dense]", svd=1,
                  maxp=o.maxp)


def test_fp8_rejects_dense_input():
    with capi.Context() as c:
        c.load_dense(np.ones((50, 300), dtype=np.float32))
        with pytest.raises(capi.PcaoneError) as e:
            c.op_init(capi.default_params(k=4, oversamples=4, standardize=0, precision=capi.PREC_FP8))
        assert e.value.code == -1
