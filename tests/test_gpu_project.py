"""Projection of new samples on the GPU (pcaone_gpu_project) against the
reference's run_projection outputs (tests/golden/proj_*: --project 1 and the
per-sample least squares of --project 2 over observed SNPs)."""
import numpy as np
import pytest

from oracle import halko as H
from pcaone_gb300 import capi, synthetic
from tests.cases import golden_cases

pytestmark = pytest.mark.gpu

CASES = [c for c in golden_cases() if "P2" in c.ref]
IDS = [c.name for c in CASES]


def _fit(case):
    k = case.opts.k
    V = case.ref["V"][:, :k]
    if case.opts.perm:  # loadings in file order, as .loadings holds them
        Vf = np.empty_like(V)
        Vf[case.ref["perm"]] = V
        V = Vf
    return case.ref["F"], V, case.ref["S"][:k]


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_projection_vs_reference(case, mode):
    F, V, S = _fit(case)
    with capi.Context() as c:
        c.load_bed(case.ref["packed_new"], int(case.ref["n_new"]))
        U = c.project(F, V, S, mode)
    ref = case.ref["P1" if mode == 1 else "P2"]
    err = np.max(np.abs(U - ref)) / np.max(np.abs(ref))
    print(f"{case.name} mode {mode}: max rel err {err:.2e}")
    assert err <= 1e-8


def test_projection_fitted_samples_recover_scores():
    """Mode 1 applied to the fitted samples themselves returns U of the fit
    (X V S^-1 = U for the converged factors, up to the power-iteration error)."""
    case = [c for c in golden_cases() if c.name == "ssvd_n203"][0]
    o = case.opts
    with capi.Context() as c:
        c.load_bed(case.packed, case.nsamples)
        c.set_omega(case.ref["Omg0"])
        p = capi.default_params(svd=o.svd, k=o.k, oversamples=o.oversamples, maxp=30, bands=o.bands, seed=o.seed,
                                rand=o.rand, perm=0, standardize=1, precision=capi.PREC_FP32)
        U, S, V, _ = c.run_halko(p)
        _, F = c.counts()
        P = c.project(F, V, S, 1)
    n = max(1, H.well_separated(S))
    assert H.sin_largest_angle(P[:, :n], U[:, :n]) < 1e-6


def test_projection_errors():
    case = CASES[0]
    F, V, S = _fit(case)
    with capi.Context() as c:
        c.load_bed(case.ref["packed_new"], int(case.ref["n_new"]))
        with pytest.raises(capi.PcaoneError):
            c.project(F, V, S, 3)
        big = np.zeros((V.shape[0], 33))
        with pytest.raises(capi.PcaoneError):
            c.project(F, big, np.ones(33), 1)
        with pytest.raises(capi.PcaoneError):
            c.project(F, V, -S, 1)
        dense = synthetic.sample_dosages(synthetic.draw_population_model(seed=3, nsamples=64, nsnps=200, npop=2,
                                                                         fst=0.1))
        c.load_dense(dense.astype(np.float32))
        with pytest.raises(capi.PcaoneError):
            c.project(np.full(200, 0.3), np.zeros((200, 2)), np.ones(2), 1)
