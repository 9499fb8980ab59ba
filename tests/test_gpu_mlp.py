"""GPU tests of the learned EM warm start: the network's forward and backward
kernels against the float64 oracle, and the warm start itself against plain
mean-fill EM on a cohort with c4-like missingness."""
import numpy as np
import pytest

from oracle import mlp as M
from oracle.halko import sin_largest_angle
from pcaone_gb300 import capi, synthetic

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("B", [1, 37, 512, 4096])
def test_forward_backward_matches_oracle(B):
    rng = np.random.default_rng(B)
    X = rng.normal(size=(B, M.N_IN)).astype(np.float32)
    X[:, 63:] = 0.0  # padding column of the feature vector
    y = rng.normal(scale=0.3, size=B).astype(np.float32)
    theta = M.he_init(B + 1)
    out, loss, g = capi.mlp_forward_backward(X, y, theta)
    out_r, loss_r, g_r = M.forward_backward(X, y, theta)
    # FP32 accumulation over at most 4096 terms against float64
    assert np.max(np.abs(out - out_r)) <= 1e-5 * max(1.0, np.max(np.abs(out_r)))
    assert abs(loss - loss_r) <= 1e-5 * max(1.0, loss_r)
    for a, b in [(M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2), (M.OFF_B2, M.OFF_W3),
                 (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.N_PARAMS)]:
        scale = max(np.max(np.abs(g_r[a:b])), 1e-12)
        assert np.max(np.abs(g[a:b] - g_r[a:b])) <= 1e-4 * scale, (a, b)


def test_forward_backward_rejects_bad_arguments():
    lib = capi.load()
    assert lib.pcaone_gpu_mlp_forward_backward(0, None, None, 4, None, None, None, None) == -1  # PCAONE_E_ARG


def _cohort():
    # c4-like missingness (per-sample Beta(1,20), per-SNP Beta(1,50)) on four populations
    return synthetic.draw_population_model(seed=7, nsamples=2000, nsnps=12000, npop=4, fst=0.05,
                                           anc="uniform", anc_range=(0.05, 0.5), miss_sample_beta=(1, 20),
                                           miss_snp_beta=(1, 50))


@pytest.mark.parametrize("precision", [capi.PREC_BF16, capi.PREC_FP32])
def test_warm_start_against_plain_em(precision):
    """The learned start imputes held-out observed genotypes better than the
    mean fill it replaces, and EM from it converges to plain EM's PCs.  (On
    cohorts without linkage EM from the mean fill already converges in a few
    iterations; the iteration counts are printed, and the learned start may
    not cost more than one extra iteration.)"""
    model = _cohort()
    p = capi.default_params(svd=capi.SVD_WINDOW, perm=0, k=3, oversamples=3, maxp=6, bands=16, emu=1,
                            maxiter=100, tolem=1e-6, precision=precision)
    with capi.Context(0) as c:
        c.load_synthetic(model)
        U0, S0, V0, it0 = c.run_halko(p)
        w = capi.mlp_default_params(train_entries=131072, holdout_entries=32768, epochs=4, batch=2048)
        c.set_warm_start(w)
        U1, S1, V1, it1 = c.run_halko(p)
        st = c.mlp_stats()
        c.set_warm_start(None)
        U2, S2, V2, it2 = c.run_halko(p)
    print(f"EM iterations plain {it0}, warm start {it1}; stats {st}")
    # held-out observed genotypes: the network's error is below the mean fill's
    assert st["holdout_mse"] < 0.97 * st["holdout_mse_mean_fill"]
    assert st["filled"] > 0 and st["train_mse"] > 0
    assert it1 <= it0 + 1
    # same converged PCs as plain EM (within EM's stopping tolerance)
    assert np.max(np.abs(S1 - S0) / S0) < 1e-4
    assert sin_largest_angle(U0[:, :2], U1[:, :2]) < 5e-3
    # switching the learned start off restores plain EM exactly
    assert it2 == it0 and np.array_equal(S2, S0)
