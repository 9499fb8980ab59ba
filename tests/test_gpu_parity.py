"""Parity of the CUDA path (through the C-ABI) with the oracle and with the
reference's own outputs (tests/golden/).

Tolerances (floating point):
  * decode, counts, allele frequencies: bit-exact (the decode and the products
    themselves are checked bit for bit in test_gpu_exact.py).
  * U, S, V of both forms vs the reference's FP64 outputs or the FP64 oracle,
    same Omega, same schedule (the benchmark spec's bar):
      - largest principal angle (sin) over the well-separated leading PCs
        (relative eigen-gap > 5%): <= 1e-6
      - relative eigenvalue error of those PCs: <= 1e-8
    Near-degenerate noise PCs are not determined by a few power iterations (the
    reference's own FP64 methods disagree on them); they are not compared.
  * first-epoch G and H vs the oracle's FP64 products: relative error <= 1e-7
    for the tensor-core form (the test matrix and G enter as 27-bit integer
    slices; rounding them to 27 bits relative to the column maximum is the
    only error left, since the integer products are exact) and <= 1e-6 for the
    FP32 CUDA-core form.
"""
import os

import numpy as np
import pytest

from oracle import halko as H
from pcaone_gb300 import build as B
from pcaone_gb300 import capi, synthetic
from tests.cases import align_signs, golden_case, golden_cases

pytestmark = pytest.mark.gpu

ANGLE_TOL = 1e-6
EIG_TOL = 1e-8
PROD_TOL = {"bf16": 1e-7, "fp32": 1e-6}
# tensor-core form: three integer BF16 slices per column (27 bits, exact integer
# accumulation in TMEM) in every epoch
PRECISIONS = {"fp32": capi.PREC_FP32, "bf16": capi.PREC_BF16}

CASES = golden_cases()
IDS = [c.name for c in CASES]


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not os.path.exists(capi.LIBPATH):
        B.build()
    return capi.load()


def c_params(opts, precision=capi.PREC_FP32):
    return capi.default_params(svd=opts.svd, k=opts.k, oversamples=opts.oversamples, maxp=opts.maxp,
                               bands=opts.bands, seed=opts.seed, rand=opts.rand, perm=int(opts.perm),
                               emu=int(opts.emu), maxiter=opts.maxiter, tol=opts.tol, tolem=opts.tolem,
                               standardize=1, precision=precision)


def compare(U, S, V, Ur, Sr, Vr, label="", angle_tol=ANGLE_TOL, eig_tol=EIG_TOL):
    n = max(1, H.well_separated(Sr))
    ang_u = H.sin_largest_angle(U[:, :n], Ur[:, :n])
    ang_v = H.sin_largest_angle(V[:, :n], Vr[:, :n])
    eig = float(np.max(H.eig_relerr(S[:n], Sr[:n])))
    print(f"{label} n={n} sin(U)={ang_u:.2e} sin(V)={ang_v:.2e} eig={eig:.2e}")
    assert ang_u <= angle_tol and ang_v <= angle_tol
    assert eig <= eig_tol
    return n, ang_u, ang_v, eig


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_counts_and_F_bit_exact(case):
    with capi.Context() as c:
        c.load_bed(case.packed, case.nsamples)
        cnt, F = c.counts()
    assert np.array_equal(cnt, H.bed_counts(case.packed, case.nsamples).astype(np.int32))
    assert np.array_equal(F, case.ref["F"])


def test_counts_edge_cases():
    code = np.array([[1] * 7, [0] * 7, [3] * 7, [2, 1, 0, 3, 1, 2, 0], [1, 1, 1, 1, 1, 1, 0]], dtype=np.uint8)
    packed = synthetic.pack_codes(code, pad_garbage=True, seed=9)
    with capi.Context() as c:
        c.load_bed(packed, 7)
        cnt, F = c.counts()
    assert np.array_equal(cnt, H.bed_counts(packed, 7).astype(np.int32))
    assert np.array_equal(F, H.allele_freq(H.bed_counts(packed, 7)))
    assert F[0] == 0.0 and F[1] == 1.0


@pytest.mark.parametrize("prec", list(PRECISIONS), ids=list(PRECISIONS))
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_rsvd_vs_reference_outputs(case, prec):
    """Same Omega as the reference (golden Omg0): U, S, V agree with the
    reference's FP64 results on the well-separated PCs."""
    o = case.opts
    with capi.Context() as c:
        c.load_bed(case.packed, case.nsamples)
        c.set_omega(case.ref["Omg0"])
        U, S, V, it = c.run_halko(c_params(o, PRECISIONS[prec]))
        if o.perm:
            assert np.array_equal(c.perm(), case.ref["perm"])
    if o.emu:
        assert abs(it - int(case.ref["meta"][2])) <= 1
    compare(U, S, V, case.ref["U"], case.ref["S"], case.ref["V"], f"{case.name}[{prec}]")


@pytest.mark.parametrize("prec", list(PRECISIONS), ids=list(PRECISIONS))
def test_first_epoch_products_vs_oracle(prec):
    """computeGandH(pi=0) of the window method vs the oracle's FP64 G and H."""
    case = golden_case("wsvd_n301")
    o = case.opts
    d = H.OracleData(case.packed, case.nsamples, perm=True, bands=o.bands, omega0=case.ref["Omg0"])
    op = H.FancyRsvdOp(d, o.k, o.oversamples)
    op.set_flags(False, True)
    Gr, Hr = op.compute_g_and_h(0)
    with capi.Context() as c:
        c.load_bed(case.packed, case.nsamples)
        c.set_omega(case.ref["Omg0"])
        c.op_init(c_params(o, PRECISIONS[prec]))
        c.set_flags(False, True)
        G, Hg = c.compute_g_and_h(0)
    eg = np.linalg.norm(G - Gr) / np.linalg.norm(Gr)
    eh = np.linalg.norm(Hg - Hr) / np.linalg.norm(Hr)
    print(f"epoch-0 products [{prec}]: rel err G {eg:.2e} H {eh:.2e}")
    assert eg <= PROD_TOL[prec] and eh <= PROD_TOL[prec]


@pytest.mark.parametrize("prec", list(PRECISIONS))
def test_wide_sketch_with_missing(prec):
    """k + p = 40 (padded to 48, three slices -> 144 accumulator columns per
    part) with missing genotypes: the tensor-core shapes of the 100k x 500k
    workload at a small size."""
    model = synthetic.draw_population_model(1500, 6000, 5, [0.01, 0.02, 0.05, 0.1, 0.2], seed=21, mcar=0.005)
    packed = synthetic.sample_packed_bed(model)
    k, os_ = 20, 20
    omega = H.random_omega(112, model.nsamples, k + os_)
    d = H.OracleData(packed, model.nsamples, perm=True, bands=64, omega0=omega)
    ref = H.run_pca_with_halko(d, k, os_, maxp=6)
    p = capi.default_params(k=k, oversamples=os_, maxp=6, bands=64, precision=PRECISIONS[prec])
    with capi.Context() as c:
        c.load_bed(packed, model.nsamples)
        c.set_omega(omega)
        U, S, V, _ = c.run_halko(p)
    compare(U, S, V, ref.U, ref.S, ref.V, f"wide[{prec}]")


@pytest.mark.parametrize("prec", list(PRECISIONS))
def test_precision_form_shape(prec):
    """The shapes of the 200,000 x 1,000,000 precision-form workload at a small
    size: k=40, p=10 (L=50, padded to 64: the three slices take 192 TMEM
    columns), 64 windows, N not a multiple of 128, eight Balding-Nichols
    populations plus 2% admixed samples (Dirichlet ancestry), allele
    frequencies from Beta(0.5, 0.5) truncated to [0.01, 0.99], and 0.5%
    missing genotypes."""
    model = synthetic.model_for("c3", seed=3, nsamples=3001, nsnps=19200, mcar=0.005)
    packed = synthetic.sample_packed_bed(model)
    k, os_ = 40, 10
    omega = H.random_omega(112, model.nsamples, k + os_)
    d = H.OracleData(packed, model.nsamples, perm=True, bands=64, omega0=omega)
    ref = H.run_pca_with_halko(d, k, os_, maxp=6)
    p = capi.default_params(k=k, oversamples=os_, maxp=6, bands=64, precision=PRECISIONS[prec])
    with capi.Context() as c:
        c.load_bed(packed, model.nsamples)
        c.set_omega(omega)
        U, S, V, _ = c.run_halko(p)
    n, *_ = compare(U, S, V, ref.U, ref.S, ref.V, f"c3-shape[{prec}]")
    assert n >= 7  # the seven population PCs are compared


def test_matvec_vs_oracle():
    case = golden_case("wsvd_n500_k10")
    d = H.OracleData(case.packed, case.nsamples)
    d.standardize_E()
    x = np.random.default_rng(3).standard_normal(case.nsamples)
    yr = H.arnoldi_matvec(d, x)
    with capi.Context() as c:
        c.load_bed(case.packed, case.nsamples)
        y = c.matvec(x, standardize=True)
    assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < 1e-12


@pytest.mark.parametrize("prec", list(PRECISIONS), ids=list(PRECISIONS))
def test_config1_vs_oracle(prec):
    """The 2,000 x 20,000 three-population workload, k=10, 7 epochs."""
    wl = synthetic.WORKLOADS["c1"]
    model = synthetic.model_for("c1", seed=1)
    packed = synthetic.sample_packed_bed(model)
    omega = H.random_omega(112, model.nsamples, wl["k"] + wl["p"])
    d = H.OracleData(packed, model.nsamples, perm=True, bands=wl["bands"], omega0=omega)
    ref = H.run_pca_with_halko(d, wl["k"], wl["p"], maxp=wl["maxp"])
    p = capi.default_params(k=wl["k"], oversamples=wl["p"], maxp=wl["maxp"], bands=wl["bands"],
                            precision=PRECISIONS[prec])
    with capi.Context() as c:
        c.load_bed(packed, model.nsamples)
        c.set_omega(omega)
        U, S, V, _ = c.run_halko(p)
    compare(U, S, V, ref.U, ref.S, ref.V, f"c1[{prec}]")


def test_device_generator_matches_numpy():
    model = synthetic.draw_population_model(333, 1000, 4, [0.05, 0.1, 0.2, 0.3], seed=4, admixed_frac=0.1,
                                            miss_sample_beta=(1, 20), miss_snp_beta=(1, 50))
    ref = synthetic.sample_packed_bed(model)
    with capi.Context() as c:
        c.load_synthetic(model)
        got = c.get_bed()
        cnt, _ = c.counts()
    assert np.array_equal(got, ref)
    assert np.array_equal(cnt, H.bed_counts(ref, 333).astype(np.int32))


def test_errors_are_reported_not_faulted():
    with capi.Context() as c:
        with pytest.raises(capi.PcaoneError) as e:
            c.load_bed_file_image(b"\x00\x00\x00" + b"\x00" * 10, 2, 20)
        assert e.value.code == -4
        with pytest.raises(capi.PcaoneError) as e:
            c.load_bed_file_image(bytes([0x6C, 0x1B, 0x01]) + b"\x00" * 5, 2, 20)
        assert e.value.code == -4
        packed = synthetic.pack_codes(np.zeros((10, 8), dtype=np.uint8))
        c.load_bed(packed, 8)
        with pytest.raises(capi.PcaoneError) as e:
            c.op_init(capi.default_params(k=5, oversamples=5))    # L > N
        assert e.value.code == -1
        with pytest.raises(capi.PcaoneError) as e:
            c.op_init(capi.default_params(k=2, oversamples=2, bands=6))
        assert e.value.code == -1
        with pytest.raises(capi.PcaoneError):
            c.compute_usv(3, 1e-4)                                  # no operator yet
