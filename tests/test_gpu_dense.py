"""Dense (FileBinary) input on the GPU: the tensor-core products over FP16
values against the reference's own FileBin outputs (tests/golden/bin_*), the
file-image loader, and the errors of the dense path.

The dense values are FP16 numbers (the storage of imputed dosages), which the
reference reads as float32 exactly.  Unlike 2-bit genotypes they are not
integers, so the tensor core's FP32 accumulation rounds like any FP32 GEMM.
The 1e-8 eigenvalue bar of the genotype path does not apply; on the
well-separated PCs the tolerance is 1e-6 for both the principal angle and the
relative eigenvalue error.
"""
import numpy as np
import pytest

from oracle import halko as H
from pcaone_gb300 import capi, synthetic
from tests.cases import binary_cases
from tests.test_gpu_parity import compare

pytestmark = pytest.mark.gpu

DENSE_ANGLE_TOL = 1e-6
DENSE_EIG_TOL = 1e-6

CASES = binary_cases()
IDS = [c.name for c in CASES]


def d_params(opts):
    return capi.default_params(svd=opts.svd, k=opts.k, oversamples=opts.oversamples, maxp=opts.maxp,
                               bands=opts.bands, seed=opts.seed, rand=opts.rand, perm=int(opts.perm),
                               standardize=0, precision=capi.PREC_BF16)


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_dense_rsvd_vs_reference_outputs(case):
    o = case.opts
    with capi.Context() as c:
        c.load_dense(case.dense.astype(np.float32))
        c.set_omega(case.ref["Omg0"])
        U, S, V, _ = c.run_halko(d_params(o))
        if o.perm:
            assert np.array_equal(c.perm(), case.ref["perm"])
    compare(U, S, V, case.ref["U"], case.ref["S"], case.ref["V"], f"{case.name}[dense]", angle_tol=DENSE_ANGLE_TOL,
            eig_tol=DENSE_EIG_TOL)


def test_dense_vs_oracle_at_larger_size():
    """A 3,000 x 20,000 dosage matrix (5 populations, k=10, p=10): the GPU
    against the FP64 oracle with the same test matrix."""
    model = synthetic.draw_population_model(seed=31, nsamples=3000, nsnps=20000, npop=5,
                                            fst=[0.01, 0.02, 0.05, 0.1, 0.2])
    dense = synthetic.sample_dosages(model)
    d = H.OracleData.from_dense(dense, perm=True, bands=16)
    op = H.run_pca_with_halko(d, 10, 10, maxp=6, maxiter=0)
    with capi.Context() as c:
        c.load_dense(dense.astype(np.float32))
        U, S, V, _ = c.run_halko(capi.default_params(svd=2, k=10, oversamples=10, maxp=6, bands=16, perm=1,
                                                     standardize=0, precision=capi.PREC_BF16))
    compare(U, S, V, op.U, op.S, op.V, "dense 3000x20000", angle_tol=DENSE_ANGLE_TOL, eig_tol=DENSE_EIG_TOL)


def test_binary_file_image_matches_dense_load(tmp_path):
    case = CASES[0]
    path = str(tmp_path / "x.bin")
    synthetic.write_binary(path, case.dense)
    img = open(path, "rb").read()
    p = d_params(case.opts)
    with capi.Context() as c:
        c.load_binary_file_image(img)
        assert (c.nsnps, c.nsamples) == case.dense.shape
        c.set_omega(case.ref["Omg0"])
        U1, S1, _, _ = c.run_halko(p)
        c.load_dense(case.dense.astype(np.float32))
        c.set_omega(case.ref["Omg0"])
        U2, S2, _, _ = c.run_halko(p)
    assert np.array_equal(S1, S2) and np.array_equal(U1, U2)


def test_dense_errors():
    lib = capi.load()
    dense = synthetic.sample_dosages(synthetic.draw_population_model(seed=3, nsamples=64, nsnps=200, npop=2,
                                                                     fst=0.1))
    with capi.Context() as c:
        # truncated image
        img = np.frombuffer(np.array([200, 64], dtype=np.uint32).tobytes() + b"\0" * 16, dtype=np.uint8)
        assert lib.pcaone_gpu_load_binary_file_image(c.h, img.ctypes.data, img.size) == -4  # PCAONE_E_FORMAT
        c.load_dense(dense.astype(np.float32))
        # the FP32 CUDA-core form, EM and the genotype-only calls are not available
        with pytest.raises(capi.PcaoneError):
            c.run_halko(capi.default_params(k=2, oversamples=2, bands=4, standardize=0, precision=capi.PREC_FP32))
        with pytest.raises(capi.PcaoneError):
            c.run_halko(capi.default_params(k=2, oversamples=2, bands=4, standardize=0, emu=1,
                                            precision=capi.PREC_BF16))
        with pytest.raises(capi.PcaoneError):
            c.counts()
