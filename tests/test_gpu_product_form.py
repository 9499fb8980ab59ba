"""The two launch forms of the G-shaped tensor-core products
(pcaone_gpu_set_product_form): resident CTAs that take (row tile, K chunk)
items in turn (form 1), and one CTA per item (form 0); the default (form 2)
picks one of them per operand type.  Every item accumulates the same MMAs in
the same order, so every output must agree bit for bit: the first epoch's G and
H, and U, S, V of whole runs, in the BF16, FP8 and FP64-grade forms, on the
golden fixtures (missing genotypes, EM, both methods) and on device-generated
matrices whose launches hold more items than resident CTAs (each CTA takes
several) and fewer (a CTA takes at most one).
"""
import os

import numpy as np
import pytest

from pcaone_gb300 import build as B
from pcaone_gb300 import capi, synthetic
from tests.cases import golden_case
from tests.test_gpu_parity import c_params

pytestmark = pytest.mark.gpu

FORMS = {"bf16": capi.PREC_BF16, "fp8": capi.PREC_FP8, "fp64": capi.PREC_FP64}
GOLDEN = ["wsvd_n301", "ssvd_n203", "em_wsvd_noshuffle", "em_ssvd"]


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not os.path.exists(capi.LIBPATH):
        B.build()
    return capi.load()


def _run(load, omega, params, form):
    with capi.Context() as c:
        c.set_product_form(form)
        load(c)
        c.set_omega(omega)
        c.op_init(params)
        c.set_flags(False, True)
        G, Hm = c.compute_g_and_h(0)
    with capi.Context() as c:
        c.set_product_form(form)
        load(c)
        c.set_omega(omega)
        U, S, V, it = c.run_halko(params)
    return G, Hm, U, S, V, it


def _same(a, b, label):
    for name, x, y in zip(("G", "H", "U", "S", "V", "iterations"), a, b):
        x, y = np.asarray(x), np.asarray(y)
        assert x.shape == y.shape, f"{label}: {name} shape"
        bad = np.argwhere(x != y)
        assert bad.size == 0, f"{label}: {name} differs at {bad[:3].tolist()}"


@pytest.mark.parametrize("prec", list(FORMS))
@pytest.mark.parametrize("name", GOLDEN)
def test_forms_agree_on_golden_cases(name, prec):
    case = golden_case(name)
    p = c_params(case.opts, FORMS[prec])
    load = lambda c: c.load_bed(case.packed, case.nsamples)  # noqa: E731
    out = [_run(load, case.ref["Omg0"], p, form) for form in (0, 1)]
    _same(out[0], out[1], f"{name}[{prec}]")


@pytest.mark.parametrize("prec", list(FORMS))
@pytest.mark.parametrize("shape", [(5003, 60000, 4, 40, 10), (1537, 3000, 4, 10, 10)], ids=["many_items", "few_items"])
def test_forms_agree_on_generated_matrices(shape, prec):
    """N not a multiple of 128, 0.5% missing genotypes; many_items: windows of
    15,000 SNPs (118 row tiles per G launch, 40 sample tiles per H launch,
    several K chunks or splits each)."""
    N, M, bands, k, os_ = shape
    model = synthetic.draw_population_model(N, M, 4, [0.02, 0.05, 0.1, 0.2], seed=17, mcar=0.005)
    omega = np.random.default_rng(9).standard_normal((N, k + os_))
    p = capi.default_params(k=k, oversamples=os_, maxp=4, bands=bands, precision=FORMS[prec])
    load = lambda c: c.load_synthetic(model)  # noqa: E731
    out = [_run(load, omega, p, form) for form in (0, 1)]
    _same(out[0], out[1], f"{shape}[{prec}]")


def test_product_form_argument_checked():
    with capi.Context() as c:
        with pytest.raises(capi.PcaoneError) as e:
            c.set_product_form(3)
        assert e.value.code == -1
