"""Failure handling of the tensor-core pipeline, without faulting the GPU.

Every mbarrier wait in the product kernels is bounded.  Here the bound is set
to one cycle through the test hook pcaone_gpu_set_wait_limit, so the first wait
that is not satisfied at once gives up: its tile sets the shared abort flag,
every other role leaves its loop, the tile waits (with the normal bound) for
its own TMA copies and MMAs in flight, frees its tensor memory and raises the
error flag.  The call must return PCAONE_E_CUDA with the message, and the same
context must then give the correct result once the bound is restored.  No
kernel traps or spins without a bound on this path.
"""
import os

import pytest

from pcaone_gb300 import build as B
from pcaone_gb300 import capi
from tests.cases import golden_case
from tests.test_gpu_parity import c_params, compare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not os.path.exists(capi.LIBPATH):
        B.build()
    return capi.load()


def test_bounded_wait_gives_up_and_context_recovers():
    case = golden_case("wsvd_n500_k10")
    p = c_params(case.opts, capi.PREC_BF16)
    with capi.Context() as c:
        c.load_bed(case.packed, case.nsamples)
        c.set_omega(case.ref["Omg0"])
        c.set_wait_limit(1)
        with pytest.raises(capi.PcaoneError) as e:
            c.run_halko(p)
        assert e.value.code == -2, e.value        # PCAONE_E_CUDA
        assert "bounded wait" in str(e.value)
        c.set_wait_limit(0)
        U, S, V, _ = c.run_halko(p)
    compare(U, S, V, case.ref["U"], case.ref["S"], case.ref["V"], "after abort")


def test_wait_limit_argument_checked():
    with capi.Context() as c:
        with pytest.raises(capi.PcaoneError) as e:
            c.set_wait_limit(-1)
        assert e.value.code == -1
