"""Host-side checks of the C-ABI library that need no GPU."""
import os
import re

import pytest

from pcaone_gb300 import build as B
from pcaone_gb300 import capi

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "pcaone_gpu.h")


def _declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pcaone_gpu_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(capi.LIBPATH):
        B.build()
    return capi.load()


def test_header_and_binding_agree():
    assert _declared_functions() == sorted(capi.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in _declared_functions():
        assert hasattr(lib, name), name


def test_abi_version_and_defaults(lib):
    assert lib.pcaone_gpu_abi_version() == 1
    p = capi.default_params()
    # reference defaults, src/Cmd.hpp:29-95
    assert (p.svd, p.k, p.oversamples, p.maxp, p.bands, p.seed, p.rand) == (2, 10, 10, 20, 64, 112, 1)
    assert (p.maxiter, p.tol, p.tolem, p.ploidy, p.standardize) == (100, 1e-4, 1e-5, 2, 1)


def test_null_context_is_an_argument_error(lib):
    assert lib.pcaone_gpu_load_bed(None, None, 0, 0) == -1
    assert lib.pcaone_gpu_close(None) == 0
