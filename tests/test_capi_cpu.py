"""Host-side checks of the C-ABI library that need no GPU."""
import os
import re

import numpy as np
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


C_CALLER = r"""
#include <stdio.h>
#include "pcaone_gpu.h"

int main(void) {
  pcaone_gpu_params p;
  pcaone_gpu_default_params(&p);
  if (pcaone_gpu_abi_version() != 1) return 1;
  if (p.k != 10 || p.oversamples != 10 || p.bands != 64) return 2;
  /* a null context is an argument error, reported without a GPU */
  if (pcaone_gpu_load_bed(NULL, NULL, 0, 0) != PCAONE_E_ARG) return 3;
  if (pcaone_gpu_close(NULL) != 0) return 4;
  puts("c caller ok");
  return 0;
}
"""


def test_header_is_plain_c_and_links_from_c(tmp_path, lib):
    """The header compiles as strict C99 and a C program links against the
    library and calls its GPU-free entry points."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(capi.LIBPATH)
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.dirname(HEADER),
                    str(src), "-o", str(exe), "-L", libdir, "-lpcaone_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    assert "c caller ok" in out.stdout


def test_stream_plan(lib):
    """The out-of-core block plan (Data::prepare, src/Data.cpp:40-84), host only."""
    stride = lambda n: (n + 127) // 128 * 32  # noqa: E731  device row bytes
    M, N = 1_000_000, 200_000
    # window method: the windows themselves, ceil(M / bands)
    assert capi.stream_plan(M, N, capi.SVD_WINDOW, 64, 0) == (15_625, 64)
    assert capi.stream_plan(M, N, capi.SVD_WINDOW, 64, 2 * 15_625 * stride(N)) == (15_625, 64)
    with pytest.raises(capi.PcaoneError) as e:
        capi.stream_plan(M, N, capi.SVD_WINDOW, 64, 2 * 15_625 * stride(N) - 1)
    assert e.value.code == -6
    assert capi.stream_plan(1001, 16, capi.SVD_WINDOW, 4, 0) == (251, 4)
    # single pass: the in-core blocks of at most 16384 SNPs, balanced ...
    assert capi.stream_plan(M, N, capi.SVD_SINGLE, 64, 0) == (16_130, 62)
    assert capi.stream_plan(16384, N, capi.SVD_SINGLE, 64, 0) == (16_384, 1)
    # ... fewer when two slots of the budget hold fewer rows
    b, nb = capi.stream_plan(M, N, capi.SVD_SINGLE, 64, 2 * 1000 * stride(N))
    assert b <= 1000 and nb == -(-M // 1000) and b == -(-M // nb)
    with pytest.raises(capi.PcaoneError) as e:
        capi.stream_plan(M, N, capi.SVD_SINGLE, 64, stride(N))  # less than a row per slot
    assert e.value.code == -6
    for bad in [(0, N, 1, 64, 0), (M, 0, 1, 64, 0), (M, N, 3, 64, 0), (M, N, 2, 6, 0), (M, N, 2, 2, 0)]:
        with pytest.raises(capi.PcaoneError) as e:
            capi.stream_plan(*bad)
        assert e.value.code == -1


def test_pgen_layout(lib):
    """The .pgen storage modes the library reads itself (no GPU needed)."""
    from tests.cases import pgen_cases, pgen_image
    case = pgen_cases()[0]
    N, M = case.nsamples, case.nsnps
    bps = (N + 3) // 4
    img = pgen_image(case.packed, N)
    assert capi.pgen_layout(img) == {"mode": 2, "nsnps": M, "nsamples": N, "offset": 12, "record_bytes": bps}
    assert capi.pgen_layout(img, N)["mode"] == 2
    # the sample count of the .psam must agree
    with pytest.raises(capi.PcaoneError) as e:
        capi.pgen_layout(img, N + 1)
    assert e.value.code == -1
    # non-reference flags stored after the header shift the records
    flags = bytes((M + 7) // 8)
    img3 = img[:11] + bytes([0xC0]) + flags + img[12:]
    assert capi.pgen_layout(img3)["offset"] == 12 + (M + 7) // 8
    # mode 0x03: hard calls and 2 N bytes of dosages per record
    rec = np.concatenate([case.packed[:, :bps], np.zeros((M, 2 * N), np.uint8)], axis=1)
    img_d = img[:2] + bytes([3]) + img[3:12] + rec.tobytes()
    assert capi.pgen_layout(img_d)["record_bytes"] == bps + 2 * N
    # PLINK 1 rows under a .pgen name: counts from the size and the .psam
    img1 = bytes([0x6C, 0x1B, 0x01]) + case.packed[:, :bps].tobytes()
    assert capi.pgen_layout(img1, N) == {"mode": 1, "nsnps": M, "nsamples": N, "offset": 3, "record_bytes": bps}
    for bad, code in [(img1, -1),                                    # mode 1 without a sample count
                      (img[:-1], -4),                                # truncated
                      (img[:2] + bytes([0x10]) + img[3:], -4),       # variable-width
                      (img[:11] + bytes([1]) + img[12:], -4),        # control byte of a variable-width file
                      (b"\x00\x00\x02" + img[3:], -4)]:           # magic
        with pytest.raises(capi.PcaoneError) as e:
            capi.pgen_layout(bad)
        assert e.value.code == code
