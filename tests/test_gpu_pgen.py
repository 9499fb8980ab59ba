"""PLINK2 input (pcaone_gpu_load_pgen_file_image / _genovecs): hard calls,
ALT allele counts 0/1/2 with 3 = missing, translated on the device to PLINK 1
codes with A1 = ALT.  Pinned to the reference's own FilePgen runs (through its
pgenlib) on fixed-width .pgen files: allele frequencies bit for bit, PCs at the
parity bars; and bit for bit to the same genotypes loaded as a .bed.
"""
import os

import numpy as np
import pytest

from oracle import halko as H
from pcaone_gb300 import build as B
from pcaone_gb300 import capi
from pcaone_gb300 import halko as HK
from tests.cases import pgen_cases, pgen_image
from tests.test_gpu_parity import c_params, compare

pytestmark = pytest.mark.gpu

CASES = pgen_cases()
IDS = [c.name for c in CASES]
FORMS = {"bf16": (capi.PREC_BF16, 1e-6, 1e-8), "fp64": (capi.PREC_FP64, 2e-8, 2e-9)}


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not os.path.exists(capi.LIBPATH):
        B.build()
    return capi.load()


def _run(load, case, precision):
    with capi.Context() as c:
        load(c)
        cnt, F = c.counts()
        c.set_omega(case.ref["Omg0"])
        U, S, V, it = c.run_halko(c_params(case.opts, precision))
    return cnt, F, U, S, V, it


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_pgen_vs_reference(case, form):
    prec, angle_tol, eig_tol = FORMS[form]
    img = pgen_image(case.packed, case.nsamples)
    cnt, F, U, S, V, it = _run(lambda c: c.load_pgen_file_image(img, case.nsamples), case, prec)
    assert np.array_equal(F, case.ref["F"])  # FilePgen's allele frequencies, bit for bit
    if case.opts.emu:
        assert abs(it - int(case.ref["meta"][2])) <= 1
    compare(U, S, V, case.ref["U"], case.ref["S"], case.ref["V"], f"{case.name}[{form}]", angle_tol=angle_tol,
            eig_tol=eig_tol)


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_pgen_forms_of_input_agree_bit_for_bit(case):
    """The same genotypes as a mode 0x02 image, hard-call rows, a mode 0x03
    image (dosage bytes after each record, not read), PLINK 1 rows under a
    .pgen header (mode 0x01) and a .bed: identical counts and PCs."""
    N, M = case.nsamples, case.nsnps
    bps = (N + 3) // 4
    bed = H.genovec_to_bed(case.packed, N)
    img2 = pgen_image(case.packed, N)
    rec3 = np.concatenate([case.packed[:, :bps], np.full((M, 2 * N), 0x5A, np.uint8)], axis=1)
    img3 = img2[:2] + bytes([3]) + img2[3:12] + rec3.tobytes()
    img1 = bytes([0x6C, 0x1B, 0x01]) + np.ascontiguousarray(bed[:, :bps]).tobytes()
    loads = {
        "bed": lambda c: c.load_bed(bed, N),
        "mode2": lambda c: c.load_pgen_file_image(img2, N),
        "genovecs": lambda c: c.load_pgen_genovecs(case.packed, N),
        "mode3": lambda c: c.load_pgen_file_image(img3, 0),
        "mode1": lambda c: c.load_pgen_file_image(img1, N),
    }
    out = {k: _run(f, case, capi.PREC_BF16) for k, f in loads.items()}
    for k in loads:
        for a, b in zip(out[k][:5], out["bed"][:5]):
            assert np.array_equal(a, b), k


def test_pgen_rejects():
    case = CASES[0]
    img = pgen_image(case.packed, case.nsamples)
    with capi.Context() as c:
        for bad, code in [(img[:2] + bytes([0x10]) + img[3:], -4), (img[:-3], -4)]:
            with pytest.raises(capi.PcaoneError) as e:
                c.load_pgen_file_image(bad, case.nsamples)
            assert e.value.code == code
        with pytest.raises(capi.PcaoneError) as e:
            c.load_pgen_file_image(img, case.nsamples + 4)
        assert e.value.code == -1


def test_mirror_file_pgen(tmp_path):
    """FilePgen(prefix) reads the .psam and .pgen like the reference (-p)."""
    case = CASES[0]
    prefix = str(tmp_path / "g")
    with open(prefix + ".pgen", "wb") as f:
        f.write(pgen_image(case.packed, case.nsamples))
    with open(prefix + ".psam", "w") as f:
        f.write("#IID\n" + "".join(f"s{i}\n" for i in range(case.nsamples)))
    o = case.opts
    p = HK.Param(svd=o.svd, k=o.k, oversamples=o.oversamples, maxp=o.maxp, bands=o.bands, seed=o.seed, rand=o.rand,
                 noshuffle=o.noshuffle, emu=o.emu, maxiter=o.maxiter, precision=capi.PREC_BF16).finalize()
    fp = HK.FilePgen(prefix)
    assert (fp.nsamples, fp.nsnps) == (case.nsamples, case.nsnps)
    assert np.array_equal(fp.F, case.ref["F"])
    fp.ctx.set_omega(case.ref["Omg0"])
    U, S, V, _ = HK.run_pca_with_halko(fp, p)
    fp.close()
    compare(U, S, V, case.ref["U"], case.ref["S"], case.ref["V"], "mirror -p")
