"""Out-of-core form (pcaone_gpu_load_bed_stream): the packed rows stay in
pinned host memory and SNP blocks are streamed to two device slots
(FileBed::read_block_initial, src/FilePlink.cpp:122-218; block plan of
Data::prepare, src/Data.cpp:40-84; block loops of computeGandH,
src/Halko.cpp:130-153, 227-268).

With the in-core blocks (no device budget, or one that holds them) a streamed
run executes the same kernels on the same bytes in the same order as an
in-core run, so U, S and V are bit-identical to it: to the in-core run itself
without the window method's shuffle, and with it to the in-core run on the
rows already in the out-of-core order (permute_plink's, which the reference's
-m mode uses instead of the in-core shuffle).  Smaller single-pass blocks
change only the FP64 summation order of H across blocks.  Both are held to
the reference's own out-of-core (-m) outputs at the parity bars.
"""
import os

import numpy as np
import pytest

from pcaone_gb300 import build as B
from pcaone_gb300 import capi
from pcaone_gb300 import halko as HK
from tests.cases import golden_case, golden_cases
from tests.test_gpu_parity import c_params, compare

pytestmark = pytest.mark.gpu

CASES = golden_cases()
IDS = [c.name for c in CASES]
FORMS = {"fp32": capi.PREC_FP32, "bf16": capi.PREC_BF16, "fp8": capi.PREC_FP8}


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not os.path.exists(capi.LIBPATH):
        B.build()
    return capi.load()


def _run(case, precision, stream, budget=0, packed=None, perm=None):
    o = case.opts
    p = c_params(o, precision)
    if perm is not None:
        p.perm = perm
    with capi.Context() as c:
        if stream:
            c.load_bed_stream(case.packed if packed is None else packed, case.nsamples, budget)
        else:
            c.load_bed(case.packed if packed is None else packed, case.nsamples)
        c.set_omega(case.ref["Omg0"])
        U, S, V, it = c.run_halko(p)
        info = c.stream_info()
    return U, S, V, it, info


@pytest.mark.parametrize("form", list(FORMS), ids=list(FORMS))
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_streamed_equals_in_core(case, form):
    if case.opts.perm:
        # the in-core run on the rows in the out-of-core order, without its own shuffle
        order = capi.ooc_order(case.nsnps, case.nsamples, case.opts.bands)
        Ui, Si, Vi, iti, info_i = _run(case, FORMS[form], False, packed=case.packed[order], perm=0)
    else:
        Ui, Si, Vi, iti, info_i = _run(case, FORMS[form], False)
    Us, Ss, Vs, its, info_s = _run(case, FORMS[form], True)
    assert info_i == (False, 0.0)
    streamed, fetched = info_s
    assert streamed
    if form == "fp32":
        assert fetched == 0.0  # the FP32 form reads the pinned rows in place
    else:
        # every epoch streams every block at least once
        stride = (case.nsamples + 127) // 128 * 32
        assert fetched >= case.nsnps * stride
    assert its == iti
    assert np.array_equal(Us, Ui) and np.array_equal(Ss, Si) and np.array_equal(Vs, Vi)


OOC = golden_cases(out_of_core=True)


# the exact tensor-core form at the parity bars, the FP64-grade form at its own
# (tests/test_gpu_fp64_form.py); the FP32 form's streamed runs equal its in-core
# runs bit for bit (above), whose accuracy tests/test_gpu_parity.py holds
OOC_FORMS = {"bf16": (capi.PREC_BF16, 1e-6, 1e-8), "fp64": (capi.PREC_FP64, 2e-8, 2e-9)}


@pytest.mark.parametrize("form", list(OOC_FORMS))
@pytest.mark.parametrize("case", OOC, ids=[c.name for c in OOC])
def test_streamed_vs_reference_out_of_core(case, form):
    """Against the reference's own -m runs (same Omega, same schedule); with the
    window shuffle the working order is the reference's rewritten file order
    (checked first)."""
    o = case.opts
    prec, angle_tol, eig_tol = OOC_FORMS[form]
    with capi.Context() as c:
        c.load_bed_stream(case.packed, case.nsamples, int(o.memory * (1 << 30)))
        c.set_omega(case.ref["Omg0"])
        U, S, V, it = c.run_halko(c_params(o, prec))
        if o.perm:
            assert np.array_equal(c.perm(), case.ref["perm"])
    if o.emu:
        assert abs(it - int(case.ref["meta"][2])) <= 1
    compare(U, S, V, case.ref["U"], case.ref["S"], case.ref["V"], f"{case.name}[{form} streamed]",
            angle_tol=angle_tol, eig_tol=eig_tol)


@pytest.mark.parametrize("name", ["ssvd_n203", "em_ssvd"])
def test_small_blocks_single_pass(name):
    """A budget of two 300-SNP slots: five and four single-pass blocks instead
    of one, against the reference's own outputs at the parity bars."""
    case = golden_case(name)
    stride = (case.nsamples + 127) // 128 * 32
    budget = 2 * 300 * stride
    blk, nblk = capi.stream_plan(case.nsnps, case.nsamples, capi.SVD_SINGLE, 64, budget)
    assert blk <= 300 and nblk >= 4
    U, S, V, it, (streamed, fetched) = _run(case, capi.PREC_BF16, True, budget)
    assert streamed and fetched >= case.nsnps * stride
    compare(U, S, V, case.ref["U"], case.ref["S"], case.ref["V"], f"{name}[streamed {nblk} blocks]")


def test_counts_matvec_and_rows_from_host_copy():
    case = golden_case("wsvd_n301")
    x = np.random.default_rng(5).standard_normal(case.nsamples)
    with capi.Context() as a, capi.Context() as b:
        a.load_bed(case.packed, case.nsamples)
        b.load_bed_stream(case.packed, case.nsamples)
        ca, Fa = a.counts()
        cb, Fb = b.counts()
        assert np.array_equal(ca, cb) and np.array_equal(Fa, Fb)
        assert np.array_equal(a.matvec(x), b.matvec(x))
        # the rows come back with their padding bits cleared, as from the in-core copy
        assert np.array_equal(b.get_bed(), a.get_bed())


def test_window_budget_too_small():
    case = golden_case("wsvd_n301")
    stride = (case.nsamples + 127) // 128 * 32
    win = -(-case.nsnps // case.opts.bands)
    with capi.Context() as c:
        c.load_bed_stream(case.packed, case.nsamples, 2 * win * stride - 1)
        with pytest.raises(capi.PcaoneError) as e:
            c.run_halko(c_params(case.opts, capi.PREC_BF16))
        assert e.value.code == -6


def test_reload_in_core_after_stream():
    """A context switches between the two loads; the second run matches a
    fresh in-core run bit for bit."""
    case = golden_case("wsvd_n301")
    Ui, Si, Vi, _, _ = _run(case, capi.PREC_BF16, False)
    with capi.Context() as c:
        c.load_bed_stream(case.packed, case.nsamples)
        c.set_omega(case.ref["Omg0"])
        c.run_halko(c_params(case.opts, capi.PREC_BF16))
        c.load_bed(case.packed, case.nsamples)
        assert c.stream_info() == (False, 0.0)
        c.set_omega(case.ref["Omg0"])
        U, S, V, _ = c.run_halko(c_params(case.opts, capi.PREC_BF16))
    assert np.array_equal(U, Ui) and np.array_equal(S, Si) and np.array_equal(V, Vi)


def test_mirror_memory_option(tmp_path):
    """FileBed(prefix, memory=GB) takes the out-of-core path (the -m option),
    against the reference's own -m run of the same fileset."""
    case = golden_case("ooc_wsvd_n301")
    prefix = str(tmp_path / "g")
    bps = (case.nsamples + 3) // 4
    with open(prefix + ".bed", "wb") as f:
        f.write(bytes([0x6C, 0x1B, 0x01]) + case.packed[:, :bps].tobytes())
    with open(prefix + ".fam", "w") as f:
        f.writelines(f"f{i} s{i} 0 0 0 -9\n" for i in range(case.nsamples))
    with open(prefix + ".bim", "w") as f:
        f.writelines(f"1 rs{j} 0 {j + 1} A C\n" for j in range(case.nsnps))
    o = case.opts
    p = HK.Param(svd=o.svd, k=o.k, oversamples=o.oversamples, maxp=o.maxp, bands=o.bands, seed=o.seed,
                 rand=o.rand, noshuffle=o.noshuffle, precision=capi.PREC_BF16).finalize()
    fb = HK.FileBed(prefix, memory=o.memory)
    assert fb.out_of_core and fb.ctx.stream_info()[0]
    fb.ctx.set_omega(case.ref["Omg0"])
    res = HK.run_pca_with_halko(fb, p)
    fb.close()
    U, S, V = res[0], res[1], res[2]
    compare(U, S, V, case.ref["U"], case.ref["S"], case.ref["V"], "mirror -m")
