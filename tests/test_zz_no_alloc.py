"""The matvec entry point that allocates no device memory.

Callers that cannot allocate device memory themselves (hosts whose own
allocator or arena owns all device memory, loops that cannot afford an
allocation's synchronisation) use pcaone_gpu_matvec_static on their own device
buffers; its intermediates live in a static device array shared by every
call.  This file is collected last so that a failure here comes after every
other test has run.
"""
import os

import numpy as np
import pytest

from oracle import halko as H
from pcaone_gb300 import build as B
from pcaone_gb300 import capi
from tests.cases import golden_case

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12   # the tolerance of the context matvec test (FP64 sums in another order)


def test_static_matvec_matches_context_matvec_twice():
    torch = pytest.importorskip("torch")
    if not os.path.exists(capi.LIBPATH):
        B.build()
    lib = capi.load()
    case = golden_case("wsvd_n500_k10")
    n, m = case.nsamples, case.nsnps
    rng = np.random.default_rng(5)
    xs = [rng.standard_normal(n), rng.standard_normal(n)]
    with capi.Context() as c:
        c.load_bed(case.packed, n)
        _, F = c.counts()
        refs = [c.matvec(x, standardize=True) for x in xs]
    dev = torch.device("cuda:0")
    d_bed = torch.from_numpy(np.ascontiguousarray(case.packed)).to(dev)
    d_F = torch.from_numpy(F).to(dev)
    d_y = torch.empty(n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    for x, ref in zip(xs, refs):          # two calls in a row share the static scratch
        d_x = torch.from_numpy(x).to(dev)
        d_y.fill_(float("nan"))
        rc = lib.pcaone_gpu_matvec_static(d_bed.data_ptr(), case.packed.shape[1], m, n, d_F.data_ptr(), 1,
                                          d_x.data_ptr(), d_y.data_ptr(), stream.cuda_stream)
        assert rc == 0
        stream.synchronize()
        y = d_y.cpu().numpy()
        assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < REL_TOL
    # and the same against the oracle
    d = H.OracleData(case.packed, n)
    d.standardize_E()
    yr = H.arnoldi_matvec(d, xs[1])
    assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < REL_TOL
    # rows at a wider pitch than the .bed body (padding bytes hold garbage)
    wide = np.full((m, case.packed.shape[1] + 13), 0xA5, dtype=np.uint8)
    wide[:, : case.packed.shape[1]] = case.packed
    d_wide = torch.from_numpy(wide).to(dev)
    rc = lib.pcaone_gpu_matvec_static(d_wide.data_ptr(), wide.shape[1], m, n, d_F.data_ptr(), 1, d_x.data_ptr(),
                                      d_y.data_ptr(), stream.cuda_stream)
    assert rc == 0
    stream.synchronize()
    assert np.linalg.norm(d_y.cpu().numpy() - refs[1]) / np.linalg.norm(refs[1]) < REL_TOL
    # sizes beyond the static array are rejected before any GPU work
    rc = lib.pcaone_gpu_matvec_static(d_bed.data_ptr(), case.packed.shape[1], (1 << 21) + 1, n, d_F.data_ptr(), 1,
                                      d_x.data_ptr(), d_y.data_ptr(), stream.cuda_stream)
    assert rc == -6
