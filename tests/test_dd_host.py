"""Double-float arithmetic of the small Cholesky factor, checked on the host.

The (k+p)^2 Cholesky and triangular inverse of CholeskyQR run on the GPU in
double-float arithmetic (pcaone_gb300/csrc/dd.cuh); the same header compiles
for the host, where tests/dd_check.cpp measures each operation against long
double and runs the right-looking factorisation and inverse the kernel uses.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def dd_results(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("dd") / "dd_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "dd_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return {k: float(v) for k, v in (line.split() for line in out.strip().splitlines())}


def test_single_operations_near_2_to_minus_46(dd_results):
    for op in ("op_mul", "op_div", "op_sqrt", "op_add"):
        assert dd_results[op] < 2.0 ** -46, (op, dd_results[op])


@pytest.mark.parametrize("L", [1, 2, 5, 40, 48, 64, 112])
def test_cholesky_and_inverse(dd_results, L):
    # R^T R reproduces the Gram matrix and X R = I to ~48-bit accuracy
    assert dd_results[f"chol_L{L}"] < 2e-14
    assert dd_results[f"inv_L{L}"] < 2e-14


def test_integer_split_and_merge(dd_results):
    """The tall products' split of a double into a float pair from its bits
    (no FP64 arithmetic) keeps 46 bits; the merge equals (double)hi +
    (double)lo; zero and exact values split exactly."""
    assert dd_results["split"] < 2.0 ** -46
    assert dd_results["merge"] == 0.0
    assert dd_results["split_exact"] == 0.0
