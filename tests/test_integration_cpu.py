"""The reference-side binding shown in INTEGRATION.md (the adapter header
src/HalkoGpu.hpp a maintainer adds to PCAone) compiles against the
reference's own headers and include/pcaone_gpu.h, and links against the
library's exported symbols.  Needs the reference tree (PCAONE_REF_TREE, or
the copy staged in oracle/_ref/tree); skipped without it."""
import os
import re
import subprocess

import pytest

from pcaone_gb300 import capi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ref_tree():
    for cand in (os.environ.get("PCAONE_REF_TREE"), os.path.join(REPO, "oracle", "_ref", "tree")):
        if cand and os.path.isfile(os.path.join(cand, "src", "Halko.hpp")):
            return cand
    return None


def _adapter_source():
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, re.S)
    src = [b for b in blocks if b.startswith("// file: src/HalkoGpu.hpp")]
    assert len(src) == 1, "INTEGRATION.md must hold exactly one src/HalkoGpu.hpp block"
    return src[0]


def test_adapter_compiles_against_the_reference_headers(tmp_path):
    tree = _ref_tree()
    if tree is None:
        pytest.skip("no reference tree to compile against")
    (tmp_path / "HalkoGpu.hpp").write_text(_adapter_source())
    unit = tmp_path / "use.cpp"
    unit.write_text('#include "HalkoGpu.hpp"\n'
                    'void use(Data* d, const Param& p) { run_pca_with_halko_gpu(d, p); }\n'
                    'void use2(pcaone_gpu_ctx* c, const double* x, double* y) { perform_op_gpu(c, x, y, true); }\n')
    obj = tmp_path / "use.o"
    cmd = ["g++", "-std=c++17", "-DWITH_GB300", "-w", "-c", str(unit), "-o", str(obj), f"-I{tmp_path}",
           f"-I{os.path.join(REPO, 'include')}", f"-I{tree}/src", f"-I{tree}/external", f"-I{tree}/external/zstd/lib",
           f"-I{tree}/external/pgenlib"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # every pcaone_gpu_* symbol the adapter needs is exported by the library
    nm = subprocess.run(["nm", "-u", str(obj)], capture_output=True, text=True).stdout
    needed = sorted(set(re.findall(r"\b(pcaone_gpu_\w+)", nm)))
    assert needed and all(n in capi.EXPORTS for n in needed), needed
