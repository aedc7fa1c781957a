"""The drop-in adapter include/qlten_gb300.h compiles against the reference's own headers
(U1QN / FP64 and fU1U1QN / complex128 instantiations of Contract, SVD, QR,
ContractContiguousAxes, the contiguous accumulate forms and LinearCombine; real and complex
U1QN instantiations of every qlten::dmrg axis entry point). Runs where
the reference tree is available and named by the environment variable QLTEN_REF_TREE;
skipped elsewhere."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("QLTEN_REF_TREE", "")


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "include", "qlten")),
                    reason="reference tree not named by QLTEN_REF_TREE")
def test_adapter_instantiates_against_reference_headers():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    cuda_inc = "/usr/local/cuda/include"
    cmd = [gxx, "-std=c++17", "-fsyntax-only", "-fopenmp", "-DHP_NUMERIC_BACKEND_OPENBLAS",
           f"-I{REF}/include", f"-I{REF}/external/hptt/include", f"-I{ROOT}/oracle/ref/shim",
           f"-I{ROOT}/include", f"-I{cuda_inc}", os.path.join(ROOT, "tests", "adapter", "instantiate.cc")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
