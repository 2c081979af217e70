"""include/htool_gpu.hpp compiled against upstream htool's headers.

GpuHMatrix (htool::VirtualHMatrix<double>, types/virtual_hmatrix.hpp:11-76)
and DeviceACA (htool::VirtualLowRankGenerator<double>, lrmat/
virtual_lrmat_generator.hpp:10-18) must be concrete classes that compile
and link against the reference's own headers and this library, so that
htool code can use them unchanged.  tests/adapter/adapter_check.cpp runs
the parts that need no GPU: the cluster hand-over (same permutation, nodes
and block tree as htool's Block::build) and the exceptions.  Only where the
upstream sources are present (oracle.oracle.reference_include); the
single-rank MPI stub and the BLAS forwarding of the oracle's recipe
(oracle/refbuild) stand in for MPI and BLAS.
"""
import os
import subprocess

import pytest

from oracle.oracle import HERE as ORACLE_DIR
from oracle.oracle import reference_include

import htool_gb300 as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_check(tmp_path):
    ref = reference_include()
    if ref is None:
        pytest.skip("upstream htool sources are not on this machine")
    refbuild = os.path.join(ORACLE_DIR, "refbuild")
    subprocess.run(["make", "-s", "REF=" + ref], cwd=refbuild, check=True)  # blas_shim.o
    openblas = subprocess.run(["make", "-s", "-f", "-", "show"], input="include Makefile\nshow:\n\t@echo $(OPENBLAS)\n", cwd=refbuild, capture_output=True, text=True).stdout.strip()
    if not openblas or not os.path.exists(openblas):
        pytest.skip("SciPy's OpenBLAS is not available")
    exe = str(tmp_path / "adapter_check")
    libdir = os.path.dirname(H.LIB_PATH)
    cmd = ["g++", "-std=c++14", "-O1", "-fopenmp", "-w", "-I" + refbuild, "-I" + ref, "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "adapter", "adapter_check.cpp"),
           os.path.join(ORACLE_DIR, "_ref", "blas_shim.o"), openblas, "-L" + libdir, "-lhtgpu", "-Wl,-rpath," + libdir + ":" + os.path.dirname(openblas), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


def test_adapter_compiles_links_and_runs_on_the_host(tmp_path):
    exe = build_check(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, env=dict(os.environ, OPENBLAS_NUM_THREADS="1", CUDA_VISIBLE_DEVICES=""), timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "host: 0 failure(s)" in r.stdout
