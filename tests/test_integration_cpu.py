"""The C++ drop-in: integration/SpringNetworkCUDA.{h,cpp} compiled against the reference's own
SpringNetwork.h, linked with the reference's compiled core and the CUDA library, and run beside
the reference's SpringNetwork by integration/drive_springnetwork_cuda.cpp.

Where the reference sources ($REF, else their default mount) or its compiled
core (oracle/_ref/libbsref.so) are absent the test is skipped. Without a CUDA device the driver
must report the library's error as the std::runtime_error the subclass throws; with one, the
two networks must agree after 50 steps."""

from __future__ import annotations

import os
import subprocess

import pytest

from biospring_gb300 import build
from oracle import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cuda_subclass_compiles_links_and_runs(tmp_path):
    ref = pyoracle.reference_dir()
    if not ref or not os.path.exists(os.path.join(ref, "src", "spn", "SpringNetwork.h")):
        pytest.skip("reference sources absent")
    if not pyoracle.have_reference():
        pytest.skip("compiled reference core (oracle/_ref/libbsref.so) absent")
    if not os.path.exists(build.LIB):
        build.build_library()
    cuda_lib = "/usr/local/cuda/lib64"
    exe = str(tmp_path / "drive_springnetwork_cuda")
    ref_dir = os.path.dirname(pyoracle.REF_SO)
    cmd = ["g++", "-std=c++20", "-O2", "-fopenmp", "-DOPENMP_SUPPORT", "-w",
           f"-I{ref}/src", f"-I{ref}/src/spn", f"-I{ref_dir}/gen", f"-I{ref}/src/IO/xdrfile/src",
           f"-I{ROOT}/include", f"-I{ROOT}/integration",
           os.path.join(ROOT, "integration", "SpringNetworkCUDA.cpp"),
           os.path.join(ROOT, "integration", "drive_springnetwork_cuda.cpp"),
           "-o", exe, f"-L{ref_dir}", "-lbsref", f"-L{os.path.dirname(build.LIB)}", "-lbiospring_gb300",
           f"-L{cuda_lib}", "-lcudart",
           f"-Wl,-rpath,{ref_dir}:{os.path.dirname(build.LIB)}:{cuda_lib}"]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert proc.returncode == 0, proc.stdout[-4000:]
    run = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    print(run.stdout)
    assert run.returncode == 0, run.stdout[-4000:]
    out = run.stdout
    assert out.startswith("device-unavailable: bs_create:") or out.startswith("compared:"), out
