"""A C++ program built against the public headers (include/nsfv1_gb300.hpp, the
C++ host class with the reference's element-disc method names, over the C ABI
of include/nsfv1_gb300.h) and linked with libnsfv1_gb300.so, as a host
application of the reference's interface would be.

CPU: it compiles, and its host-only checks pass (setters, string ids, the
reference's error texts, the host pattern build). GPU: its per-element
callbacks (prep_elem + add_def_A_elem / add_jac_A_elem, which add into the
caller's LocalVector / LocalMatrix) equal its batched call bit for bit and
match the oracle within 1e-12.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from _cases import rel_err
from plugin_navierstokes_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "abi_client.cpp")


@pytest.fixture(scope="module")
def client(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib = _capi.LIB_PATH
    exe = str(tmp_path_factory.mktemp("cpp") / "abi_client")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-L", str(lib.parent),
           "-lnsfv1_gb300", f"-Wl,-rpath,{lib.parent}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cpp_client_host_checks(client):
    r = subprocess.run([client], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


@pytest.mark.gpu
def test_cpp_client_element_callbacks_match_the_oracle(client, cuda):
    r = subprocess.run([client, "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout[-2000:] + r.stderr
    vals = {"C": [], "U": [], "D": [], "J": []}
    for line in r.stdout.splitlines():
        if line[:2] in ("C ", "U ", "D ", "J "):
            vals[line[0]].append(float(line[2:]))
    C = np.array(vals["C"]).reshape(2, 8, 3)
    U = np.array(vals["U"]).reshape(2, 32)
    o = oracle.Oracle(3)
    o.set_kinematic_viscosity(0.0025)
    o.set_upwind("lps")
    o.set_stabilization("flow", "raw")
    ref = o.elem_batch(8, C, U, want=("defA", "jacA"))
    assert rel_err(np.array(vals["D"]).reshape(2, 32), ref["defA"]) <= 1e-12
    assert rel_err(np.array(vals["J"]).reshape(2, 1024), ref["jacA"]) <= 1e-12
