"""The ctypes mirrors of the C-ABI structs have the header's fields, in order,
with matching types; host-only helpers of the library (no GPU needed)."""
import ctypes
import re

import numpy as np
import pytest

from plugin_navierstokes_gb300 import _capi

_CTYPE = {"int": ctypes.c_int, "double": ctypes.c_double, "float": ctypes.c_float, "int64_t": ctypes.c_int64,
          "uint64_t": ctypes.c_uint64}


def _header_struct(name):
    txt = _capi.HEADER.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    end = re.search(r"\}\s*" + name + r"\s*;", txt)
    assert end, name
    start = txt.rfind("typedef struct {", 0, end.start())
    body = txt[start + len("typedef struct {"):end.start()]
    fields = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        if "*" in decl:
            names = [n.strip().lstrip("*") for n in decl.split("*", 1)[1].split(",")]
            fields += [(n, "ptr") for n in names]
            continue
        typ, rest = decl.split(" ", 1)
        if typ == "const":
            typ, rest = rest.split(" ", 1)
        fields += [(n.strip(), typ) for n in rest.split(",")]
    return fields


@pytest.mark.parametrize("cname,pyname", [("nsfv1_newton_params", "NewtonParams"), ("nsfv1_newton_result", "NewtonResult"),
                                          ("nsfv1_batch_options", "BatchOptions"), ("nsfv1_mlp_config", "MlpConfig"),
                                          ("nsfv1_mlp_dataset", "MlpDataset"), ("nsfv1_mlp_train_params", "MlpTrainParams")])
def test_struct_mirrors_match_the_header(cname, pyname):
    hdr = _header_struct(cname)
    py = getattr(_capi, pyname)._fields_
    assert [n for n, _ in hdr] == [n for n, _ in py], (hdr, py)
    for (n, t), (_, pt) in zip(hdr, py):
        if t == "ptr":
            assert pt in (ctypes.c_void_p,), (n, pt)
        else:
            assert pt == _CTYPE[t], (n, t, pt)


def test_condition_matches_the_oracle():
    from oracle import mlp_oracle as mo
    from plugin_navierstokes_gb300.warm_start import condition

    for re_, lid in [(10.0, 0.5), (100.0, 1.25), (1000.0, 2.0), (37.5, 0.9)]:
        assert np.allclose(condition(re_, lid), mo.condition(re_, lid), rtol=1e-6, atol=1e-7)


def test_gemm_split_counts():
    lib = _capi.load()
    assert lib.nsfv1_gemm_bf16_splits(64, 1) == 1
    assert lib.nsfv1_gemm_bf16_splits(4096, 8) == 8
    assert lib.nsfv1_gemm_bf16_splits(640, 3) == 3          # 10 tiles -> chunks of 4, 4, 2
    assert lib.nsfv1_gemm_bf16_splits(128, 16) == 2         # never more splits than K tiles
    assert lib.nsfv1_gemm_bf16_splits(100, 1) == 0          # K must be a multiple of 64


def test_bench_arguments_parse_without_a_gpu():
    import subprocess
    import sys

    r = subprocess.run([sys.executable, "bench.py", "--help"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    for opt in ("--workload", "--impl", "--cells", "--time-steps", "--instances"):
        assert opt in r.stdout
