"""The C-ABI library builds for sm_103a, loads without a GPU, and exports
every function that include/dqmc_gpu.h declares (no compute calls here)."""
import ctypes
import os
import re
import subprocess

import pytest

from dqmc_gb300 import api, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "dqmc_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*DQMC_API\s+(?:const\s+)?\w+\*?\s+\*?(dqmc_\w+)\s*\(", txt, flags=re.M)))


@pytest.fixture(scope="module")
def libpath():
    return build.build()


def test_header_parses():
    names = header_functions()
    assert "dqmc_create" in names and "dqmc_sweep" in names and len(names) >= 20


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\s[TW]\s+(dqmc_\w+)$", out, flags=re.M))
    missing = [f for f in header_functions() if f not in exported]
    assert not missing, f"declared but not exported: {missing}"
    # nothing but the C ABI is exported
    assert all(name.startswith("dqmc_") for name in exported)


def test_ctypes_binding_covers_header(libpath):
    assert set(header_functions()) == set(api.SIGNATURES)
    lib = ctypes.CDLL(libpath)
    for name in header_functions():
        assert hasattr(lib, name)


def test_version_string_without_gpu(libpath):
    lib = api.load_library(libpath)
    assert b"sm_103a" in lib.dqmc_version()


def test_params_struct_layout():
    # dqmc_params: 4 int32, 7 doubles, 4 doubles, 5 int32, 3 int32 -> 112 bytes
    assert ctypes.sizeof(api.CParams) == 4 * 4 + 7 * 8 + 4 * 8 + 5 * 4 + 3 * 4


def header_prototypes():
    """name -> number of parameters of every DQMC_API prototype."""
    txt = open(os.path.join(ROOT, "include", "dqmc_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for m in re.finditer(r"DQMC_API\s+[^;(]*?\b(dqmc_\w+)\s*\(([^)]*)\)\s*;", txt, flags=re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_signatures_match_header_arity():
    protos = header_prototypes()
    assert set(protos) == set(header_functions())
    wrong = {n: (len(api.SIGNATURES[n][0]), k) for n, k in protos.items() if len(api.SIGNATURES[n][0]) != k}
    assert not wrong, f"binding argument count differs from the header (binding, header): {wrong}"


def test_kernel_kinds_match_header():
    txt = open(os.path.join(ROOT, "include", "dqmc_gpu.h")).read()
    ids = {int(v) for v in re.findall(r"#define DQMC_K_\w+\s+(\d+)", txt)}
    nk = int(re.search(r"#define DQMC_NKINDS\s+(\d+)", txt).group(1))
    assert ids == set(range(nk)) and len(api.KERNEL_KINDS) == nk
    # names in the header's order: the comment word after each index matches the binding's name
    order = [m.group(1).lower() for m in re.finditer(r"#define DQMC_K_(\w+)\s+\d+", txt)]
    alias = {"slice_cols": "slice_cols", "slice_rows": "slice_rows", "local": "local_updates", "gemm": "zgemm",
             "qrp": "qrp", "applyq": "apply_q", "trsm": "trsm", "misc": "misc", "ozgemm": "ozaki_gemm",
             "flush": "flush", "lu": "lu"}
    assert [alias[o] for o in order] == api.KERNEL_KINDS
