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
