"""The C-ABI library loads and exports every symbol the header declares (no GPU calls)."""
import re
import subprocess

import pytest

from scalit_gb300 import capi

ROOT = __import__("os").path.dirname(__import__("os").path.dirname(__import__("os").path.abspath(__file__)))


def header_functions():
    text = open(f"{ROOT}/include/scalit_gb300.h").read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set()
    for m in re.finditer(r"^(?!typedef)(?:const\s+)?(?:int|void|double|long long|char)\s*\*?\s*"
                         r"([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M):
        names.add(m.group(1))
    return sorted(names)


def test_header_parsed():
    names = header_functions()
    assert "scalit_hx" in names and "qmr_mpi_" in names and "pist_conv_mpi_" in names


def test_every_header_symbol_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", capi.library_path()], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in header_functions() if n not in exported]
    assert not missing, missing


def test_every_header_symbol_bound(lib):
    assert set(header_functions()) == set(capi.SIGNATURES)


def test_fortran_names_are_lowercase_underscored():
    for n in ("h1x_xyz_", "h1x_dep_", "vx_", "vtx_", "hosbdiag_", "qmr_", "qmr_mpi_", "pist_conv_",
              "pist_conv_mpi_", "mgs_orth_", "norm_mpi_", "dotprod_mpi_", "pisth0_", "pisth0_mpi_",
              "hosbdiag_mpi_", "mjacobi_"):
        assert n in capi.SIGNATURES


def test_last_error_callable_without_gpu(lib):
    assert isinstance(lib.scalit_last_error(), bytes)


def test_create_rejects_bad_sizes_without_gpu(lib):
    import ctypes as C
    h = C.c_void_p()
    sizes = (C.c_int * 3)(24, 0, 20)
    rc = lib.scalit_create(C.byref(h), 3, sizes, None, 0, 0)
    assert rc == -101
    assert b"out of range" in lib.scalit_last_error()
