"""The C-ABI library loads and exports every function include/*.h declares; the
drop-in C++ header compiles, links and fails loudly without a GPU (no CPU
fallback). No device compute here."""
import ctypes
import os
import re
import subprocess

import pytest

from tests.conftest import ROOT


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        if "extern \"C\"" not in src:
            continue
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(fk_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported(built_lib):
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(built_lib, n)]
    assert not missing, missing


def test_status_strings_and_version(built_lib):
    assert b"sm_103a" in built_lib.fk_version()
    assert built_lib.fk_status_string(0) == b"ok"
    assert built_lib.fk_status_string(3) == b"malformed sparsity pattern"


def test_engine_create_validates_arguments(built_lib):
    h = ctypes.c_void_p()
    assert built_lib.fk_engine_create(0, 7, 0, ctypes.byref(h)) == 1   # bad kind
    assert built_lib.fk_engine_create(0, 0, 9, ctypes.byref(h)) == 1   # bad precision
    assert built_lib.fk_engine_create(0, 0, 0, None) == 1


def test_cpp_dropin_header_compiles_and_links(built_lib, tmp_path):
    src = tmp_path / "dropin.cpp"
    src.write_text(r'''
#include "fastkpm.h"
#include <cstdio>
#include <stdexcept>
int main() {
    using namespace fkpm;
    SpMatElems<cx_double> el(4, 4, 2);
    cx_double blk[4] = {1.0, 0.0, 0.0, 1.0};
    for (int i = 0; i < 4; i++) { el.add(i, i, blk); el.add(i, (i + 1) % 4, blk); el.add((i + 1) % 4, i, blk); }
    SpMatBsr<cx_double> H(el);
    if (H.n_blocks() != 12 || H.row_ptr[4] != 12) return 2;
    auto c = expansion_coefficients(20, 40, [](double x) { return fermi_density(x, 0.0, 0.0); }, EnergyScale{-3, 3});
    if (c.size() != 20) return 3;
    try { mk_engine_cpu<double>(); return 4; } catch (std::runtime_error&) {}
    try { auto e = mk_engine<double>(); (void)e; std::printf("gpu\n"); } catch (std::runtime_error& e) { std::printf("nogpu\n"); }
    return 0;
}
''')
    exe = tmp_path / "dropin"
    lib_dir = os.path.join(ROOT, "fastkpm_gb300", "_build")
    r = subprocess.run(["g++", "-std=c++17", "-I" + os.path.join(ROOT, "include"), str(src), "-L" + lib_dir,
                        "-lfastkpm_gb300", "-Wl,-rpath," + lib_dir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() in ("gpu", "nogpu")


def test_library_uses_no_blas(built_lib):
    # every product on the path, the second-order moments' FP64 products included, is a kernel of
    # this library: the shared object links no BLAS and references no BLAS symbol
    from fastkpm_gb300 import _lib
    deps = subprocess.run(["ldd", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "cublas" not in deps.lower()
    syms = subprocess.run(["nm", "-D", "--undefined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "cublas" not in syms.lower()
