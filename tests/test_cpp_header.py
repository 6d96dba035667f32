"""The drop-in C++ header (include/fastkpm.h) compiles and links against the in-tree
libfastkpm_gb300.so on the CPU, for the program the GPU test runs, and for double,
cx_double, float and cx_float engines (no device needed to build)."""
import os
import subprocess

import pytest

from tests.conftest import ROOT
from tests.test_gpu_cpp_dropin import PROGRAM

LIB_DIR = os.path.join(ROOT, "fastkpm_gb300", "_build")

ALL_TYPES = r'''
#include "fastkpm.h"
using namespace fkpm;
template <class T> void use() {
    auto e = mk_engine<T>();
    SpMatElems<T> el(4, 4, 1);
    SpMatBsr<T> H(el);
    e->set_H(H, EnergyScale{-1, 1});
    RNG rng(1);
    e->set_R_uncorrelated(4, 2, rng);
    Vec<double> c(8, 0.0);
    auto mu = e->moments(8);
    e->autodiff_matrix(c, H);
    e->stoch_matrix(c, H);
    (void)mu;
}
int main(int argc, char**) {
    if (argc > 5) { use<double>(); use<cx_double>(); use<float>(); use<cx_float>(); }
    return 0;
}
'''


def _build(tmp_path, name, source):
    if not os.path.exists(os.path.join(LIB_DIR, "libfastkpm_gb300.so")):
        pytest.skip("libfastkpm_gb300.so not built")
    src = tmp_path / (name + ".cpp")
    src.write_text(source)
    exe = tmp_path / name
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I" + os.path.join(ROOT, "include"), str(src),
                        "-L" + LIB_DIR, "-lfastkpm_gb300", "-Wl,-rpath," + LIB_DIR, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_dropin_program_builds(tmp_path):
    _build(tmp_path, "dropin", PROGRAM)


def test_every_scalar_type_builds(tmp_path):
    _build(tmp_path, "types", ALL_TYPES)
