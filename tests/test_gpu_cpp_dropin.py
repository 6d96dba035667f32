"""The drop-in C++ interface (include/fastkpm.h) on the GPU: a program written
against fkpm::Engine<cx_double> exactly as a FastKPM caller would (SpMatElems ->
SpMatBsr, mk_engine, set_H, set_R_correlated, moments, autodiff_matrix,
stoch_matrix) is compiled, linked to libfastkpm_gb300.so and run; its R, moments
and D are compared with the product's probe generator and the oracle
(FP64 tolerance: 1e-10 relative)."""
import os
import subprocess

import numpy as np
import pytest

import fastkpm_gb300 as fk
from fastkpm_gb300 import workloads as W
from oracle import oracle as O
from tests.conftest import ROOT

pytestmark = pytest.mark.gpu

PROGRAM = r'''
#include "fastkpm.h"
#include <cstdio>
#include <fstream>
#include <vector>
using namespace fkpm;
template <class T> std::vector<T> rd(const char* path) {
    std::ifstream f(path, std::ios::binary); f.seekg(0, std::ios::end); size_t n = f.tellg(); f.seekg(0);
    std::vector<T> v(n / sizeof(T)); f.read((char*)v.data(), n); return v;
}
template <class T> void wr(const char* path, const T* p, size_t n) {
    std::ofstream f(path, std::ios::binary); f.write((const char*)p, n * sizeof(T));
}
int main(int argc, char** argv) {
    // blocks as unsorted (i, j, 2x2 column-major block) triples
    auto ri = rd<int>(argv[1]); auto ci = rd<int>(argv[2]); auto vv = rd<cx_double>(argv[3]);
    auto groups = rd<int>(argv[4]); auto es_v = rd<double>(argv[5]); auto c = rd<double>(argv[6]);
    const int n_b = (int)groups.size() / 2, M = (int)c.size();
    SpMatElems<cx_double> el(n_b, n_b, 2);
    for (size_t k = 0; k < ri.size(); k++) el.add(ri[k], ci[k], &vv[4 * k]);
    SpMatBsr<cx_double> H(el);
    EnergyScale es{es_v[0], es_v[1]};
    auto engine = mk_engine<cx_double>();
    engine->set_H(H, es);
    RNG rng(1234);
    engine->set_R_correlated(groups, rng);
    wr("R.bin", engine->R.memptr(), engine->R.size());
    auto mu = engine->moments(M);
    wr("mu.bin", mu.data(), mu.size());
    SpMatBsr<cx_double> D = H;
    engine->autodiff_matrix(c, D);
    wr("D_auto.bin", D.val.data(), D.val.size());
    engine->stoch_matrix(c, D);
    wr("D_stoch.bin", D.val.data(), D.val.size());
    auto es2 = engine->energy_scale(H, 0.0, 200);
    wr("es.bin", &es2.lo, 1); wr("es_hi.bin", &es2.hi, 1);
    std::printf("ok %d %d\n", H.n_blocks(), M);
    return 0;
}
'''


def test_cpp_dropin_engine_on_gpu(gpu, tmp_path):
    src = tmp_path / "dropin_gpu.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "dropin_gpu"
    lib_dir = os.path.join(ROOT, "fastkpm_gb300", "_build")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), str(src), "-L" + lib_dir,
                        "-lfastkpm_gb300", "-Wl,-rpath," + lib_dir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # inputs: the cubic L=4 spin lattice, shuffled so SpMatBsr's build has to sort
    H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, seed=2)
    rng = np.random.default_rng(0)
    order = rng.permutation(H.n_blocks())
    blocks = H.val.reshape(-1, 4)
    groups = W.cubic_colour_groups(4, 2)
    M = 30
    c = W.fermi_coefficients(M, es, "fermi_energy")
    files = {"ri.bin": H.row_idx[order].astype(np.int32), "ci.bin": H.col_idx[order].astype(np.int32),
             "v.bin": np.ascontiguousarray(blocks[order]).astype(np.complex128), "g.bin": groups.astype(np.int32),
             "es.in": np.array([es.lo, es.hi]), "c.bin": c}
    for k, v in files.items():
        v.tofile(str(tmp_path / k))
    r = subprocess.run([str(exe)] + [str(tmp_path / k) for k in files], capture_output=True, text=True, cwd=tmp_path,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    n = H.n_rows * 2
    R = np.fromfile(tmp_path / "R.bin", np.complex128).reshape((n, -1), order="F")
    R_ref = fk.probe_correlated(groups, fk.RNG(1234), complex_values=True)
    assert np.array_equal(R, R_ref)
    o = O.OracleEngine(True)
    o.set_H(H, es)
    o.set_R(R_ref)
    mu_ref = o.moments(M)
    mu = np.fromfile(tmp_path / "mu.bin")
    assert np.max(np.abs(mu - mu_ref)) / abs(mu_ref[0]) <= 1e-10
    D_ref = o.autodiff_matrix(c, H)
    D = np.fromfile(tmp_path / "D_auto.bin", np.complex128)
    assert np.linalg.norm(D - D_ref) <= 1e-10 * np.linalg.norm(D_ref)
    D_ref = o.stoch_matrix(c, H)
    D = np.fromfile(tmp_path / "D_stoch.bin", np.complex128)
    assert np.linalg.norm(D - D_ref) <= 1e-10 * np.linalg.norm(D_ref)
    lam = np.linalg.eigvalsh(H.to_dense())
    lo, hi = np.fromfile(tmp_path / "es.bin")[0], np.fromfile(tmp_path / "es_hi.bin")[0]
    assert abs(lo - lam.min()) < 1e-6 and abs(hi - lam.max()) < 1e-6


SPLIT_PROGRAM = r'''
#include "fastkpm.h"
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <vector>
using namespace fkpm;
template <class T> std::vector<T> rd(const char* path) {
    std::ifstream f(path, std::ios::binary); f.seekg(0, std::ios::end); size_t n = f.tellg(); f.seekg(0);
    std::vector<T> v(n / sizeof(T)); f.read((char*)v.data(), n); return v;
}
template <class T> void wr(const std::string& path, const T* p, size_t n) {
    std::ofstream f(path, std::ios::binary); f.write((const char*)p, n * sizeof(T));
}
int main(int argc, char** argv) {
    auto ri = rd<int>(argv[1]); auto ci = rd<int>(argv[2]); auto vv = rd<cx_double>(argv[3]);
    auto groups = rd<int>(argv[4]); auto es_v = rd<double>(argv[5]); auto c = rd<double>(argv[6]);
    const int n_b = (int)groups.size() / 2, M = (int)c.size();
    SpMatElems<cx_double> el(n_b, n_b, 2);
    for (size_t k = 0; k < ri.size(); k++) el.add(ri[k], ci[k], &vv[4 * k]);
    SpMatBsr<cx_double> H(el);
    EnergyScale es{es_v[0], es_v[1]};
    for (int nd : {1, 2, 3}) {
        auto engine = mk_engine_cuSPARSE<cx_double>(Vec<int>(nd, 0));   // nd engines, all on device 0
        engine->set_H(H, es);
        RNG rng(77);
        engine->set_R_correlated(groups, rng);
        const unsigned next = rng();   // the master generator advanced by one draw per column
        auto mu = engine->moments(M);
        SpMatBsr<cx_double> D = H;
        engine->autodiff_matrix(c, D);
        const std::string tag = std::to_string(nd);
        wr("mu" + tag + ".bin", mu.data(), mu.size());
        wr("Da" + tag + ".bin", D.val.data(), D.val.size());
        engine->stoch_matrix(c, D);
        wr("Ds" + tag + ".bin", D.val.data(), D.val.size());
        wr("next" + tag + ".bin", &next, 1);
        bool threw = false;
        try { engine->moments2_v2(4, H, H); } catch (std::exception&) { threw = true; }
        wr("v2" + tag + ".bin", &threw, 1);
    }
    std::printf("ok\n");
    return 0;
}
'''


def test_cpp_probe_split_engines_match_one_engine(gpu, tmp_path):
    """mk_engine_cuSPARSE with 2 and 3 device entries (all device 0 here: one GPU per box) splits R's
    columns over 2 and 3 engines and sums moments and D on the host (the reference's threaded
    engine): equal to the one-engine results and the oracle to 1e-10; the master generator ends
    in the same state; moments2_v2 refuses a split engine."""
    src = tmp_path / "split.cpp"
    src.write_text(SPLIT_PROGRAM)
    exe = tmp_path / "split"
    lib_dir = os.path.join(ROOT, "fastkpm_gb300", "_build")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), str(src), "-L" + lib_dir,
                        "-lfastkpm_gb300", "-Wl,-rpath," + lib_dir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, seed=8)
    groups = W.cubic_colour_groups(4, 2)   # 16 colour columns: 8, (5, 5, 6) per engine
    M = 24
    c = W.fermi_coefficients(M, es, "fermi_energy")
    files = {"ri.bin": H.row_idx.astype(np.int32), "ci.bin": H.col_idx.astype(np.int32),
             "v.bin": np.ascontiguousarray(H.val).astype(np.complex128), "g.bin": groups.astype(np.int32),
             "es.in": np.array([es.lo, es.hi]), "c.bin": c}
    for k, v in files.items():
        v.tofile(str(tmp_path / k))
    r = subprocess.run([str(exe)] + [str(tmp_path / k) for k in files], capture_output=True, text=True, cwd=tmp_path,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    R_ref = fk.probe_correlated(groups, fk.RNG(77), complex_values=True)
    o = O.OracleEngine(True)
    o.set_H(H, es)
    o.set_R(R_ref)
    mu_ref = o.moments(M)
    Da_ref = o.autodiff_matrix(c, H)
    Ds_ref = o.stoch_matrix(c, H)
    one = {k: np.fromfile(tmp_path / (k + "1.bin"), dt) for k, dt in
           [("mu", np.float64), ("Da", np.complex128), ("Ds", np.complex128), ("next", np.uint32)]}
    for nd in (1, 2, 3):
        mu = np.fromfile(tmp_path / ("mu%d.bin" % nd))
        Da = np.fromfile(tmp_path / ("Da%d.bin" % nd), np.complex128)
        Ds = np.fromfile(tmp_path / ("Ds%d.bin" % nd), np.complex128)
        assert np.max(np.abs(mu - mu_ref)) / abs(mu_ref[0]) <= 1e-10
        assert np.linalg.norm(Da - Da_ref) <= 1e-10 * np.linalg.norm(Da_ref)
        assert np.linalg.norm(Ds - Ds_ref) <= 1e-10 * np.linalg.norm(Ds_ref)
        assert np.max(np.abs(mu - one["mu"])) / abs(mu_ref[0]) <= 1e-12
        assert np.fromfile(tmp_path / ("next%d.bin" % nd), np.uint32)[0] == one["next"][0]
        assert bool(np.fromfile(tmp_path / ("v2%d.bin" % nd), np.uint8)[0]) == (nd > 1)
