"""Host conductivity helpers of the drop-in C++ interface (electrical_conductivity_coefficients,
2D moment_transform, 2D density_function; reference src/fastkpm.cpp:80-361) against the oracle's
restatement and against direct sums (CPU only). Tolerance 1e-12 relative to the largest entry."""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r'''
#include "fastkpm.h"
#include <cstdio>
using namespace fkpm;
int main() {
    const int M = 12, Mq = 40;
    EnergyScale es{-3.0, 5.0};
    auto g = jackson_kernel(M);
    for (double omega : {0.0, 0.9}) {
        auto c = electrical_conductivity_coefficients(M, Mq, 0.05, 0.4, omega, es, g);
        for (int a = 0; a < M; a++)
            for (int b = 0; b < M; b++) std::printf("%.17g %.17g\n", c[a][b].real(), c[a][b].imag());
    }
    Vec<Vec<cx_double>> mu(M, Vec<cx_double>(M));
    for (int a = 0; a < M; a++)
        for (int b = 0; b < M; b++) mu[a][b] = cx_double(1.0 / (1 + a + 2 * b), 0.1 * (a - b));
    auto gam = moment_transform(mu, 16, g);
    for (int i = 0; i < 16; i++)
        for (int j = 0; j < 16; j++) std::printf("%.17g %.17g\n", gam[i][j].real(), gam[i][j].imag());
    Vec<double> x, y;
    Vec<Vec<cx_double>> rho;
    density_function(gam, es, x, y, rho);
    std::printf("%.17g %.17g %.17g %.17g\n", x[0], y[15], rho[0][0].real(), rho[3][5].imag());
    return 0;
}
'''


@pytest.fixture(scope="module")
def outputs(built_lib, tmp_path_factory):
    d = tmp_path_factory.mktemp("cond")
    src = d / "cond.cpp"
    src.write_text(PROGRAM)
    exe = d / "cond"
    lib_dir = os.path.join(ROOT, "fastkpm_gb300", "_build")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), str(src), "-L" + lib_dir,
                        "-lfastkpm_gb300", "-Wl,-rpath," + lib_dir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    vals = np.array([[float(t) for t in line.split()] for line in r.stdout.strip().splitlines()[:-1]])
    tail = [float(t) for t in r.stdout.strip().splitlines()[-1].split()]
    return vals[:, 0] + 1j * vals[:, 1], tail


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("k,omega", [(0, 0.0), (1, 0.9)])
def test_conductivity_coefficients_match_oracle(outputs, k, omega):
    M, Mq = 12, 40
    got = outputs[0][k * M * M:(k + 1) * M * M].reshape(M, M)
    ref = O.electrical_conductivity_coefficients(M, Mq, 0.05, 0.4, omega, -3.0, 5.0, O.jackson_kernel(M))
    assert _rel(got, ref) <= 1e-12
    if omega == 0.0:
        assert _rel(got, ref.conj().T) <= 1e-12   # the static coefficients are Hermitian


def test_2d_moment_transform_and_density(outputs):
    M, Mq = 12, 16
    got = outputs[0][2 * M * M:].reshape(Mq, Mq)
    g = O.jackson_kernel(M)
    a, b = np.meshgrid(np.arange(M), np.arange(M), indexing="ij")
    mu = 1.0 / (1 + a + 2 * b) + 0.1j * (a - b)
    w = np.where(np.arange(M) == 0, 1.0, 2.0) * g
    mup = np.outer(w, w) * mu
    x = np.cos(np.pi * (np.arange(Mq) + 0.5) / Mq)
    T = np.array([np.cos(m * np.arccos(x)) for m in range(M)])   # T[m, i]
    ref = T.T @ mup @ T
    assert _rel(got, ref) <= 1e-12
    x0, y15, rho00, rho35 = outputs[1]
    mag, avg = 4.0, 1.0
    assert x0 == pytest.approx(x[Mq - 1] * mag + avg, rel=1e-14)
    assert y15 == pytest.approx(x[0] * mag + avg, rel=1e-14)
    i1, i2 = Mq - 1, Mq - 1
    assert rho00 == pytest.approx((ref[i1, i2] / (np.pi * np.sqrt(1 - x[i1] ** 2) * np.pi * np.sqrt(1 - x[i2] ** 2) * mag * mag)).real, rel=1e-12)
    i1, i2 = Mq - 1 - 3, Mq - 1 - 5
    assert rho35 == pytest.approx((ref[i1, i2] / (np.pi * np.sqrt(1 - x[i1] ** 2) * np.pi * np.sqrt(1 - x[i2] ** 2) * mag * mag)).imag, rel=1e-12)
