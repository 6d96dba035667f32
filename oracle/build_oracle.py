"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/kpm_oracle.cpp -- the CPU restatement of the reference's CPU
engine -- into oracle/_build/libkpm_oracle.so with the host C++ compiler.
No -march flags: the same source builds on x86_64 and aarch64 hosts.

The reference itself is not compiled: its public header includes <armadillo>
and its build makes Armadillo and Boost mandatory; neither is installed, so
there is no oracle/_ref.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libkpm_oracle.so")
SRC = os.path.join(HERE, "kpm_oracle.cpp")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "kpm_oracle.h")]
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps)):
        return LIB
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", SRC, "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
