"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/qmc_oracle.cpp, the FP64 CPU restatement of the reference's
walker path, into oracle/build/libqmc_oracle.so.  The reference itself is a
Rust crate and there is no Rust toolchain here, so there is no oracle/_ref.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "qmc_oracle.cpp")
OUT_DIR = os.path.join(HERE, "build")
LIB = os.path.join(OUT_DIR, "libqmc_oracle.so")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", SRC, "-o", LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
