"""TEST INFRASTRUCTURE ONLY: build the CPU oracle as a shared library.

gcc -O2 -ffp-contract=off: no fused multiply-add, the evaluation order of a
baseline x86-64 gfortran -O2 build of the reference.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle_molsim.so")
SRCS = [os.path.join(HERE, f) for f in ("molsim_oracle.c", "oracle_fft.c")]


def build(force=False):
    deps = SRCS + [os.path.join(HERE, "molsim_oracle.h"), os.path.join(HERE, "oracle_par.h"),
                   os.path.join(HERE, "..", "include", "molsim_gb300.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-Wall", "-o", LIB, *SRCS, "-lm"]
    sys.stderr.write("[oracle build] " + " ".join(cmd) + "\n")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
