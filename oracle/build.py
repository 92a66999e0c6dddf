"""Build recipe for the CPU oracle (test infrastructure).

Compiles the plain-C restatement (lrt_oracle.c, lrt_oracle_build.c,
lrt_oracle_dr.c) into
oracle/_build/liblrt_oracle.so with OpenMP and -ffp-contract=off.  Only tests,
__graft_entry__.smoke() and bench.py's CPU legs load it.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liblrt_oracle.so")


def build():
    os.makedirs(OUT, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
           "-o", LIB, os.path.join(HERE, "lrt_oracle.c"), os.path.join(HERE, "lrt_oracle_build.c"),
           os.path.join(HERE, "lrt_oracle_dr.c"), "-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("oracle build failed")
    return LIB


if __name__ == "__main__":
    print(build())
