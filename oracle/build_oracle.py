"""Builds the oracle (test infrastructure): oracle/lib/liboracle_h2eri.so from
oracle/h2eri_oracle.c with the system C compiler, OpenMP, portable flags."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "lib", "liboracle_h2eri.so")


def build(verbose=False):
    srcs = [os.path.join(HERE, "h2eri_oracle.c"), os.path.join(HERE, "h2eri_oracle_k.c")]
    hdr = os.path.join(REPO, "include", "h2eri_types.h")
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max([os.path.getmtime(s) for s in srcs] + [os.path.getmtime(hdr)]):
        return LIB
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-std=gnu11", "-ffp-contract=off",
           "-I" + os.path.join(REPO, "include"), "-o", LIB] + srcs + ["-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
