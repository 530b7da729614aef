"""Recipe that compiles the unmodified reference H2P-ERI C sources into
oracle/_ref/libh2peri_ref.so (test infrastructure only).

Inputs: the reference sources under /root/reference/src (read in place, never
copied), the shims in oracle/ref_shim (SIMINT-API subset, CBLAS forwarding to
scipy's bundled OpenBLAS, empty LAPACKE header, a small driver) and the
project's integral engine h2p-eri_gb300/csrc/host/h2g_ints.c, which stands in
for SIMINT. Flags follow the reference makefile (src/common.make:12,19-22):
-O2 -fPIC -std=gnu11 -fopenmp. The library exists only where the reference
tree is present; it never ships to the GPU host.
"""
import glob
import os
import subprocess
import sys

REF_SRC = "/root/reference/src"
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def available():
    """True where the reference sources exist (the machine the repository is
    developed on); elsewhere the reference build is skipped."""
    return os.path.isdir(REF_SRC)


def openblas_lib():
    import scipy
    libdir = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    libs = sorted(glob.glob(os.path.join(libdir, "libscipy_openblas*.so")))
    if not libs:
        raise RuntimeError("scipy's bundled OpenBLAS not found")
    return libs[0]


def build(verbose=True):
    if not os.path.isdir(REF_SRC):
        if verbose:
            print("reference sources absent; oracle/_ref not built")
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libh2peri_ref.so")
    srcs = sorted(glob.glob(os.path.join(REF_SRC, "*.c")))
    srcs += [os.path.join(HERE, "ref_shim", f) for f in ("simint_shim.c", "cblas_shim.c", "ref_driver.c")]
    srcs += [os.path.join(REPO, "h2p-eri_gb300", "csrc", "host", "h2g_ints.c")]
    newest = max(os.path.getmtime(s) for s in srcs + [__file__])
    if os.path.exists(out) and os.path.getmtime(out) > newest:
        return out
    blas = openblas_lib()
    cmd = ["gcc", "-O2", "-fPIC", "-std=gnu11", "-fopenmp", "-shared", "-w",
           "-Wl,-Bsymbolic",
           "-I" + os.path.join(HERE, "ref_shim"), "-I" + REF_SRC,
           "-I" + os.path.join(REPO, "h2p-eri_gb300", "csrc", "host"),
           "-o", out] + srcs + [blas, "-Wl,-rpath," + os.path.dirname(blas), "-lm", "-lpthread"]
    if verbose:
        print(" ".join(cmd[:12]), "...")
    subprocess.check_call(cmd)
    return out


if __name__ == "__main__":
    print(build())
