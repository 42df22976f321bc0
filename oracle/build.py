"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``drp_oracle.c`` and ``drp_oracle_tex.c`` (texture sampling)
twice with gcc:

* ``liborc_f32.so`` -- float shading, the bit-exact parity build;
* ``liborc_f64.so`` -- double shading, the gradient / finite-difference build.

Both use ``-ffp-contract=off`` so that every float operation rounds once in
source order (explicit ``fmaf`` is the only fused operation), matching the
CUDA kernels' ``--fmad=false`` contract.  OpenMP is used when the compiler
supports it; otherwise the oracle runs single-threaded.  Outputs go to
``oracle/_build/`` (git-ignored).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRCS = [os.path.join(HERE, "drp_oracle.c"), os.path.join(HERE, "drp_oracle_tex.c")]


def _compile(target, defines, openmp):
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-D_GNU_SOURCE", "-Wall", "-Wno-unknown-pragmas"]
    if openmp:
        cmd.append("-fopenmp")
    cmd += defines + SRCS + ["-o", target, "-lm"]
    return subprocess.run(cmd, capture_output=True, text=True)


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    variants = {
        "liborc_f32.so": ["-DREAL=float"],
        "liborc_f64.so": ["-DREAL=double", "-DREAL_IS_DOUBLE=1"],
    }
    for name, defs in variants.items():
        target = os.path.join(OUT, name)
        if os.path.exists(target) and os.path.getmtime(target) >= max(os.path.getmtime(f) for f in SRCS):
            continue
        r = _compile(target, defs, openmp=True)
        if r.returncode != 0:
            r = _compile(target, defs, openmp=False)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stderr)
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True))
