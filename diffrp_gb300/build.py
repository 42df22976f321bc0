"""Build libdiffrp_gb300.so for sm_103a with nvcc.

Each ``csrc/*.cu`` translation unit is compiled in parallel
(``-gencode arch=compute_103a,code=sm_103a -O3 -lineinfo --fmad=false``) and
linked into ``diffrp_gb300/_lib/libdiffrp_gb300.so`` (git-ignored).
``--fmad=false`` is part of the numerical contract: forward outputs round
once per operation in source order, so visibility and images are bit-exact
against a CPU evaluation of the same expressions.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "libdiffrp_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "--expt-relaxed-constexpr"]


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "diffrp_gb300.h"))
    return hs


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, force=False):
    os.makedirs(OBJDIR, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([cc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    target = lib_path()
    if force or jobs or _stale(target, objs):
        run([cc] + ARCH + ["-shared", "-o", target] + objs + ["-lcudart"])
    build_fast(force or bool(jobs), verbose)
    return target


FAST_NAME = "_drp_fast.so"


def fast_path():
    return os.path.join(LIBDIR, FAST_NAME)


def build_fast(force=False, verbose=False):
    """The CPython fast path (csrc/pyext.cpp, host C++ only) linked against
    libdiffrp_gb300.so.  Optional: without Python headers or a C++ compiler
    the ctypes binding is used alone."""
    import sysconfig
    src = os.path.join(CSRC, "pyext.cpp")
    out = fast_path()
    header = os.path.join(os.path.dirname(HERE), "include", "diffrp_gb300.h")
    if not force and not _stale(out, [src, header, lib_path()]):
        return out
    inc = sysconfig.get_paths().get("include")
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx or not inc or not os.path.exists(os.path.join(inc, "Python.h")):
        return None
    cmd = [cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden", "-I", inc, src, "-o", out,
           "-L", LIBDIR, "-ldiffrp_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        if verbose:
            print("CPython fast path not built:", r.stderr[-2000:])
        return None
    return out


if __name__ == "__main__":
    print(build(verbose=True))
