"""Builds libodil_gb300.so from csrc/*.cu with nvcc for sm_103a.

Each translation unit compiles in parallel to an object file; the objects
link into one shared library with a plain C ABI (no torch symbols), which the
Python host loads with ctypes.  Outputs stay in-tree under odil_gb300/lib/.
"""
import concurrent.futures
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
BUILDDIR = os.path.join(PKG, "_build")
LIBNAME = "libodil_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    cand = [shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build "
                       "libodil_gb300.so")


def cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc_path())))


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith(".cu"))


def _compile(nvcc, src, obj, extra):
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler",
           "-fPIC,-fvisibility=hidden", "--expt-relaxed-constexpr",
           "-I", os.path.join(PKG, "..", "include"), "-c", src, "-o", obj,
           *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" %
                           (os.path.basename(src), r.stdout, r.stderr))
    return r.stderr


def _stale(lib, deps):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    """Compiles (if stale) and returns the path of libodil_gb300.so."""
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BUILDDIR, exist_ok=True)
    lib = os.path.join(LIBDIR, LIBNAME)
    srcs = sources()
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                   if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(PKG, "..", "include", "odil_gb300.h"))
    if not force and not _stale(lib, deps):
        return lib
    nvcc = nvcc_path()
    objs = [os.path.join(BUILDDIR, os.path.basename(s)[:-3] + ".o")
            for s in srcs]
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(
            1, min(len(srcs), os.cpu_count() or 1))) as ex:
        futs = [ex.submit(_compile, nvcc, s, o, list(extra_flags))
                for s, o in zip(srcs, objs)]
        for f in futs:
            msg = f.result()
            if verbose and msg:
                print(msg)
    libdir_cuda = os.path.join(cuda_home(), "lib64")
    tmp = lib + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-L" + libdir_cuda,
           "-Xlinker", "-rpath=" + libdir_cuda, "-lcusparse", "-lcublas", "-lcusolver"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force=True, verbose=True))
