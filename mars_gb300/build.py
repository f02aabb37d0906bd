"""Build recipe for the GB300 forward-pass library.

Compiles every ``csrc/*.cu`` for sm_103a with nvcc and every ``csrc/*.cpp``
(host code) with g++, one translation unit per process in parallel, and links
``mars_gb300/lib/libmars_gpu.so``, a plain
C-ABI shared library (include/mars_gpu.h) with the CUDA runtime linked
statically. Objects go to ``mars_gb300/_build/``.

Floating-point contraction is off in both device (``--fmad=false``) and host
(``-ffp-contract=off``) code: the kernels spell out every fused multiply-add
they want, so their rounding follows the arithmetic written in the source.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libmars_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.isfile(cand):
            return cand
    raise RuntimeError("nvcc not found (set NVCC or add CUDA to PATH)")


def flags():
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden,-O3",
        "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
    ]


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith(".cu") or f.endswith(".cpp"))


def host_flags():
    # plain C++ (no ISA-specific flags: the library builds on x86_64 and aarch64)
    return ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden",
            "-pthread", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _compile(src, extra):
    base = os.path.basename(src)
    obj = os.path.join(OBJ, base.rsplit(".", 1)[0] + (".cu.o" if base.endswith(".cu") else ".o"))
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC)
                    if h.endswith(".cuh") or h.endswith(".h")]
    deps.append(os.path.join(ROOT, "include", "mars_gpu.h"))
    if os.path.isfile(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj, ""
    if src.endswith(".cpp"):
        cmd = [os.environ.get("CXX", "g++")] + host_flags() + ["-c", src, "-o", obj]
    else:
        cmd = [nvcc()] + flags() + extra + ["-c", src, "-o", obj]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), out.stderr))
    return obj, out.stderr


def build(verbose=False, extra=()):
    """Compile and link; returns the path of libmars_gpu.so."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    objs = [r[0] for r in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    newest = max(os.path.getmtime(o) for o in objs)
    if not (os.path.isfile(LIB) and os.path.getmtime(LIB) >= newest):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-pthread"]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), out.stderr))
    build_marslib(verbose)
    return LIB


PYBIND_SRC = os.path.join(HERE, "pybind", "marslib.cpp")


def pybind_include():
    """Directory holding pybind11/pybind11.h: the pybind11 package, else the
    copy PyTorch ships with its C++ headers; None when neither is there."""
    try:
        import pybind11

        return pybind11.get_include()
    except ImportError:
        pass
    import importlib.util

    spec = importlib.util.find_spec("torch")
    if spec and spec.submodule_search_locations:
        inc = os.path.join(list(spec.submodule_search_locations)[0], "include")
        if os.path.isfile(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    return None


def marslib_path():
    import sysconfig

    return os.path.join(LIB_DIR, "marslib" + sysconfig.get_config_var("EXT_SUFFIX"))


def build_marslib(verbose=False):
    """The compiled `marslib` module (mars_gb300/pybind/marslib.cpp) beside
    libmars_gpu.so, linked to it; skipped (returns None) without pybind11
    headers."""
    import sysconfig

    inc = pybind_include()
    if inc is None:
        if verbose:
            sys.stderr.write("pybind11 headers not found: compiled marslib skipped\n")
        return None
    out_path = marslib_path()
    deps = [PYBIND_SRC, LIB, os.path.join(ROOT, "include", "mars_gpu.h")]
    if os.path.isfile(out_path) and all(os.path.getmtime(out_path) >= os.path.getmtime(d)
                                        for d in deps):
        return out_path
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared",
           "-fvisibility=hidden", "-I" + os.path.join(ROOT, "include"), "-I" + inc,
           "-I" + sysconfig.get_paths()["include"], PYBIND_SRC, "-o", out_path,
           "-L" + LIB_DIR, "-lmars_gpu", "-Wl,-rpath,$ORIGIN"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("marslib build failed:\n%s\n%s" % (" ".join(cmd), out.stderr))
    return out_path


if __name__ == "__main__":
    print(build(verbose=True))
