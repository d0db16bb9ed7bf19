"""In-tree build of the native engine: nvcc straight to a shared library.

``build_native()`` compiles every translation unit under ``csrc/`` for
sm_103a in parallel and links ``_lib/liblatticeflow_gpu.so`` (CUDA runtime
linked statically, no torch dependency).  Rebuilds only when a source is
newer than the library.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "liblatticeflow_gpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: host double arithmetic (TV set-up and output) rounds
# every operation as written, as the reference's x86 build does; an Arm
# host compiler would otherwise fuse multiply-adds
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
         "-ffp-contract=off", "-I" + INCLUDE]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    p = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(p):
        return p
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + \
        [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build_native(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    cc = nvcc()
    srcs = sources()
    objs = [os.path.join(LIBDIR, os.path.basename(s) + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        cmd = [cc] + FLAGS + ARCH + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-4000:]))
        if verbose:
            print("compiled", os.path.basename(src))
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_native(force=True, verbose=True))
