"""Build the native library numcosmo_gb300/lib/libncg.so for sm_103a.

CUDA translation units are compiled by nvcc (-gencode arch=compute_103a,code=sm_103a),
the host C files by gcc, in parallel, and linked with the static CUDA runtime.
Objects go to numcosmo_gb300/_build/, the library to numcosmo_gb300/lib/.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libncg.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("CUDA toolkit not found (nvcc)")


def sources() -> tuple[list[str], list[str]]:
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    c = sorted(f for f in os.listdir(CSRC) if f.endswith(".c"))
    return cu, c


def _headers_digest() -> str:
    h = hashlib.sha1()
    for d in (CSRC, INCLUDE):
        for f in sorted(os.listdir(d)):
            if f.endswith((".h", ".cuh")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(fh.read())
    return h.hexdigest()[:12]


def _needs(obj: str, src: str, stamp: str) -> bool:
    return (not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(src)
            or os.path.getmtime(obj) < os.path.getmtime(stamp))


def build(verbose: bool = False, jobs: int | None = None) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)

    # header changes rebuild everything
    stamp = os.path.join(BUILD, "headers." + _headers_digest())
    if not os.path.exists(stamp):
        for f in os.listdir(BUILD):
            if f.startswith("headers."):
                os.remove(os.path.join(BUILD, f))
        open(stamp, "w").close()

    cu, c = sources()
    inc = [f"-I{CSRC}", f"-I{INCLUDE}", f"-I{os.path.join(cuda, 'include')}"]
    cmds = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _needs(obj, src, stamp):
            cmds.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-warn-spills", *inc, "-c", src, "-o", obj])
    for f in c:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _needs(obj, src, stamp):
            cmds.append(["gcc", "-O2", "-std=gnu11", "-fPIC", "-Wall", "-Wno-unused-function",
                         *inc, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return r

    if cmds:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
            list(ex.map(run, cmds))

    if cmds or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread", "-lrt", "-ldl"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
