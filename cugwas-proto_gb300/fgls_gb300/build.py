"""In-tree build of libfgls_gb300.so (sm_103a) and the CLI driver.

    python -m fgls_gb300.build          (from cugwas-proto_gb300/)

Every .cu under csrc/ is compiled by its own nvcc process in parallel with
``-gencode arch=compute_103a,code=sm_103a``; the objects are linked into
fgls_gb300/lib/libfgls_gb300.so.  The driver (csrc/fgls_driver.c, the
reference's command-line interface) is linked against that library into
fgls_gb300/lib/fgls-driver.  Outputs are git-ignored build artefacts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                    # cugwas-proto_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "libfgls_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def build(verbose: bool = False, force: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    nv = nvcc()
    base = [nv, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
            "--expt-relaxed-constexpr"]
    if ptxas_v:
        base += ["-Xptxas", "-v"]
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "fgls_gb300.h"))
    hdr_mtime = max(os.path.getmtime(h) for h in headers)

    def compile_one(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src[:-3] + ".o")
        if (not force and not ptxas_v and os.path.exists(o)
                and os.path.getmtime(o) >= max(os.path.getmtime(s), hdr_mtime)):
            return o, ""
        out = _run(base + ["-c", s, "-o", o])
        return o, out

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, srcs))
    if verbose or ptxas_v:
        for (o, out) in results:
            if out:
                print(f"== {os.path.basename(o)}\n{out}", file=sys.stderr)
    objs = [o for o, _ in results]
    lib = os.path.join(LIBDIR, LIBNAME)
    tmp = lib + ".tmp"
    _run([nv, ARCH, "-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"])
    os.replace(tmp, lib)
    # command-line driver with the reference's interface (src/driver.c)
    drv = os.path.join(LIBDIR, "fgls-driver")
    _run(["gcc", "-O2", "-std=c11", "-D_FILE_OFFSET_BITS=64", "-I", INCLUDE,
          os.path.join(CSRC, "fgls_driver.c"), "-o", drv, "-L", LIBDIR, "-lfgls_gb300",
          "-Wl,-rpath," + LIBDIR, "-lm"])
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_v="--ptxas" in sys.argv))
