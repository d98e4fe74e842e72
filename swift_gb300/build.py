"""In-tree build of the CUDA library (libswift_gb300.so) and the swift CLI.

Every translation unit is compiled for sm_103a only; objects go to
swift_gb300/_build/, the shared library and the CLI next to this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libswift_gb300.so")
CLI = os.path.join(HERE, "swift")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-O2", *extra]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
               if f.endswith(".h") or f.endswith(".cuh")]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "swift_gb300.h"))
    srcs = sorted(f for f in os.listdir(CSRC)
                  if (f.endswith(".cu") or f.endswith(".cpp")) and f != "cli.cpp")
    cc = nvcc()
    jobs = []
    objs = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _stale(obj, [src, *headers, __file__]):
            extra = ["-Xptxas", "-v"] if (ptxas_info and s.endswith(".cu")) else []
            jobs.append([cc, *_flags(extra), "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0 or ptxas_info:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("compile failed: " + " ".join(cmd))
    if _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB, *headers]):
        cmd = [cc, *_flags(), "-o", CLI, cli_src, "-L" + HERE, "-lswift_gb300",
               "-Xlinker", "-rpath=$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("CLI link failed")
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
