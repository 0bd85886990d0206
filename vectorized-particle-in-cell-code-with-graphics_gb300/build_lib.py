"""Build libpicgb.so (the CUDA step library) in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into a
shared library next to this file.  pgb_fields.cu is compiled with
--fmad=false so that its FP64 multigrid performs the reference's operations
one at a time (no fused multiply-add), which keeps it bit-identical to the
reference's Mglin for the same right-hand side.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "libpicgb.so")
EXE = os.path.join(HERE, "picgb_run")
HOST = os.path.join(HERE, "host")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          f"-I{os.path.join(REPO, 'include')}", f"-I{CSRC}", "-Xptxas", "-warn-spills"]
UNITS = {
    "pgb_api.cu": [],
    "pgb_particles.cu": [],
    "pgb_walls.cu": [],
    "pgb_fields.cu": ["--fmad=false"],
    "pgb_sort.cu": [],
    "pgb_reduce.cu": [],
    "pgb_graphs.cu": [],
    "pgb_render.cu": ["--fmad=false"],
    "pgb_static.cu": [],
    "pgb_dst.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(target: str, deps: list) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(REPO, "include", "picgb.h"))
    jobs = []
    for unit, extra in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
            jobs.append((unit, cmd))
    def run(job):
        unit, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}:\n{p.stdout}\n{p.stderr}")
        if verbose and (p.stdout or p.stderr):
            print(p.stdout + p.stderr, flush=True)
        return unit
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        list(ex.map(run, jobs))
    host_src = os.path.join(HOST, "pic_host.cpp")
    host_objs = []
    for name in ("pic_host.cpp", "pgb_server.cpp"):
        src = os.path.join(HOST, name)
        obj = os.path.join(BUILD, name.replace(".cpp", ".o"))
        host_objs.append(obj)
        if force or _stale(obj, [src, os.path.join(HOST, "pic_host.h")] + headers):
            cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", f"-I{os.path.join(REPO, 'include')}",
                   f"-I{CSRC}", f"-I{HOST}", "-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd), flush=True)
            p = subprocess.run(cmd, capture_output=True, text=True)
            if p.returncode != 0:
                raise RuntimeError(f"g++ failed on {name}:\n{p.stdout}\n{p.stderr}")
            jobs.append((name, None))
    objs = [os.path.join(BUILD, u.replace(".cu", ".o")) for u in UNITS] + host_objs
    if force or jobs or _stale(OUT, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", OUT] + objs + ["-lcudart", "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed:\n{p.stdout}\n{p.stderr}")
    main_src = os.path.join(HOST, "picgb_main.cpp")
    if force or _stale(EXE, [main_src, host_src, OUT, os.path.join(HOST, "pic_host.h")]):
        cmd = ["g++", "-std=c++17", "-O2", "-DPGB_HOST_IN_EXE", f"-I{os.path.join(REPO, 'include')}", f"-I{HOST}",
               f"-I{CSRC}", main_src, host_src, "-o", EXE, f"-L{HERE}", "-lpicgb", "-Wl,-rpath,$ORIGIN"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"g++ failed on picgb_main.cpp:\n{p.stdout}\n{p.stderr}")
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
