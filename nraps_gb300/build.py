"""Build recipe for libnraps_gb300.so (sm_103a, in-tree).

Each .cu is compiled separately by nvcc for `-gencode arch=compute_103a,
code=sm_103a`, the host .cpp files by g++, in parallel, then linked into
nraps_gb300/_build/libnraps_gb300.so against the shared CUDA runtime (the
same libcudart that PyTorch loads, so streams and events interoperate).
nraps_main.cpp becomes the command-line program nraps_gb300/_build/nraps,
which finds the library beside itself.

Flags that carry meaning:
  -ffp-contract=off   host code: table arithmetic must round as written on
                      both x86_64 and aarch64 (GCC fuses multiply-adds on
                      aarch64 by default).
  --fmad=false        plain.cu, bank.cu and noalloc.cu: the plain kernel and
                      its derived tables reproduce a CPU restatement bit for
                      bit.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libnraps_gb300.so")
CLI = os.path.join(OUT, "nraps")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = {
    "plain.cu": ["--fmad=false"],
    "bank.cu": ["--fmad=false"],
    "engine.cu": [],
    "event.cu": [],
    "noalloc.cu": ["--fmad=false"],
    "serve.cu": [],
}
CPP_SOURCES = ["host_frontend.cpp", "host_output.cpp", "host_diffusion.cpp", "tables.cpp"]
CLI_SOURCE = "nraps_main.cpp"  # the `nraps` program, linked against the library


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _deps() -> list[str]:
    out = [os.path.join(ROOT, "include", "nraps_gpu.h")]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.stderr.strip() and os.environ.get("NRAPS_BUILD_VERBOSE"):
        sys.stderr.write(r.stderr)


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    deps = _deps()
    if not force and not _stale(LIB, deps) and not _stale(CLI, deps):
        return LIB
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    jobs = []
    objs = []
    for src, extra in CU_SOURCES.items():
        obj = os.path.join(OUT, src + ".o")
        cmd = [nvcc, *ARCH, *common, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose_ptxas:
            cmd += ["-Xptxas", "-v"]
        jobs.append(cmd)
        objs.append(obj)
    for src in CPP_SOURCES + [CLI_SOURCE]:
        obj = os.path.join(OUT, src + ".o")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
               "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
               "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append(cmd)
        if src != CLI_SOURCE:
            objs.append(obj)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-cudart", "shared", *objs, "-o", tmp,
          "-Xlinker", "-rpath", "-Xlinker", os.path.join(cuda, "lib64")])
    os.replace(tmp, LIB)
    tmp = CLI + ".tmp"
    _run(["g++", os.path.join(OUT, CLI_SOURCE + ".o"), "-o", tmp, "-L", OUT, "-lnraps_gb300",
          "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
