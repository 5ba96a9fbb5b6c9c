"""Compile the circuit library (CUDA for sm_103a + host C++) into
legionorigins_gb300/_build/libckt.so, and the measurement and verification
helpers of csrc/tools (include/ckt_tools.h) into _build/libckt_tools.so.

nvcc cross-compiles without a GPU, so this runs anywhere the CUDA toolkit
is installed.  Translation units compile in parallel; the whole build takes
well under a minute.
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
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "libckt.so")
TOOLS = os.path.join(CSRC, "tools")
TOOLS_LIB = os.path.join(BUILD, "libckt_tools.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v", *ARCH]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("CUDA toolkit (nvcc) not found")


def sources(where: str = CSRC) -> list[str]:
    return sorted(os.path.join(where, f) for f in os.listdir(where)
                  if f.endswith((".cu", ".cpp")))


def _newest_input() -> float:
    files = sources() + sources(TOOLS) + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                                          if f.endswith((".h", ".cuh"))]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def _compile(src: str, cuda: str, log: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    inc = ["-I", INCLUDE, "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [os.path.join(cuda, "bin", "nvcc"), "-c", src, "-o", obj, *NVCC_FLAGS, *inc]
    else:
        cmd = [os.environ.get("CXX", "g++"), "-c", src, "-o", obj, *CXX_FLAGS, *inc,
               "-I", os.path.join(cuda, "include")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    log.append(f"$ {' '.join(cmd)}\n{r.stdout}{r.stderr}")
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    return obj


def _link(out: str, objs: list[str], cuda: str, log: list[str], extra: list[str]) -> None:
    tmp = out + ".tmp"
    cmd = [os.path.join(cuda, "bin", "nvcc"), "-shared", *ARCH, "-o", tmp, *objs, *extra,
           "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    log.append(f"$ {' '.join(cmd)}\n{r.stdout}{r.stderr}")
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)


def build(force: bool = False, verbose: bool = False) -> str:
    """Build libckt.so and libckt_tools.so if any source is newer than them;
    return libckt.so's path."""
    newest = _newest_input()
    if not force and all(os.path.exists(p) and os.path.getmtime(p) >= newest
                         for p in (LIB, TOOLS_LIB)):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cuda = _cuda_home()
    log: list[str] = []
    lib_src, tool_src = sources(), sources(TOOLS)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(lambda s: _compile(s, cuda, log), lib_src + tool_src))
    _link(LIB, objs[:len(lib_src)], cuda, log, [])
    # the tools report errors through libckt.so's ckt_last_error
    _link(TOOLS_LIB, objs[len(lib_src):], cuda, log,
          ["-L", BUILD, "-lckt", "-Xlinker", "-rpath=$ORIGIN"])
    with open(os.path.join(BUILD, "build.log"), "w") as f:
        f.write("\n".join(log))
    if verbose:
        print("\n".join(log))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
