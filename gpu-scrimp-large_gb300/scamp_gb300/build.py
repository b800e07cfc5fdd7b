"""Builds libscamp_gb300.so in-tree with nvcc for sm_103a only, and the
command-line program ``scamp_gb300/scamp`` over it.

Translation units compile in parallel into ``gpu-scrimp-large_gb300/_build``
and link into ``scamp_gb300/libscamp_gb300.so``.  Usage:
    python -m scamp_gb300.build        (from gpu-scrimp-large_gb300/)
or  __graft_entry__.build().
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)              # gpu-scrimp-large_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG_DIR, "libscamp_gb300.so")
CLI_SRC = os.path.join(ROOT, "cli", "scamp_main.cpp")
CLI = os.path.join(PKG_DIR, "scamp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _compile(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("compile failed:\n%s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p.stderr


def build(verbose=False, ptxas_verbose=False):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp = sources()
    jobs = []
    objs = []
    for f in cu:
        o = os.path.join(BUILD, f[:-3] + ".o")
        extra = ["-Xptxas", "-v"] if ptxas_verbose else []
        jobs.append([nvcc] + ARCH + NVCC_FLAGS + extra + ["-c", os.path.join(CSRC, f), "-o", o])
        objs.append(o)
    cxx = os.environ.get("CXX", "g++")
    for f in cpp:
        o = os.path.join(BUILD, f[:-4] + ".o")
        cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
        jobs.append([cxx] + CXX_FLAGS + ["-I" + cuda_inc, "-c", os.path.join(CSRC, f), "-o", o])
        objs.append(o)
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        logs = list(ex.map(_compile, jobs))
    if verbose or ptxas_verbose:
        for j, log in zip(jobs, logs):
            if log.strip():
                sys.stderr.write("== %s\n%s\n" % (os.path.basename(j[-3]), log))
    tmp = LIB + ".tmp"
    _compile([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, LIB)
    # the command-line program (the reference's src/main.cpp) over the library
    tmp = CLI + ".tmp"
    _compile([cxx, "-O2", "-std=c++17", "-I" + INCLUDE, CLI_SRC, "-o", tmp, "-L" + PKG_DIR,
              "-lscamp_gb300", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_verbose="-v" in sys.argv))
