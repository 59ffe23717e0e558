"""Build libtedq_gb300.so for GB300 (sm_103a) in-tree.

    python ted-q_gb300/csrc/build.py [--jobs N] [--verbose]

Compiles the CUDA sources with ``nvcc -gencode arch=compute_103a,code=sm_103a``
and the host sources with g++, in parallel, into ``ted-q_gb300/_build/`` and
links ``ted-q_gb300/tedq_gb300/libtedq_gb300.so`` (static CUDA runtime).
Works on x86-64 and aarch64 hosts (no architecture-specific host flags).
"""

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
REPO = os.path.dirname(PKG_ROOT)
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(PKG_ROOT, "_build")
OUT = os.path.join(PKG_ROOT, "tedq_gb300", "libtedq_gb300.so")

CU_SOURCES = ["sv_kernels.cu", "noalloc.cu", "tn_kernels.cu", "tn_gemm.cu"]
CPP_SOURCES = ["sv_program.cpp", "capi.cpp", "sv_jit.cpp", "server.cpp", "tn_plan.cpp", "tn_capi.cpp"]
# headers compiled again at run time by NVRTC for the per-circuit kernels
JIT_HEADERS = ["sv_plan.h", "sv_device.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def write_jit_headers():
    """Embed the device headers as C string literals (_build/jit_headers.inc)."""
    names, srcs = [], []
    for h in JIT_HEADERS:
        with open(os.path.join(HERE, h)) as f:
            text = f.read()
        assert ')tedqjit"' not in text
        names.append('"%s"' % h)
        srcs.append('R"tedqjit(' + text + ')tedqjit"')
    out = ("static const char* const kJitHeaderNames[%d] = {%s};\n" % (len(names), ", ".join(names)) +
           "static const char* const kJitHeaderSrc[%d] = {\n%s};\n" % (len(srcs), ",\n".join(srcs)))
    path = os.path.join(BUILD, "jit_headers.inc")
    old = open(path).read() if os.path.exists(path) else None
    if old != out:
        with open(path, "w") as f:
            f.write(out)


def build(jobs=4, verbose=False, ptxas_verbose=False):
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    write_jit_headers()
    common_inc = ["-I", INCLUDE, "-I", HERE, "-I", BUILD]
    cmds, objs = [], []
    for src in CU_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        flags = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
        if ptxas_verbose:
            flags += ["-Xptxas", "-v"]
        cmds.append([nvcc] + ARCH + flags + common_inc + ["-c", os.path.join(HERE, src), "-o", obj])
        objs.append(obj)
    for src in CPP_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"] + common_inc +
                     ["-I", os.path.join(cuda, "include"), "-c", os.path.join(HERE, src), "-o", obj])
        objs.append(obj)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        outs = list(ex.map(lambda c: run(c, verbose), cmds))
    if ptxas_verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = OUT + ".tmp"
    run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static", "-lrt", "-ldl", "-lpthread"], verbose)
    os.replace(tmp, OUT)
    return OUT


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=4)
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas", action="store_true", help="print register/spill usage (-Xptxas -v)")
    a = ap.parse_args()
    print(build(a.jobs, a.verbose, a.ptxas))


if __name__ == "__main__":
    sys.exit(main())
