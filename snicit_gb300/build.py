"""In-tree build of the CUDA library and the SDGC command-line driver.

Every CUDA translation unit is compiled for sm_103a only
(`-gencode arch=compute_103a,code=sm_103a`) into snicit_gb300/_build/, then
linked into snicit_gb300/libsnicit_gb300.so (the C ABI of
include/snicit_gb300.h) and snicit_gb300/_build/SDGC (the CLI).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsnicit_gb300.so")
CLI_BIN = os.path.join(BUILD, "SDGC")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
          "-ffp-contract=off", "-I", INC, "-I", CSRC]

SOURCES = [
    "layer_q1024.cu", "layer_q4096.cu", "layer_q16384.cu", "layer_generic.cu",
    "layer_dispatch.cu", "layer0_bits.cu", "post_chain.cu", "post_grid.cu", "aux.cu", "engine.cpp", "wpack.cpp", "packfile.cpp", "inputs_bin.cpp", "tsv.cpp", "gen.cpp",
    "autotune.cpp", "serve.cpp", "dedup.cu", "gen_device.cu", "selftest.cu", "noalloc.cu", "residue_sparse.cu",
]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(INC, "snicit_gb300.h")]
    for f in os.listdir(CSRC):
        if f.endswith((".h", ".cuh")):
            hs.append(os.path.join(CSRC, f))
    return hs


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(nvcc, src, obj, verbose):
    cmd = [nvcc, *COMMON, *ARCH]
    if src.endswith(".cpp"):
        cmd += ["-x", "cu"]
    cmd += ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, jobs: int = 0) -> str:
    """Compiles what changed and links the library and the CLI; returns the .so path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    objs, todo = [], []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, os.path.splitext(s)[0] + ".o")
        objs.append(obj)
        if _stale(obj, [src, *headers, __file__]):
            todo.append((src, obj))
    jobs = jobs or min(len(todo) or 1, max(2, os.cpu_count() or 2))
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            futs = [ex.submit(_compile, nvcc, s, o, verbose) for s, o in todo]
            for f in futs:
                f.result()
    if todo or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    cli_src = os.path.join(CLI, "sdgc_main.cpp")
    if os.path.exists(cli_src) and (_stale(CLI_BIN, [cli_src, LIB, *headers])):
        cmd = [nvcc, *COMMON, "-x", "cu", cli_src, "-o", CLI_BIN, *ARCH, "-L", PKG,
               "-lsnicit_gb300", "-Xlinker", "-rpath=$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
