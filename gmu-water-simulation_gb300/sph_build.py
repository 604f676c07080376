"""Builds libsph_gb300.so (sm_103a kernels + C ABI) in-tree.

    python gmu-water-simulation_gb300/sph_build.py [--force] [--verbose]

Translation units compile in parallel: the CUDA kernels with nvcc for sm_103a only,
the host C++ with g++. Host code is compiled without floating-point contraction so
that scene coordinates are identical on x86-64 and aarch64.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsph_gb300.so")
# the same library with device bounds checks and guarded allocations (SPH_CHECKED), for tests
LIB_CHECKED = os.path.join(OUT_DIR, "libsph_gb300_checked.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    hdr = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hdr.append(os.path.join(INCLUDE, "sph_cuda.h"))
    return cu, cpp, hdr


def _compile(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _jobs(cuda, checked, ptxas_verbose):
    """(compile command, object) of every translation unit of one library."""
    nvcc = os.path.join(cuda, "bin", "nvcc")
    cu, cpp, _ = sources()
    tag = ".checked" if checked else ""
    defs = ["-DSPH_CHECKED"] if checked else []
    jobs = []
    for f in cu:
        obj = os.path.join(OBJ_DIR, f + tag + ".o")
        cmd = [nvcc, "-c", os.path.join(CSRC, f), "-o", obj, "-O3", "-std=c++17", "-lineinfo", *ARCH, *defs,
               "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]
        if ptxas_verbose:
            cmd += ["-Xptxas", "-v"]
        jobs.append((cmd, obj))
    for f in cpp:
        obj = os.path.join(OBJ_DIR, f + tag + ".o")
        cmd = ["g++", "-c", os.path.join(CSRC, f), "-o", obj, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
               "-Wall", "-Wextra", "-Wno-unused-parameter", *defs, "-I", os.path.join(cuda, "include"), "-I", INCLUDE,
               "-I", CSRC]
        jobs.append((cmd, obj))
    return jobs


def build(force=False, verbose=False, ptxas_verbose=False, checked=None):
    """Compile and link; returns the library path. checked=None builds both libraries (the
    checked one for the tests), True or False one of them. Skips work when up to date."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    cu, cpp, hdr = sources()
    srcs = [os.path.join(CSRC, f) for f in cu + cpp]
    newest = max(os.path.getmtime(p) for p in srcs + hdr + [os.path.abspath(__file__)])
    wanted = [False, True] if checked is None else [bool(checked)]
    libs = {False: LIB, True: LIB_CHECKED}
    todo = [k for k in wanted if force or not os.path.exists(libs[k]) or os.path.getmtime(libs[k]) < newest]
    if todo:
        os.makedirs(OUT_DIR, exist_ok=True)
        os.makedirs(OBJ_DIR, exist_ok=True)
        per = {k: _jobs(cuda, k, ptxas_verbose) for k in todo}
        logs = []
        allj = [j for k in todo for j in per[k]]
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(allj)) as ex:
            futs = [ex.submit(_compile, cmd, verbose) for cmd, _ in allj]
            for fu in futs:
                logs.append(fu.result())
        for k in todo:
            tmp = libs[k] + ".tmp"
            link = [nvcc, "-shared", *ARCH, "-o", tmp] + [o for _, o in per[k]] + ["-lcudart_static", "-lrt", "-ldl",
                                                                                   "-lpthread"]
            logs.append(_compile(link, verbose))
            os.replace(tmp, libs[k])
        if ptxas_verbose:
            print("\n".join(l for l in logs if l.strip()))
    return libs[False] if False in wanted else libs[True]


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose="--verbose" in sys.argv,
                 ptxas_verbose="--ptxas" in sys.argv, checked=False if "--ptxas" in sys.argv else None)
    print(path)
