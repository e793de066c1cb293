"""In-tree build of libgtc.so: nvcc for sm_103a, objects compiled in parallel.

No cmake: each translation unit is one nvcc (or g++) command, then one link.
Objects go to glsl-tree-construction_gb300/_build/, the library to
glsl-tree-construction_gb300/lib/libgtc.so (both git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(REPO_ROOT, "include")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libgtc.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgtc.so")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _cu_cmd(src: str, obj: str, ptxas_verbose: bool) -> list[str]:
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
    if ptxas_verbose:
        cmd += ["-Xptxas", "-v"]
    return cmd


def _cpp_cmd(src: str, obj: str) -> list[str]:
    cxx = os.environ.get("CXX", "g++")
    return [cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden", "-I", INCLUDE,
            "-I", os.path.join(_cuda_home(), "include"), "-c", src, "-o", obj]


def _stale(src: str, obj: str, headers: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or any(os.path.getmtime(h) > t for h in headers)


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False, jobs: int | None = None) -> str:
    """Compile every CUDA/C++ source under csrc/ and link libgtc.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    jobs_list = []
    objs = []
    for src in srcs:
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or ptxas_verbose or _stale(src, obj, headers):
            cmd = _cu_cmd(src, obj, ptxas_verbose) if src.endswith(".cu") else _cpp_cmd(src, obj)
            jobs_list.append((src, cmd))

    def run(item):
        src, cmd = item
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, cmd, r

    errors = []
    logs = []
    if jobs_list:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(jobs_list), os.cpu_count() or 4)) as ex:
            for src, cmd, r in ex.map(run, jobs_list):
                if r.returncode != 0:
                    errors.append(f"$ {' '.join(cmd)}\n{r.stdout}{r.stderr}")
                elif verbose or ptxas_verbose:
                    logs.append(f"[{os.path.basename(src)}]\n{r.stdout}{r.stderr}")
    if errors:
        raise RuntimeError("libgtc build failed:\n" + "\n".join(errors))
    if logs:
        print("\n".join(logs))
    if jobs_list or not os.path.exists(LIB_PATH):
        link = [_nvcc(), *ARCH, "-shared", "-o", LIB_PATH, *objs, "-cudart", "static", "-Xcompiler", "-fPIC"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("libgtc link failed:\n" + " ".join(link) + "\n" + r.stdout + r.stderr)
    return LIB_PATH


if __name__ == "__main__":
    import sys

    print(build(verbose=True, force="--force" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))
