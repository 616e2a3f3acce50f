"""Build recipe for libbem_gb300.so: nvcc for sm_103a, objects compiled in
parallel into _build/, linked against cuBLAS, cuSOLVER and cuRAND."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbem_gb300.so")

SOURCES = ["kernels.cu", "linalg.cu", "block.cu", "block_simt.cu", "tc_gemm.cu", "qr_tc.cu", "chief.cu", "noalloc.cu", "hmat_gpu.cu", "mesh.cpp", "mesh_io.cpp", "generators.cpp", "hmat.cpp",
           "solver.cpp", "solve.cpp", "server.cpp", "capi.cpp"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _cuda_lib_dir() -> str:
    return os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")


def _compile(src: str) -> tuple[str, str]:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    cmd = [_nvcc(), *GENCODE, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
           "-Xptxas", "-v", "-I", CSRC, "-c", path, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    with open(os.path.join(BUILD, src + ".ptxas.log"), "w") as f:
        f.write(res.stderr)
    return obj, res.stderr


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "bem_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, jobs: int | None = None) -> str:
    """Compile every source for sm_103a and link libbem_gb300.so (in-tree)."""
    if not force and not _stale():
        if not os.path.exists(DRIVER):
            _build_driver()
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = [o for o, _ in ex.map(_compile, SOURCES)]
    libdir = _cuda_lib_dir()
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), *GENCODE, "-shared", "-cudart", "shared", "-o", tmp, *objs,
           "-L", libdir, "-lcublas", "-lcusolver", "-lcurand",
           "-Xlinker", f"-rpath,{libdir}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    _build_driver()
    return LIB


DRIVER = os.path.join(HERE, "bem_sphere_driver")


def _build_driver() -> None:
    """The C++ program that runs the reference driver's call sequence through
    include/bem_gb300.hpp (host-only C++, linked to libbem_gb300.so)."""
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    cmd = ["g++", "-std=c++17", "-O2", "-I", cuda_inc, os.path.join(HERE, "cpp", "sphere_driver.cpp"),
           "-o", DRIVER, "-L", HERE, "-lbem_gb300", "-Wl,-rpath,$ORIGIN"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{res.stdout}\n{res.stderr}")


if __name__ == "__main__":
    print(build(force=True))
