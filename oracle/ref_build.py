"""Builds the reference-kernel checker under oracle/_ref/ (test and benchmark
infrastructure).

* ref_kernels.cubin -- the reference's own device code, compiled for sm_103a
  from its sources where they lie (oracle/ref_unity.cu includes numerical.cu,
  mesh.cu and atomicFuncs.cu from the reference checkout) with the flags of its
  Makefile (-O3 -use_fast_math).  Only where the checkout exists; the cubin is
  device code, so a copy built on one machine runs on any GB300 host.  GSL,
  which numerical.cu's host code calls, is not installed: oracle/ref_shim
  holds declarations only, and no host code of the reference is compiled.
* libref_harness.so -- oracle/ref_harness.cpp (the launcher), built wherever
  the CUDA toolkit is.
* meshes/ -- the reference's own head and torso meshes (Head_20kHz_iso.obj,
  Head_20kHz_iso.ply, KEMARTORSO_12000Hz.obj), staged beside the cubin so
  that the GPU tests of realistic workloads can read them where the reference
  checkout is absent.  They are the reference's data: never committed.

The reference checkout is named by the environment variable BEM_REFERENCE_DIR;
without it nothing is taken from the reference and what oracle/_ref already
holds is used.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT, "ref_kernels.cubin")
HARNESS = os.path.join(OUT, "libref_harness.so")
REF_DIR = os.environ.get("BEM_REFERENCE_DIR", "")
MESH_DIR = os.path.join(OUT, "meshes")
MESHES = ("Head_20kHz_iso.obj", "Head_20kHz_iso.ply", "KEMARTORSO_12000Hz.obj")


def _cuda() -> str:
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build_cubin(force: bool = False) -> bool:
    """Compile the reference kernels when the reference sources are present."""
    srcs = [os.path.join(REF_DIR, f) for f in ("numerical.cu", "mesh.cu", "atomicFuncs.cu")]
    if not REF_DIR or not all(os.path.exists(s) for s in srcs):
        return os.path.exists(CUBIN)
    if not force and os.path.exists(CUBIN) and all(os.path.getmtime(CUBIN) > os.path.getmtime(s) for s in srcs):
        return True
    os.makedirs(OUT, exist_ok=True)
    nvcc = os.path.join(_cuda(), "bin", "nvcc")
    nvcc = nvcc if os.path.exists(nvcc) else (shutil.which("nvcc") or "nvcc")
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-use_fast_math",
           "-w", "-I", os.path.join(HERE, "ref_shim"), "-I", REF_DIR,
           os.path.join(HERE, "ref_unity.cu"), "-o", CUBIN]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference cubin build failed:\n{res.stderr[-4000:]}")
    return True


def build_harness(force: bool = False) -> str:
    src = os.path.join(HERE, "ref_harness.cpp")
    if not force and os.path.exists(HARNESS) and os.path.getmtime(HARNESS) > os.path.getmtime(src):
        return HARNESS
    os.makedirs(OUT, exist_ok=True)
    cuda = _cuda()
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", src, "-o", HARNESS,
           "-I", os.path.join(cuda, "include"), "-L", os.path.join(cuda, "lib64"),
           "-L", os.path.join(cuda, "lib64", "stubs"), "-lcuda", "-lcudart", "-lcusolver", "-lcublas",
           f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference harness build failed:\n{res.stderr[-4000:]}")
    return HARNESS


def stage_meshes() -> list:
    """Copies the reference's head and torso meshes into oracle/_ref/meshes
    when the checkout is named; returns the staged paths that exist."""
    if REF_DIR:
        os.makedirs(MESH_DIR, exist_ok=True)
        for f in MESHES:
            src, dst = os.path.join(REF_DIR, f), os.path.join(MESH_DIR, f)
            if os.path.exists(src) and not (os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(src)):
                shutil.copyfile(src, dst)
    return [os.path.join(MESH_DIR, f) for f in MESHES if os.path.exists(os.path.join(MESH_DIR, f))]


def build_if_possible() -> bool:
    """Harness always; cubin and staged meshes when the reference checkout is
    named.  True when cubin and harness exist afterwards."""
    have_cubin = build_cubin()
    stage_meshes()
    build_harness()
    return have_cubin and os.path.exists(HARNESS)


if __name__ == "__main__":
    print(build_if_possible())
