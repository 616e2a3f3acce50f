"""Regenerates the fixtures in this folder (run where the reference
checkout is available; the results are committed).

* sphere.obj, test.obj, cube.obj       -- meshes shipped with the reference
* sphere171Hz_CHIEF, sphere171Hz_NoCHIEF -- the reference's golden outputs
  (pulsating sphere, 171.5 Hz; wrtCplxMat format)
* chief_candidates.txt -- the uniform triples cuRAND's default host
  generator (XORWOW) returns after curandSetPseudoRandomGeneratorSeed(seed)
  for seeds 0..255, i.e. the candidate sequence of mesh::genCHIEF
  (mesh.cu:1441-1456).

Usage: python tests/golden/make_golden.py [reference_dir]
"""
import ctypes
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BEM_REFERENCE_DIR", "")
    if not ref:
        sys.exit("name the reference checkout: make_golden.py <dir> or BEM_REFERENCE_DIR=<dir>")
    for f in ["sphere.obj", "test.obj", "cube.obj", "sphere171Hz_CHIEF", "sphere171Hz_NoCHIEF"]:
        shutil.copyfile(os.path.join(ref, f), os.path.join(HERE, f))
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cr = ctypes.CDLL(os.path.join(cuda, "lib64", "libcurand.so"))
    gen = ctypes.c_void_p()
    assert cr.curandCreateGeneratorHost(ctypes.byref(gen), 100) == 0   # CURAND_RNG_PSEUDO_DEFAULT
    with open(os.path.join(HERE, "chief_candidates.txt"), "w") as f:
        f.write("# seed u0 u1 u2 : curandSetPseudoRandomGeneratorSeed(seed); curandGenerateUniform(3)\n")
        for seed in range(256):
            assert cr.curandSetPseudoRandomGeneratorSeed(gen, ctypes.c_ulonglong(seed)) == 0
            buf = (ctypes.c_float * 3)()
            assert cr.curandGenerateUniform(gen, buf, ctypes.c_size_t(3)) == 0
            f.write(f"{seed} {buf[0]:.9g} {buf[1]:.9g} {buf[2]:.9g}\n")
    cr.curandDestroyGenerator(gen)


if __name__ == "__main__":
    main()
