/* One translation unit over the reference's device sources, as they lie in
 * the reference checkout (include path set by oracle/ref_build.py), compiled
 * with -cubin: only the device code (the assembly kernels and the element
 * integrals they call) is produced.  Nothing of the reference is copied. */
#include "numerical.cu"
#include "mesh.cu"
#include "atomicFuncs.cu"
