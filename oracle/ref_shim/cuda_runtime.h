/*
 * Host stand-in for <cuda_runtime.h>, used only by oracle/ref_harness.cpp to compile the
 * reference's kernel file (gpuFunctions_undir.cuh) as plain C++ and run every kernel one
 * thread at a time.  Test infrastructure; never part of the product.
 */
#ifndef DSSSP_REF_SHIM_CUDA_RUNTIME_H
#define DSSSP_REF_SHIM_CUDA_RUNTIME_H
#define __global__
#define __device__
#define __host__
struct ref_dim3 {
    unsigned x, y, z;
};
extern ref_dim3 threadIdx, blockIdx, blockDim, gridDim;
/* kernels run one thread at a time, so the atomic is a plain read-modify-write */
inline int atomicAdd(int* p, int v) {
    int old = *p;
    *p = old + v;
    return old;
}
typedef int cudaError_t;
#endif
