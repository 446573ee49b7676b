/*
 * mcx_kernel_exact.cu -- the verification instantiation of the transport
 * kernel: IEEE basic operations only (mcx_pmath.cuh), no contraction, event
 * counters on.  Compiled with -fmad=false -prec-div=true -prec-sqrt=true
 * -ftz=false so that a photon's path is the same bits as in the CPU oracle.
 */
#include "mcx_kernel.cuh"
#include "mcx_launch.h"

namespace mcxg {

cudaError_t exact_upload(const mcxg_kparams* p, const float* det4, unsigned int ndet, const float* srcx16,
                         unsigned int nsrcx, cudaStream_t st) {
    cudaError_t e = cudaMemcpyToSymbolAsync(c_p, p, sizeof(*p), 0, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && ndet) {
        e = cudaMemcpyToSymbolAsync(c_det, det4, sizeof(float) * 4 * ndet, 0, cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess && nsrcx) {
        e = cudaMemcpyToSymbolAsync(c_srcx, srcx16, sizeof(float) * 16 * nsrcx, 0, cudaMemcpyHostToDevice, st);
    }
    return e;
}

cudaError_t exact_launch(const KArgs& a, int flags, int grid, int block, size_t smem, cudaStream_t st) {
    (void)flags;
    void* f = (void*)mcx_transport<true, true, true, false, true, 2, false, true, false, true, true, true>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) {
            return e;
        }
    }
    void* args[] = {(void*)&a};
    return cudaLaunchKernel(f, dim3(grid), dim3(block), args, smem, st);
}

cudaError_t exact_rngdump(const KArgs& a, int grid, int block, cudaStream_t st) {
    void* args[] = {(void*)&a};
    return cudaLaunchKernel((void*)mcx_rng_dump, dim3(grid), dim3(block), args, 0, st);
}

}  // namespace mcxg
