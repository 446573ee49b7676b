/*
 * mcx_kernel_batch.cu -- the batch instantiations of the transport kernel
 * (fast math, as mcx_kernel_fast.cu).  A separate translation unit so that
 * its constant bank holds the descriptors of a whole wave of simulations:
 * every thread reads the parameter block of the simulation it is running
 * from constant memory, as the single-simulation kernel does.
 */
#define MCXG_BATCH_TU
#include "mcx_kernel.cuh"
#include "mcx_launch.h"

namespace mcxg {

static_assert(kBatchWave == MCXG_BATCH_WAVE, "wave size of the batch unit");
static_assert(sizeof(c_sims) + sizeof(c_p) + 1024 <= 65536, "a wave of descriptors fits the constant bank");

cudaError_t batch_wave_upload(const mcxg_simdesc* d_descs, unsigned int n, cudaStream_t st) {
    if (n > MCXG_BATCH_WAVE) {
        return cudaErrorInvalidValue;
    }
    return cudaMemcpyToSymbolAsync(c_sims, d_descs, sizeof(mcxg_simdesc) * n, 0, cudaMemcpyDeviceToDevice, st);
}

/* COMMON: every simulation of the batch is 3-D (batches already take only
   label volumes and the Henyey-Greenstein phase function) */
template <bool REFL, bool WAGG, bool COMMON>
static void* kbatch(bool capped) {
    return capped ? (void*)mcx_transport<false, false, REFL, WAGG, false, 4, true, false, COMMON>
           : (void*)mcx_transport<false, false, REFL, WAGG, false, 2, true, false, COMMON>;
}

template <bool COMMON>
static void* kshape(bool refl, bool wagg, bool cap) {
    if (wagg) {
        return refl ? kbatch<true, true, COMMON>(cap) : kbatch<false, true, COMMON>(cap);
    }
    return refl ? kbatch<true, false, COMMON>(cap) : kbatch<false, false, COMMON>(cap);
}

/* the precision check of a batch: every deposit also to the FP64, plain
   float and spill fields; 3 blocks/SM, direct deposits */
template <bool REFL, bool COMMON>
static void* kbatch_acc64() {
    return (void*)mcx_transport<false, false, REFL, false, false, 3, true, false, COMMON, false, false, false, true>;
}

static void* select(int flags) {
    const bool refl = flags & LF_REFL, wagg = flags & LF_WAGG, cap = flags & LF_CAPPED;
    if (flags & LF_ACC64) {
        return (flags & LF_COMMON) ? (refl ? kbatch_acc64<true, true>() : kbatch_acc64<false, true>())
                                   : (refl ? kbatch_acc64<true, false>() : kbatch_acc64<false, false>());
    }
    return (flags & LF_COMMON) ? kshape<true>(refl, wagg, cap) : kshape<false>(refl, wagg, cap);
}

cudaError_t batch_launch(const KArgs& a, int flags, int grid, int block, size_t smem, cudaStream_t st) {
    void* args[] = {(void*)&a};
    return cudaLaunchKernel(select(flags), dim3(grid), dim3(block), args, smem, st);
}

cudaError_t batch_occupancy(int flags, int block, size_t smem, int* blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, select(flags), block, smem);
}

}  // namespace mcxg
