/*
 * mcx_kernel_fast.cu -- the production instantiations of the transport
 * kernel: MUFU transcendentals (__logf, __expf, __sincosf, rsqrtf,
 * __fdividef).  Compiled with --use_fast_math.
 */
#include "mcx_kernel.cuh"
#include "mcx_launch.h"

namespace mcxg {

cudaError_t fast_upload(const mcxg_kparams* p, const float* det4, unsigned int ndet, const float* srcx16,
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

/* the register-capped instantiation (64 registers: 1,024 resident threads a
   SM) or the uncapped one (for shapes of at most 512 threads a SM) */
template <bool DET, bool REFL, bool WAGG, bool COMMON>
static void* kfun(bool capped) {
    return capped ? (void*)mcx_transport<false, DET, REFL, WAGG, false, 4, false, false, COMMON>
           : (void*)mcx_transport<false, DET, REFL, WAGG, false, 2, false, false, COMMON>;
}

template <bool COMMON>
static void* kshape(bool det, bool refl, bool wagg, bool cap) {
    if (wagg) {
        if (det) {
            return refl ? kfun<true, true, true, COMMON>(cap) : kfun<true, false, true, COMMON>(cap);
        }
        return refl ? kfun<false, true, true, COMMON>(cap) : kfun<false, false, true, COMMON>(cap);
    }
    if (det) {
        return refl ? kfun<true, true, false, COMMON>(cap) : kfun<true, false, false, COMMON>(cap);
    }
    return refl ? kfun<false, true, false, COMMON>(cap) : kfun<false, false, false, COMMON>(cap);
}

/* the RF (frequency-domain) transport: complex photon weights, 80-register
   cap (3 blocks of 256 a SM; at 64 it ran 1 % slower), direct deposits */
template <bool DET, bool REFL>
static void* krf() {
    return (void*)mcx_transport<false, DET, REFL, false, false, 3, false, false, false, true>;
}

/* the polarised transport: Stokes vectors and Mueller tables, 80-register
   cap, direct deposits */
template <bool DET, bool REFL>
static void* kpol() {
    return (void*)mcx_transport<false, DET, REFL, false, false, 3, false, false, false, false, true>;
}

/* split-voxel volumes: 80-register cap (3 blocks of 256 a SM: at 64 they
   spill), direct deposits */
template <bool DET, bool REFL>
static void* ksvmc() {
    return (void*)mcx_transport<false, DET, REFL, false, false, 3, false, false, false, false, false, true>;
}

/* volumes in the less common encodings: 80-register cap, direct deposits */
template <bool DET, bool REFL>
static void* kxmedia() {
    return (void*)mcx_transport<false, DET, REFL, false, false, 3, false, true>;
}

/* the common configuration with the FP64 / plain-float / spill accumulators
   of the precision check: 80-register cap, direct deposits */
template <bool DET, bool REFL>
static void* kacc64() {
    return (void*)mcx_transport<false, DET, REFL, false, false, 3, false, false, true, false, false, false, true>;
}

/* the fluence-gradient passes: general media handling (labels or float mua),
   no detectors, 64-register cap (4 blocks of 256 a SM: the two passes ran
   5 % faster than at 80) */
template <bool REFL>
static void* kadj() {
    return (void*)mcx_transport<false, false, REFL, false, false, 4, false, false, false, false, false, false, false,
                                true>;
}

/* the common configuration with the hot-voxel tile in shared memory:
   80-register cap, direct deposits */
template <bool DET, bool REFL>
static void* ktile() {
    return (void*)mcx_transport<false, DET, REFL, false, false, 3, false, false, true, false, false, false, false,
                                false, true>;
}

static void* select(int flags) {
    const bool det = flags & LF_DET, refl = flags & LF_REFL, wagg = flags & LF_WAGG, cap = flags & LF_CAPPED;
    if (flags & LF_TILE) {
        return det ? (refl ? ktile<true, true>() : ktile<true, false>())
                   : (refl ? ktile<false, true>() : ktile<false, false>());
    }
    if (flags & LF_ADJ) {
        return refl ? kadj<true>() : kadj<false>();
    }
    if (flags & LF_ACC64) {
        return det ? (refl ? kacc64<true, true>() : kacc64<true, false>())
                   : (refl ? kacc64<false, true>() : kacc64<false, false>());
    }
    if (flags & LF_SVMC) {
        return det ? (refl ? ksvmc<true, true>() : ksvmc<true, false>())
                   : (refl ? ksvmc<false, true>() : ksvmc<false, false>());
    }
    if (flags & LF_POL) {
        return det ? (refl ? kpol<true, true>() : kpol<true, false>()) : (refl ? kpol<false, true>() : kpol<false, false>());
    }
    if (flags & LF_RF) {
        return det ? (refl ? krf<true, true>() : krf<true, false>()) : (refl ? krf<false, true>() : krf<false, false>());
    }
    if (flags & LF_XMEDIA) {
        return det ? (refl ? kxmedia<true, true>() : kxmedia<true, false>())
                   : (refl ? kxmedia<false, true>() : kxmedia<false, false>());
    }
    return (flags & LF_COMMON) ? kshape<true>(det, refl, wagg, cap) : kshape<false>(det, refl, wagg, cap);
}

cudaError_t fast_launch(const KArgs& a, int flags, int grid, int block, size_t smem, cudaStream_t st) {
    void* f = select(flags);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) {
            return e;
        }
    }
    void* args[] = {(void*)&a};
    return cudaLaunchKernel(f, dim3(grid), dim3(block), args, smem, st);
}

cudaError_t fast_occupancy(int flags, int block, size_t smem, int* blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, select(flags), block, smem);
}

cudaError_t fast_attributes(int flags, cudaFuncAttributes* attr) {
    return cudaFuncGetAttributes(attr, select(flags));
}

}  // namespace mcxg
