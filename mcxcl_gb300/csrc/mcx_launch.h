/*
 * mcx_launch.h -- internal interface between the session code (mcx_device.cu)
 * and the two kernel translation units.  Each unit owns its own copy of the
 * constant block, so each exports its own upload and launch entry.
 */
#ifndef MCX_LAUNCH_H
#define MCX_LAUNCH_H

#include <cuda_runtime.h>

#include "mcx_kparams.h"

namespace mcxg {

/* device pointers handed to the transport kernel */
struct KArgs {
    const uint8_t* media8;
    const uint32_t* media32;
    const float4* gprop;
    const float* invcdf;
    const float* angleinvcdf;
    const float* srcpattern;
    const uint4* seeds;            /* 4 x 32-bit seed words per reference thread */
    float* field;                  /* the field buffer: fixed-point planes (comps x fieldlen int64), then
                                      remainder planes (comps x fieldlen float); raw float scratch for
                                      the fluence-gradient passes */
    unsigned long long* fhi;       /* fixed-point counts of component c at fhi + c x plane length */
    float* flo;                    /* float remainders of component c at flo + c x plane length */
    float2* energy;                /* per reference thread: escaped, launched weight */
    float* detp;                   /* maxdetphoton x reclen */
    unsigned long long* detseed;   /* maxdetphoton x 2 */
    float2* detw;                  /* maxdetphoton x {weight, time of flight} when detected, or null */
    unsigned int* detcount;
    unsigned int* vtcounter;       /* work queue head */
    unsigned int* status;
    unsigned long long* counters;  /* step, scatter, launch, reflect, failed */
    /* replay: per photon, the saved RNG state, detected weight, time of flight, detector id */
    const ulonglong2* rseed;
    const float* rweight;
    const float* rtof;
    const int* rdetid;
    /* batch wave: per-simulation reference-thread counters (nsim, zeroed),
       the number of simulations in the wave, the batch's field length */
    unsigned int* simctr;
    unsigned int nsim;
    unsigned int lo;
    /* polarised transport: Mueller elements {S11, S12, S33, S34} at 181 polar
       angles per scattering medium (maxpol media, labels 1..maxpol), and the
       Stokes vector every photon starts with */
    const float4* smatrix;
    float4 s0;
    unsigned int maxpol;
    /* trajectory capture (-D M): record counter, records of 6 floats, capacity
       (0: off; only the general single-simulation instantiations record) */
    unsigned int* jumpctr;
    float* traj;
    unsigned int maxjump;
    /* precision check (instantiations with ACC64 only): every deposit also goes
       to an FP64 field, a plain float field and a float field with the
       reference's +-1000 spill into a second plane (2 x fieldlen) */
    double* acc64;
    float* accf;
    float* accs;
    /* fluence gradient (instantiations with ADJ only): dLoss/d(raw field) per
       field element, the per-photon loss totals J (nthread x (threadphoton +
       1)), and the pass: 1 computes J, 2 accumulates d/dmua into field plane
       0 and d/dmus into plane 1 (nvox each, voxel units) */
    const float* adjc;
    float* adjJ;
    unsigned int adjmode;
    /* hot-voxel tile (instantiations with TILE only): the field elements of
       the box [x0, x0 + nx) x [y0, y0 + ny) x [z0, z0 + nz) in gates [0, ng)
       accumulate in each block's shared memory, from byte smemoff of the
       dynamic shared memory, and go to the field when the block ends.  A voxel
       index i is tested as: (i - lo) < span (the box's z planes), then
       z = umulhi(i, mxy) >> sxy, and y = umulhi(i - z dimxy, mx) >> sx --
       divisions by dimxy and dimx that the host checked exact for every index
       of the volume */
    struct Tile {
        int x0, y0, z0;
        unsigned int nx, ny, nz, ng;
        unsigned int lo, span;
        unsigned int mx, mxy, sx, sxy;
        unsigned int smemoff;
    } tile;
};

/* flag bits for the launch entries */
enum { LF_DET = 1, LF_REFL = 2, LF_WAGG = 4, LF_CAPPED = 8, LF_XMEDIA = 32, LF_COMMON = 64, LF_RF = 128, LF_POL = 256, LF_SVMC = 512,
       LF_ACC64 = 1024, LF_ADJ = 2048, LF_TILE = 4096 };

/* fast instantiation: hardware transcendental approximations */
cudaError_t fast_upload(const mcxg_kparams* p, const float* det4, unsigned int ndet, const float* srcx16,
                        unsigned int nsrcx, cudaStream_t st);
cudaError_t fast_launch(const KArgs& a, int flags, int grid, int block, size_t smem, cudaStream_t st);
cudaError_t fast_occupancy(int flags, int block, size_t smem, int* blocks_per_sm);
cudaError_t fast_attributes(int flags, cudaFuncAttributes* attr);

/* exact instantiation: IEEE basic operations only, bit-identical to the oracle */
cudaError_t exact_upload(const mcxg_kparams* p, const float* det4, unsigned int ndet, const float* srcx16,
                         unsigned int nsrcx, cudaStream_t st);
cudaError_t exact_launch(const KArgs& a, int flags, int grid, int block, size_t smem, cudaStream_t st);
cudaError_t exact_rngdump(const KArgs& a, int grid, int block, cudaStream_t st);

/* batch instantiations: simulation descriptors of one wave into constant
   memory (from device memory), then the launch */
constexpr int kBatchWave = 136;
cudaError_t batch_wave_upload(const mcxg_simdesc* d_descs, unsigned int n, cudaStream_t st);
cudaError_t batch_launch(const KArgs& a, int flags, int grid, int block, size_t smem, cudaStream_t st);
cudaError_t batch_occupancy(int flags, int block, size_t smem, int* blocks_per_sm);
}  // namespace mcxg

#endif
