/*
 * mcx_device.cu -- the thin device layer (mcxg_* in include/mcx_gb300.h).
 *
 * Replaces the OpenCL buffer creation, launch and readback of the reference's
 * mcx_run_simulation (src/mcx_host.cpp:739-1345).  A session owns one CUDA
 * stream and the device buffers of one problem; buffers grow on demand and
 * are reused across calls, so repeated runs (respin, autotuning, bench
 * steps) allocate nothing after the first.
 *
 * The FP64 work of the path lives here: the per-thread escaped/launched
 * weights are summed in double on the GPU (the reference sums them in double
 * on the host, mcx_host.cpp:1303-1306) and the two-plane field is merged and
 * normalised in double before rounding to float (the reference merges and
 * scales in float, mcx_host.cpp:1252-1257, mcx_utils.c:1208-1218).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/mcx_gb300.h"
#include "mcx_kparams.h"
#include "mcx_launch.h"

using mcxg::KArgs;

struct mcxg_session {
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    mcxg_devinfo info{};
    mcxg_kparams kp{};
    bool has_problem = false;
    bool has_seeds = false;
    bool up_fast = false, up_exact = false;

    void* d_media = nullptr;
    size_t media_cap = 0;
    float4* d_prop = nullptr;
    size_t prop_cap = 0;
    float* d_tables = nullptr;       /* invcdf then angleinvcdf */
    size_t tables_cap = 0;
    float* d_pattern = nullptr;
    size_t pattern_cap = 0;
    uint4* d_seeds = nullptr;
    size_t seeds_cap = 0;
    uint32_t* d_words32 = nullptr;   /* 32-bit label words before packing (MCXG_MEDIA_PACK) */
    size_t words32_cap = 0;
    unsigned int* d_jump = nullptr;  /* trajectory capture: record counter and records */
    float* d_traj = nullptr;
    size_t traj_cap = 0, jump_cap = 0;
    uint32_t maxjump = 0;
    uint32_t* d_lfib = nullptr;      /* 31-word generator windows, one per block of seed words */
    size_t lfib_cap = 0;
    float* d_field = nullptr;        /* per component: hi, lo, spill count planes (3 x fieldlen) */
    size_t field_cap = 0;
    float2* d_energy = nullptr;
    size_t energy_cap = 0;
    float* d_detp = nullptr;
    size_t detp_cap = 0;             /* floats */
    unsigned long long* d_detseed = nullptr;
    size_t detseed_cap = 0;
    float2* d_detw = nullptr;
    size_t detw_cap = 0;
    unsigned int* d_words = nullptr; /* detcount, vtcounter, status[2] */
    unsigned long long* d_events = nullptr;
    double* d_red = nullptr;         /* reduction partials + result */
    void* d_out = nullptr;           /* merged field, float or double */
    size_t out_cap = 0;

    ulonglong2* d_rseed = nullptr;   /* replay: per photon RNG state, weight, tof, detector id */
    size_t rseed_cap = 0;
    float* d_rweight = nullptr;
    size_t rweight_cap = 0;
    float* d_rtof = nullptr;
    size_t rtof_cap = 0;
    int* d_rdetid = nullptr;
    size_t rdetid_cap = 0;
    uint32_t nreplay = 0;
    double* d_scales = nullptr;      /* per-block normalisation factors */
    size_t scales_cap = 0;
    bool out_valid = false;          /* d_out holds the last normalised float field */
    float* d_adj = nullptr;          /* adjoint Jacobians */
    size_t adj_cap = 0;
    float* d_adjc = nullptr;         /* fluence gradient: dLoss/d(raw field), fieldlen */
    size_t adjc_cap = 0;
    float* d_adjJ = nullptr;         /* per-photon loss totals, nthread x (threadphoton + 1) */
    size_t adjJ_cap = 0;
    bool adj_ready = false;
    double* d_acc64 = nullptr;       /* precision check: FP64, plain float and spill fields */
    size_t acc64_cap = 0;
    float* d_accf = nullptr;
    size_t accf_cap = 0;
    float* d_accs = nullptr;         /* 2 x fieldlen */
    size_t accs_cap = 0;

    /* batch of simulations in one persistent launch */
    std::vector<mcxg_simdesc> h_sims;
    mcxg_simdesc* d_sims = nullptr;
    size_t sims_cap = 0;
    unsigned long long* d_simvt = nullptr;
    size_t simvt_cap = 0;
    unsigned int* d_simctr = nullptr;   /* per-simulation reference-thread counters */
    float4* d_smatrix = nullptr;        /* polarised transport: Mueller rows, 181 per medium */
    size_t smatrix_cap = 0;
    uint32_t npol = 0;
    float4 pol_s0 = {1.f, 0.f, 0.f, 0.f};
    size_t simctr_cap = 0;
    uint8_t* d_bmedia = nullptr;
    size_t bmedia_cap = 0;
    std::vector<unsigned long long> h_simvt;
    float* d_bfield = nullptr;       /* int64 fixed-point counts (2 x totalfield floats), then float remainders */
    size_t bfield_cap = 0;
    float2* d_benergy = nullptr;     /* per reference thread of the batch */
    size_t benergy_cap = 0;
    double* d_bsum = nullptr;        /* per simulation: escaped, launched */
    size_t bsum_cap = 0;
    float* d_bout = nullptr;
    size_t bout_cap = 0;
    uint32_t nsim = 0;
    unsigned long long totalvt = 0, totalfield = 0;
    bool has_batch = false;
    int bt_block = 256, bt_bpsm = 4, bt_grid = 0;
    cudaGraph_t bgraph = nullptr;
    cudaGraphExec_t bgraph_exec = nullptr;

    std::vector<float> h_det, h_srcx;
    int block_req = 0, bpsm_req = 0;
    uint32_t tile_req = 0;           /* hot-voxel tile: at most this many field elements (0: off) */
    /* L2 persisting window over the field's count plane (l2_window) */
    bool l2_set = false;             /* this session raised the context's persisting limit */
    size_t l2_prev = 0;              /* the limit before */
    const void* l2_base = nullptr;   /* the window set on the stream (nullptr: none) */
    size_t l2_bytes = 0;
    mcxg::KArgs::Tile tile_used{};   /* the last launch's tile (nx = 0: none) */
    int tuned = 0;                   /* 1 once mcxg_autotune picked a shape for this problem */
    int tuned_noagg = 0;
    int grid = 0, block = 0, regs = 0;
};

namespace {

constexpr int kRedBlocks = 256;
constexpr int kRedThreads = 256;
/* the transport kernel's compensated field: an int64 fixed-point plane and a
   float remainder plane per component, 3 floats of memory per element */
constexpr size_t kFieldPlanes = 3;

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) {
        return MCXG_OK;
    }
    if (e == cudaErrorMemoryAllocation) {
        return MCXG_ERR_NOMEM;
    }
    return MCXG_ERR_CUDA;
}

#define MCXG_TRY(x)                       \
    do {                                  \
        int _rc = cuda_status((x));       \
        if (_rc) {                        \
            return _rc;                   \
        }                                 \
    } while (0)

template <typename T>
int ensure(T** ptr, size_t* cap, size_t count) {
    if (count <= *cap && *ptr) {
        return MCXG_OK;
    }
    if (*ptr) {
        cudaFree(*ptr);
        *ptr = nullptr;
        *cap = 0;
    }
    if (count == 0) {
        return MCXG_OK;
    }
    MCXG_TRY(cudaMalloc((void**)ptr, count * sizeof(T)));
    *cap = count;
    return MCXG_OK;
}

/* per-block partial FP64 sums of {escaped, launched} */
__global__ void energy_partials(const float2* __restrict__ e, unsigned int n, double* __restrict__ part) {
    double se = 0.0, sl = 0.0;
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float2 v = e[i];
        se += (double)v.x;
        sl += (double)v.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        se += __shfl_down_sync(0xffffffffu, se, o);
        sl += __shfl_down_sync(0xffffffffu, sl, o);
    }
    __shared__ double wse[32], wsl[32];
    if ((threadIdx.x & 31) == 0) {
        wse[threadIdx.x >> 5] = se;
        wsl[threadIdx.x >> 5] = sl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (unsigned int w = 0; w < (blockDim.x + 31) / 32; w++) {
            a += wse[w];
            b += wsl[w];
        }
        part[blockIdx.x * 2] = a;
        part[blockIdx.x * 2 + 1] = b;
    }
}

/* fixed-order final sum, so the result is the same bits on every run */
__global__ void energy_final(double* part, int nblocks) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int i = 0; i < nblocks; i++) {
            a += part[i * 2];
            b += part[i * 2 + 1];
        }
        part[nblocks * 2] = a;
        part[nblocks * 2 + 1] = b;
    }
}

/* Element i of a field buffer of total elements (all components): the
   fixed-point planes of all components (int64 counts of unit), then their
   float remainder planes; value = count x unit + remainder in FP64. */
__device__ __forceinline__ double cell_value(const float* __restrict__ f, size_t total, double unit, size_t i) {
    return (double)reinterpret_cast<const long long*>(f)[i] * unit + (double)f[2 * total + i];
}

/* Output element i of a field of n elements per component and total
   elements over all components: component c = i / n (1 real, or real then
   imaginary for RF), element j = i % n. */
__device__ __forceinline__ double merged_at(const float* __restrict__ f, size_t n, size_t total, double unit, size_t i,
                                            size_t& j) {
    const size_t c = i / n;
    j = i - c * n;
    return cell_value(f, total, unit, i);
}

__global__ void field_merge_f32(const float* __restrict__ f, size_t n, size_t total, double unit, double scale,
                                float* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        size_t j;
        out[i] = (float)(merged_at(f, n, total, unit, i, j) * scale);
    }
}

/* element j belongs to source j % nsrc (photon sharing interleaves the
   patterns innermost) */
__global__ void field_merge_interleaved(const float* __restrict__ f, size_t n, size_t total, double unit,
                                        unsigned int nsrc, const double* __restrict__ scales, float* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        size_t j;
        const double v = merged_at(f, n, total, unit, i, j);
        out[i] = (float)(v * scales[j % nsrc]);
    }
}

__global__ void field_merge_blocks(const float* __restrict__ f, size_t n, size_t total, double unit, size_t blocklen,
                                   const double* __restrict__ scales, float* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        size_t j;
        const double v = merged_at(f, n, total, unit, i, j);
        out[i] = (float)(v * scales[j / blocklen]);
    }
}

/* reciprocals of each simulation's property rows, as the single-simulation
   kernel stages them */
__global__ void batch_recip(mcxg_simdesc* __restrict__ sims, unsigned int nsim) {
    const unsigned int n = nsim * MCXG_BATCH_MAXMEDIA;
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        mcxg_simdesc& d = sims[i / MCXG_BATCH_MAXMEDIA];
        const mcxg_float4 q = d.prop[i % MCXG_BATCH_MAXMEDIA];
        mcxg_float4& r = d.recip[i % MCXG_BATCH_MAXMEDIA];
        r.x = __fdividef(1.f, q.y);
        r.y = __fdividef(1.f, q.y * (1.f - q.z));
        r.z = __fdividef(1.f, q.x);
        r.w = __fdividef(1.f, 2.f * q.z);
    }
}

/* per-simulation FP64 energy sums: one block per simulation, fixed order */
__global__ void batch_energy(const float2* __restrict__ e, const mcxg_simdesc* __restrict__ sims,
                             double* __restrict__ out) {
    const mcxg_simdesc& d = sims[blockIdx.x];
    const unsigned long long base = d.vt_off;
    const unsigned int n = d.kp.nthread;
    double se = 0.0, sl = 0.0;
    for (unsigned int i = threadIdx.x; i < n; i += blockDim.x) {
        float2 v = e[base + i];
        se += (double)v.x;
        sl += (double)v.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        se += __shfl_down_sync(0xffffffffu, se, o);
        sl += __shfl_down_sync(0xffffffffu, sl, o);
    }
    __shared__ double wse[32], wsl[32];
    if ((threadIdx.x & 31) == 0) {
        wse[threadIdx.x >> 5] = se;
        wsl[threadIdx.x >> 5] = sl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (unsigned int w = 0; w < (blockDim.x + 31) / 32; w++) {
            a += wse[w];
            b += wsl[w];
        }
        out[blockIdx.x * 2] = a;
        out[blockIdx.x * 2 + 1] = b;
    }
}

/* merged, scaled field of every simulation: row y of the grid is simulation y */
__global__ void batch_merge(const float* __restrict__ f, unsigned long long total, const mcxg_simdesc* __restrict__ sims,
                            const double* __restrict__ scales, float* __restrict__ out) {
    const mcxg_simdesc& d = sims[blockIdx.y];
    const unsigned long long off = d.field_off;
    const unsigned int n = d.kp.fieldlen;
    const double sc = scales[blockIdx.y];
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        out[off + i] = (float)(cell_value(f, total, (double)d.kp.fxunit, off + i) * sc);
    }
}

/* every simulation's compensated field merged in FP64, unscaled */
__global__ void batch_merge_f64(const float* __restrict__ f, unsigned long long total,
                                const mcxg_simdesc* __restrict__ sims, double* __restrict__ out) {
    const mcxg_simdesc& d = sims[blockIdx.y];
    const unsigned long long off = d.field_off;
    const unsigned int n = d.kp.fieldlen;
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        out[off + i] = cell_value(f, total, (double)d.kp.fxunit, off + i);
    }
}

/* Adjoint post-kernels (the reference's mcx_adjoint_kernel and
   mcx_adjoint_dcoeff_kernel, mcx_core.cl:3320-3512) on the normalised float
   field: per voxel, the time-integrated fluence of each source times that of
   each detector, or the dot product of their finite-difference gradients.
   Explicit _rn operations keep the reference's evaluation order (no
   contraction). */
__device__ __forceinline__ float adj_cw(const float* f, unsigned int vox, unsigned int slot, unsigned int maxgate,
                                        unsigned int nvox) {
    float sum = 0.f;
    for (unsigned int t = 0; t < maxgate; t++) {
        sum = __fadd_rn(sum, f[vox + (size_t)(t + slot * maxgate) * nvox]);
    }
    return sum;
}

__device__ __forceinline__ float adj_grad(const float* f, unsigned int vox, unsigned int slot, unsigned int maxgate,
                                          unsigned int nvox, unsigned int i, unsigned int n, unsigned int stride) {
    if (n <= 1) {
        return 0.f;
    }
    const float f0 = adj_cw(f, vox, slot, maxgate, nvox);
    if (i == 0) {
        const float fp1 = adj_cw(f, vox + stride, slot, maxgate, nvox);
        if (n == 2) {
            return __fsub_rn(fp1, f0);
        }
        const float fp2 = adj_cw(f, vox + 2 * stride, slot, maxgate, nvox);
        return __fmul_rn(__fsub_rn(__fadd_rn(__fmul_rn(-3.f, f0), __fmul_rn(4.f, fp1)), fp2), 0.5f);
    } else if (i == n - 1) {
        const float fm1 = adj_cw(f, vox - stride, slot, maxgate, nvox);
        if (n == 2) {
            return __fsub_rn(f0, fm1);
        }
        const float fm2 = adj_cw(f, vox - 2 * stride, slot, maxgate, nvox);
        return __fmul_rn(__fadd_rn(__fsub_rn(fm2, __fmul_rn(4.f, fm1)), __fmul_rn(3.f, f0)), 0.5f);
    }
    const float fp1 = adj_cw(f, vox + stride, slot, maxgate, nvox);
    const float fm1 = adj_cw(f, vox - stride, slot, maxgate, nvox);
    return __fmul_rn(__fsub_rn(fp1, fm1), 0.5f);
}

__global__ void adjoint_mua(const float* __restrict__ f, float* __restrict__ out, unsigned int nvox,
                            unsigned int maxgate, unsigned int ns, unsigned int nd) {
    for (unsigned int vox = blockIdx.x * blockDim.x + threadIdx.x; vox < nvox; vox += gridDim.x * blockDim.x) {
        for (unsigned int s = 0; s < ns; s++) {
            const float cs = adj_cw(f, vox, s, maxgate, nvox);
            for (unsigned int d = 0; d < nd; d++) {
                const float cd = adj_cw(f, vox, ns + d, maxgate, nvox);
                out[vox + (size_t)(s * nd + d) * nvox] = __fsub_rn(__fmul_rn(cs, cd), __fmul_rn(0.f, 0.f));
            }
        }
    }
}

__global__ void adjoint_dcoeff(const float* __restrict__ f, float* __restrict__ out, unsigned int nvox,
                               unsigned int maxgate, unsigned int ns, unsigned int nd, unsigned int nx,
                               unsigned int ny) {
    const unsigned int nxy = nx * ny, nz = nvox / nxy;
    for (unsigned int vox = blockIdx.x * blockDim.x + threadIdx.x; vox < nvox; vox += gridDim.x * blockDim.x) {
        const unsigned int ix = vox % nx, iy = (vox / nx) % ny, iz = vox / nxy;
        for (unsigned int s = 0; s < ns; s++) {
            const float sx = adj_grad(f, vox, s, maxgate, nvox, ix, nx, 1);
            const float sy = adj_grad(f, vox, s, maxgate, nvox, iy, ny, nx);
            const float sz = adj_grad(f, vox, s, maxgate, nvox, iz, nz, nxy);
            for (unsigned int d = 0; d < nd; d++) {
                const float dx = adj_grad(f, vox, ns + d, maxgate, nvox, ix, nx, 1);
                const float dy = adj_grad(f, vox, ns + d, maxgate, nvox, iy, ny, nx);
                const float dz = adj_grad(f, vox, ns + d, maxgate, nvox, iz, nz, nxy);
                out[vox + (size_t)(s * nd + d) * nvox] =
                    __fadd_rn(__fadd_rn(__fmul_rn(sx, dx), __fmul_rn(sy, dy)), __fmul_rn(sz, dz));
            }
        }
    }
}

__global__ void field_merge_f64(const float* __restrict__ f, size_t n, size_t total, double unit,
                                double* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        size_t j;
        out[i] = merged_at(f, n, total, unit, i, j);
    }
}

/* FP32 issue peak: 8 independent FMA chains per thread, so the FMA pipe --
   not latency -- limits; each FMA counts as one FP32 operation */
__global__ void fma_peak(float* out, int iters, float b, float c) {
    float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
    float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
    for (int i = 0; i < iters; i++) {
        a0 = fmaf(a0, b, c);
        a1 = fmaf(a1, b, c);
        a2 = fmaf(a2, b, c);
        a3 = fmaf(a3, b, c);
        a4 = fmaf(a4, b, c);
        a5 = fmaf(a5, b, c);
        a6 = fmaf(a6, b, c);
        a7 = fmaf(a7, b, c);
    }
    float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (r == 12345.678f) {
        out[0] = r;              /* never true; keeps the chains live */
    }
}

int grid_for(const mcxg_session* s, size_t n) {
    size_t g = (n + 255) / 256;
    size_t cap = (size_t)s->info.sm * 8;
    if (g > cap) {
        g = cap;
    }
    return g < 1 ? 1 : (int)g;
}

/* property rows and their reciprocals (2 x 16 B per medium), 32 B of
   launch-time state per thread, the phase tables, and the detector partial
   data per thread */
/* 2 for a complex (RF) field: the RF transport, or an rf / rfmus replay */
unsigned int field_comps(const mcxg_kparams& kp) {
    return ((kp.omega > 0.f && !kp.replay) || (kp.replay && (kp.outputtype == otRF || kp.outputtype == otRFmus))) ? 2u : 1u;
}

size_t shared_bytes(const mcxg_kparams& kp, int block) {
    /* per-thread slots: detector partial data, then one weight per shared
       pattern (their slots start after the partial data) */
    size_t det = (kp.srcnum > 1) ? (size_t)kp.partialdata + kp.srcnum : (kp.savedet ? kp.partialdata : 0);
    if (kp.replay && (kp.outputtype == otRF || kp.outputtype == otRFmus)) {
        det = (size_t)kp.partialdata + 2;    /* the launch phase's cos and sin follow the partial data */
    }
    return (size_t)kp.medianum * 32 + (size_t)block * 32 + (size_t)(kp.nphase + kp.nangle) * 4 + det * (size_t)block * 4;
}

/* q = umulhi(n, m) >> sh equals n / d for every n < bound: m = ceil(2^(32+sh) / d)
   with the largest sh that keeps m below 2^32, exact when (bound - 1) e <
   2^(32+sh), e = m d - 2^(32+sh) (the rounding error of m times d) */
bool exact_divider(uint32_t d, uint32_t bound, uint32_t* m, uint32_t* sh) {
    if (d < 2) {
        return false;
    }
    for (int k = 31; k >= 0; k--) {
        const unsigned long long p = 1ull << (32 + k);
        const unsigned long long mm = (p + d - 1) / d;
        if (mm >= (1ull << 32)) {
            continue;
        }
        const unsigned long long e = mm * d - p;
        if ((unsigned long long)(bound ? bound - 1 : 0) * e < p) {
            *m = (uint32_t)mm;
            *sh = (uint32_t)k;
            return true;
        }
        return false;
    }
    return false;
}

/* The hot-voxel tile of a single simulation: a box of voxels next to the
   source, along its direction, in the first gates.  Most deposits of a
   pencil beam fall there (the oracle's deposit counts: 17 % of the cube +
   sphere workload's in 11 x 11 x 11 voxels x 3 gates, 33 % of the head's in
   16^3 voxels x 1 gate).  Gates: enough that they span about 64 voxels of
   path at n = 1.4; the cube side is what the element budget then allows. */
bool tile_geometry(const mcxg_kparams& kp, uint32_t maxelem, mcxg::KArgs::Tile& t) {
    t = mcxg::KArgs::Tile{};
    if (maxelem < 8 || kp.maxgate < 1 || kp.Rtstep <= 0.f || kp.oneoverc0 <= 0.f) {
        return false;
    }
    const double pathvox = 1.0 / ((double)kp.Rtstep * kp.oneoverc0 * 1.4);
    uint32_t ng = (uint32_t)std::ceil(64.0 / (pathvox > 1e-3 ? pathvox : 1e-3));
    ng = std::max(1u, std::min(ng, std::min(8u, kp.maxgate)));
    int side = (int)std::floor(std::cbrt((double)maxelem / ng));
    while (side > 1 && (unsigned long long)side * side * side * ng > maxelem) {
        side--;
    }
    if (side < 2) {
        return false;
    }
    const int dims[3] = {(int)kp.dimx, (int)kp.dimy, (int)kp.dimz};
    const float c[3] = {kp.srcpos.x + kp.srcdir.x * side * 0.5f, kp.srcpos.y + kp.srcdir.y * side * 0.5f,
                        kp.srcpos.z + kp.srcdir.z * side * 0.5f};
    int n[3], o[3];
    for (int i = 0; i < 3; i++) {
        n[i] = std::min(side, dims[i]);
        float lo = std::floor(c[i] - n[i] * 0.5f);
        if (!(lo >= 0.f)) {
            lo = 0.f;
        }
        o[i] = std::min((int)lo, dims[i] - n[i]);
    }
    t.x0 = o[0];
    t.y0 = o[1];
    t.z0 = o[2];
    t.nx = (uint32_t)n[0];
    t.ny = (uint32_t)n[1];
    t.nz = (uint32_t)n[2];
    t.ng = ng;
    t.lo = (uint32_t)o[2] * kp.dimxy;
    t.span = (uint32_t)n[2] * kp.dimxy;
    if (!exact_divider(kp.dimxy, kp.nvox, &t.mxy, &t.sxy) || !exact_divider(kp.dimx, kp.dimxy, &t.mx, &t.sx)) {
        t = mcxg::KArgs::Tile{};
        return false;
    }
    return true;
}

/* Keep the fixed-point count plane of the field in L2.  The deposits of a
   single simulation hit the int64 counts and the float remainders of random
   field elements with fire-and-forget reductions; when the planes together
   approach L2's size (the cube + sphere workload's are 130 MB) the lines
   thrash and the reductions write evicted lines back to DRAM (95 GB a
   1e8-photon launch).  A persisting access-policy window on the session's
   stream over the count plane (when it fits in the largest window the
   device allows) keeps it in L2's persisting set-aside, which this
   session raises to the device's maximum for its context; the remainders
   and the streamed seeds and records share the rest.  Measured on the cube +
   sphere workload: DRAM writes 95 GB -> 33 GB a launch, same kernel time. */
void l2_window(mcxg_session* s, const mcxg_kparams& kp, bool on) {
    int maxpersist = 0, maxwin = 0;
    if (cudaDeviceGetAttribute(&maxpersist, cudaDevAttrMaxPersistingL2CacheSize, s->device) != cudaSuccess ||
            cudaDeviceGetAttribute(&maxwin, cudaDevAttrMaxAccessPolicyWindowSize, s->device) != cudaSuccess) {
        cudaGetLastError();
        return;          /* no persisting L2 on this device: nothing to do */
    }
    /* only a count plane that fits in one window: a larger one (the head's 570 MB)
       is mostly cold, and a window over its first gates took L2 from the hot
       elements elsewhere (DRAM writes 0.6 GB -> 13 GB a launch) */
    const size_t counts = sizeof(long long) * (size_t)kp.fieldlen * field_comps(kp);
    const size_t nb = on && maxpersist > 0 && maxwin > 0 && counts <= (size_t)maxwin ? counts : 0;
    const void* base = nb ? (const void*)s->d_field : nullptr;
    if (base == s->l2_base && nb == s->l2_bytes) {
        return;
    }
    if (!nb && s->l2_set) {
        /* no window for this problem: the lines an earlier problem marked
           persisting would keep their share of L2 from it, so they go back
           to normal and the set-aside to what it was */
        cudaCtxResetPersistingL2Cache();
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, s->l2_prev);
        cudaGetLastError();
        s->l2_set = false;
    }
    if (nb && !s->l2_set) {
        /* best effort: a context that refuses the set-aside runs without the window */
        if (cudaDeviceGetLimit(&s->l2_prev, cudaLimitPersistingL2CacheSize) != cudaSuccess ||
                cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, (size_t)maxpersist) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        s->l2_set = true;
    }
    cudaStreamAttrValue v;
    memset(&v, 0, sizeof(v));
    if (nb) {
        v.accessPolicyWindow.base_ptr = (void*)s->d_field;
        v.accessPolicyWindow.num_bytes = nb;
        v.accessPolicyWindow.hitRatio = std::min(1.f, (float)maxpersist / (float)nb);
        v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    }
    if (cudaStreamSetAttribute(s->st, cudaStreamAttributeAccessPolicyWindow, &v) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    s->l2_base = base;
    s->l2_bytes = nb;
    return;
}

}  // namespace

extern "C" {

const char* mcxg_error_string(int code) {
    switch (code) {
        case MCXG_OK: return "ok";
        case MCXG_ERR_CUDA: return "CUDA runtime error";
        case MCXG_ERR_ARG: return "invalid argument";
        case MCXG_ERR_NOMEM: return "out of device memory";
        case MCXG_ERR_LIMIT: return "input exceeds a compiled limit";
        case MCXG_ERR_STATE: return "call out of order";
        case MCXG_ERR_NODEVICE: return "no CUDA device";
        default: return "unknown error";
    }
}

/* the calling thread's current device, and setting it back: the host
   driver restores the caller's device when a public call returns
   (internal to the library, not in the public header) */
int mcxg_internal_current_device(void) {
    int d = -1;
    if (cudaGetDevice(&d) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return d;
}

void mcxg_internal_restore_device(int d) {
    if (d >= 0 && cudaSetDevice(d) != cudaSuccess) {
        cudaGetLastError();
    }
}

int mcxg_device_count(int* n) {
    if (!n) {
        return MCXG_ERR_ARG;
    }
    *n = 0;
    cudaError_t e = cudaGetDeviceCount(n);
    if (e != cudaSuccess) {
        *n = 0;
        cudaGetLastError();
        return MCXG_ERR_NODEVICE;
    }
    return MCXG_OK;
}

int mcxg_device_info(int device, mcxg_devinfo* info) {
    if (!info) {
        return MCXG_ERR_ARG;
    }
    /* cudaGetDeviceProperties takes about 9 ms on a GB300 and every
       mcx_run_simulation lists the devices: the properties do not change
       while the process runs, so each device is queried once */
    static std::mutex lock;
    static mcxg_devinfo cache[64];
    static bool cached[64] = {};
    std::lock_guard<std::mutex> guard(lock);
    if (device >= 0 && device < 64 && cached[device]) {
        *info = cache[device];
        return MCXG_OK;
    }
    cudaDeviceProp p;
    MCXG_TRY(cudaGetDeviceProperties(&p, device));
    memset(info, 0, sizeof(*info));
    snprintf(info->name, sizeof(info->name), "%s", p.name);
    info->major = p.major;
    info->minor = p.minor;
    info->sm = p.multiProcessorCount;
    int clk = 0;
    cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, device);
    info->clock_khz = clk;
    info->globalmem = p.totalGlobalMem;
    info->sharedmem_per_block = p.sharedMemPerBlockOptin;
    info->constmem = p.totalConstMem;
    info->regs_per_block = p.regsPerBlock;
    info->max_threads_per_sm = p.maxThreadsPerMultiProcessor;
    if (device >= 0 && device < 64) {
        cache[device] = *info;
        cached[device] = true;
    }
    return MCXG_OK;
}

int mcxg_create(int device, mcxg_session** out) {
    if (!out) {
        return MCXG_ERR_ARG;
    }
    *out = nullptr;
    int n = 0;
    if (mcxg_device_count(&n) || device < 0 || device >= n) {
        return MCXG_ERR_NODEVICE;
    }
    mcxg_session* s = new (std::nothrow) mcxg_session();
    if (!s) {
        return MCXG_ERR_NOMEM;
    }
    s->device = device;
    int rc = cuda_status(cudaSetDevice(device));
    if (!rc) {
        rc = mcxg_device_info(device, &s->info);
    }
    if (!rc) {
        rc = cuda_status(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
    }
    if (!rc) {
        rc = cuda_status(cudaEventCreate(&s->e0));
    }
    if (!rc) {
        rc = cuda_status(cudaEventCreate(&s->e1));
    }
    if (!rc) {
        rc = cuda_status(cudaMalloc((void**)&s->d_words, 8 * sizeof(unsigned int)));
    }
    if (!rc) {
        rc = cuda_status(cudaMalloc((void**)&s->d_events, 8 * sizeof(unsigned long long)));
    }
    if (!rc) {
        rc = cuda_status(cudaMalloc((void**)&s->d_red, (2 * kRedBlocks + 2) * sizeof(double)));
    }
    if (rc) {
        mcxg_destroy(s);
        return rc;
    }
    *out = s;
    return MCXG_OK;
}

int mcxg_destroy(mcxg_session* s) {
    if (!s) {
        return MCXG_OK;
    }
    cudaSetDevice(s->device);
    if (s->st) {
        cudaStreamSynchronize(s->st);
    }
    if (s->l2_set) {
        /* give the persisting set-aside back: no lines stay persisting, the
           context's limit returns to what it was */
        cudaCtxResetPersistingL2Cache();
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, s->l2_prev);
        cudaGetLastError();
    }
    void* bufs[] = {s->d_media, s->d_prop, s->d_tables, s->d_pattern, s->d_seeds, s->d_field, s->d_energy,
                    s->d_detp, s->d_detseed, s->d_words, s->d_events, s->d_red, s->d_out,
                    s->d_rseed, s->d_rweight, s->d_rtof, s->d_rdetid, s->d_scales, s->d_detw,
                    s->d_sims, s->d_simvt, s->d_simctr, s->d_smatrix, s->d_bmedia, s->d_bfield, s->d_benergy, s->d_bsum, s->d_bout,
                    s->d_adj, s->d_lfib, s->d_jump, s->d_traj, s->d_acc64, s->d_accf, s->d_accs, s->d_adjc,
                    s->d_adjJ, s->d_words32};
    if (s->bgraph_exec) {
        cudaGraphExecDestroy(s->bgraph_exec);
    }
    if (s->bgraph) {
        cudaGraphDestroy(s->bgraph);
    }
    for (void* b : bufs) {
        if (b) {
            cudaFree(b);
        }
    }
    if (s->e0) {
        cudaEventDestroy(s->e0);
    }
    if (s->e1) {
        cudaEventDestroy(s->e1);
    }
    if (s->st) {
        cudaStreamDestroy(s->st);
    }
    delete s;
    return MCXG_OK;
}

namespace {
/* 32-bit label words (label | detector bit 31) to the kernel's bytes (label |
   detector bit 7, the bits of keep), labels below 128 */
__global__ void pack_labels(const uint32_t* __restrict__ words, size_t n, uint32_t keep, uint8_t* __restrict__ bytes) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t w = words[i];
        bytes[i] = (uint8_t)(((w & 0x7Fu) | ((w >> 24) & 0x80u)) & keep);
    }
}
}  // namespace

int mcxg_set_problem(mcxg_session* s, const void* kparams, size_t kparams_size, const void* media,
                     uint32_t mediaword, const float* prop, const float* detpos, const float* srcextra,
                     const float* invcdf, const float* angleinvcdf, const float* srcpattern, size_t npattern) {
    if (!s || !kparams || kparams_size != sizeof(mcxg_kparams) || !media || !prop) {
        return MCXG_ERR_ARG;
    }
    const mcxg_kparams& kp = *(const mcxg_kparams*)kparams;
    /* MCXG_MEDIA_PACK: 32-bit words in, bytes on the device */
    const bool pack = mediaword == MCXG_MEDIA_PACK;
    if (pack) {
        if (kp.mediaformat > 4 || kp.medianum > 128) {
            return MCXG_ERR_ARG;
        }
        mediaword = 1;
    }
    if (mediaword != 1 && mediaword != 4) {
        return MCXG_ERR_ARG;
    }
    if (kp.medianum < 2 && kp.mediaformat <= 4) {
        return MCXG_ERR_ARG;
    }
    if (kp.medianum > MCXG_MAX_MEDIA || kp.detnum > MCXG_MAX_DET || kp.extrasrclen > MCXG_MAX_EXTRASRC) {
        return MCXG_ERR_LIMIT;
    }
    if ((kp.detnum && !detpos) || (kp.extrasrclen && !srcextra) || (kp.nphase && !invcdf) ||
            (kp.nangle && !angleinvcdf) || ((kp.srctype == MCX_SRC_PATTERN || kp.srctype == MCX_SRC_PATTERN3D) && !srcpattern)) {
        return MCXG_ERR_ARG;
    }
    if (kp.nvox == 0 || kp.fieldlen == 0 || kp.nthread == 0) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    s->kp = kp;
    s->kp.mediaword = mediaword;
    s->kp.npattern = (uint32_t)(npattern ? npattern : 1);
    /* split-voxel volumes carry a second plane (plane point and normal) */
    size_t mbytes = (size_t)kp.nvox * mediaword * (kp.mediaformat == 97 ? 2 : 1);
    int rc = ensure((uint8_t**)&s->d_media, &s->media_cap, mbytes);
    if (!rc) {
        rc = ensure(&s->d_prop, &s->prop_cap, kp.medianum);
    }
    if (!rc) {
        rc = ensure(&s->d_tables, &s->tables_cap, (size_t)kp.nphase + kp.nangle + 1);
    }
    if (!rc && npattern) {
        rc = ensure(&s->d_pattern, &s->pattern_cap, npattern);
    }
    if (!rc) {
        rc = ensure(&s->d_field, &s->field_cap, kFieldPlanes * (size_t)kp.fieldlen * field_comps(kp));
    }
    if (!rc && kp.savedet) {
        size_t recs = kp.maxdetphoton;
        rc = ensure(&s->d_detp, &s->detp_cap, recs * (kp.reclen ? kp.reclen : 1));
        if (!rc && kp.issaveseed) {
            rc = ensure(&s->d_detseed, &s->detseed_cap, recs * 2 + 2);
        }
        if (!rc) {
            rc = ensure(&s->d_detw, &s->detw_cap, recs + 1);
        }
    }
    if (!rc && pack) {
        rc = ensure(&s->d_words32, &s->words32_cap, (size_t)kp.nvox);
    }
    if (rc) {
        return rc;
    }
    if (pack) {
        MCXG_TRY(cudaMemcpyAsync(s->d_words32, media, sizeof(uint32_t) * (size_t)kp.nvox, cudaMemcpyHostToDevice, s->st));
        pack_labels<<<grid_for(s, kp.nvox), 256, 0, s->st>>>(s->d_words32, kp.nvox, 0xFFu, (uint8_t*)s->d_media);
        MCXG_TRY(cudaGetLastError());
    } else {
        MCXG_TRY(cudaMemcpyAsync(s->d_media, media, mbytes, cudaMemcpyHostToDevice, s->st));
    }
    MCXG_TRY(cudaMemcpyAsync(s->d_prop, prop, sizeof(float) * 4 * kp.medianum, cudaMemcpyHostToDevice, s->st));
    if (kp.nphase) {
        MCXG_TRY(cudaMemcpyAsync(s->d_tables, invcdf, sizeof(float) * kp.nphase, cudaMemcpyHostToDevice, s->st));
    }
    if (kp.nangle) {
        MCXG_TRY(cudaMemcpyAsync(s->d_tables + kp.nphase, angleinvcdf, sizeof(float) * kp.nangle,
                                 cudaMemcpyHostToDevice, s->st));
    }
    if (npattern) {
        MCXG_TRY(cudaMemcpyAsync(s->d_pattern, srcpattern, sizeof(float) * npattern, cudaMemcpyHostToDevice, s->st));
    }
    s->h_det.assign(detpos ? detpos : prop, detpos ? detpos + 4 * kp.detnum : prop);
    s->h_srcx.assign(srcextra ? srcextra : prop, srcextra ? srcextra + 16 * kp.extrasrclen : prop);
    s->up_fast = s->up_exact = false;
    s->has_problem = true;
    s->npol = 0;
    s->tuned = 0;
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_set_params(mcxg_session* s, const void* kparams, size_t kparams_size) {
    if (!s || !kparams || kparams_size != sizeof(mcxg_kparams)) {
        return MCXG_ERR_ARG;
    }
    if (!s->has_problem) {
        return MCXG_ERR_STATE;
    }
    const mcxg_kparams& kp = *(const mcxg_kparams*)kparams;
    if (kp.nvox != s->kp.nvox || kp.fieldlen != s->kp.fieldlen || kp.medianum != s->kp.medianum ||
            kp.detnum != s->kp.detnum || kp.extrasrclen != s->kp.extrasrclen || kp.nphase != s->kp.nphase ||
            kp.nangle != s->kp.nangle || kp.savedet != s->kp.savedet || kp.maxdetphoton != s->kp.maxdetphoton ||
            kp.reclen != s->kp.reclen) {
        return MCXG_ERR_ARG;    /* buffer shapes change only through mcxg_set_problem */
    }
    uint32_t mw = s->kp.mediaword, np = s->kp.npattern;
    s->kp = kp;
    s->kp.mediaword = mw;
    s->kp.npattern = np;
    s->up_fast = s->up_exact = false;
    return MCXG_OK;
}

int mcxg_set_seeds(mcxg_session* s, const uint32_t* seeds, uint32_t nthread) {
    if (!s || !seeds || nthread == 0) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    int rc = ensure(&s->d_seeds, &s->seeds_cap, nthread);
    if (!rc) {
        rc = ensure(&s->d_energy, &s->energy_cap, nthread);
    }
    if (rc) {
        return rc;
    }
    MCXG_TRY(cudaMemcpyAsync(s->d_seeds, seeds, sizeof(uint4) * nthread, cudaMemcpyHostToDevice, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    s->has_seeds = true;
    return MCXG_OK;
}

/* Seed words of the additive lagged-Fibonacci generator o[k] = o[k-3] +
   o[k-31] (mod 2^32), each word o[k] >> 1: block j (one thread) starts from
   the window starts[31 j .. 31 j + 30] = o[j B - 31 .. j B - 1] and writes
   words j B .. min((j + 1) B, nword) - 1.  The ring lives in registers: in
   each unrolled group of 31, r[t] holds o[k - 31] before and o[k] after its
   update, and r[(t + 28) % 31] holds o[k - 3] (this group's new value for
   t >= 3, the previous group's, not yet overwritten, for t < 3). */
namespace {
__device__ __forceinline__ void lfib_expand(uint32_t (&r)[31], size_t begin, size_t end, uint32_t* __restrict__ out) {
    for (size_t base = begin; base < end; base += 31) {
#pragma unroll
        for (int t = 0; t < 31; t++) {
            r[t] += r[(t + 28) % 31];
            if (base + t < end) {
                out[base + t] = r[t] >> 1;
            }
        }
    }
}

__global__ void __launch_bounds__(128) lfib_words(const uint32_t* __restrict__ starts, uint32_t nblock,
                                                  uint32_t blocklen, uint32_t nword, uint32_t* __restrict__ out) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nblock) {
        return;
    }
    uint32_t r[31];
#pragma unroll
    for (int t = 0; t < 31; t++) {
        r[t] = starts[31 * (size_t)j + t];
    }
    const size_t begin = (size_t)j * blocklen;
    lfib_expand(r, begin, begin + blocklen < nword ? begin + blocklen : nword, out);
}

/* The jump-ahead on the device.  One step of the generator is the window
   map W' = M W (W = o[k-31 .. k-1]; W'[t] = W[t+1] for t < 30, W'[30] =
   W[0] + W[28]), so block j's window is (M^B)^j W0.  lf_powers (one CTA, a
   thread per matrix element, products mod 2^32 in shared memory) makes Q_0 =
   M^B by square-and-multiply and Q_b = Q_{b-1}^2; lfib_jump_words then
   applies Q_b to W0 for each set bit b of its block index and expands the
   block as lfib_words does. */
__device__ __forceinline__ void lf_mul_shared(const uint32_t* X, const uint32_t* Y, uint32_t* Z, int t) {
    uint32_t acc = 0;
    if (t < 31 * 31) {
        const int i = t / 31, k = t - 31 * (t / 31);
#pragma unroll
        for (int m = 0; m < 31; m++) {
            acc += X[31 * i + m] * Y[31 * m + k];
        }
    }
    __syncthreads();
    if (t < 31 * 31) {
        Z[t] = acc;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(1024) lf_powers(uint32_t blocklen, uint32_t npow, uint32_t* __restrict__ pows) {
    __shared__ uint32_t P[31 * 31], B[31 * 31];
    const int t = threadIdx.x;
    if (t < 31 * 31) {
        const int i = t / 31, k = t - 31 * (t / 31);
        P[t] = (i == k) ? 1u : 0u;
        B[t] = (i < 30 && k == i + 1) || (i == 30 && (k == 0 || k == 28)) ? 1u : 0u;
    }
    __syncthreads();
    for (uint32_t e = blocklen; e;) {
        if (e & 1u) {
            lf_mul_shared(P, B, P, t);
        }
        e >>= 1;
        if (e) {
            lf_mul_shared(B, B, B, t);
        }
    }
    for (uint32_t b = 0; b < npow; b++) {
        if (t < 31 * 31) {
            pows[31 * 31 * (size_t)b + t] = P[t];
        }
        if (b + 1 < npow) {
            lf_mul_shared(P, P, P, t);
        }
    }
}

__global__ void __launch_bounds__(128) lfib_jump_words(const uint32_t* __restrict__ w0, const uint32_t* __restrict__ pows,
                                                       uint32_t npow, uint32_t nblock, uint32_t blocklen, uint32_t nword,
                                                       uint32_t* __restrict__ out) {
    /* one 31-word group of each lane at a time, through a per-warp tile: the
       warp then writes lane L's 31 consecutive words with 31 lanes (one
       coalesced run) instead of 32 words 4 x blocklen bytes apart */
    __shared__ uint32_t tile[4][32 * 33];
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned int lane = threadIdx.x & 31u;
    uint32_t* my = tile[threadIdx.x >> 5];
    const uint32_t j0 = j - lane;             /* the warp's first block */
    if (j0 >= nblock) {
        return;                               /* the whole warp is past the last block */
    }
    uint32_t r[31];
#pragma unroll
    for (int t = 0; t < 31; t++) {
        r[t] = w0[t];
    }
    for (uint32_t b = 0; b < npow; b++) {
        if (j < nblock && ((j >> b) & 1u)) {
            const uint32_t* Q = pows + 31 * 31 * (size_t)b;
            uint32_t w[31];
#pragma unroll
            for (int i = 0; i < 31; i++) {
                uint32_t acc = 0;
#pragma unroll
                for (int m = 0; m < 31; m++) {
                    acc += __ldg(Q + 31 * i + m) * r[m];
                }
                w[i] = acc;
            }
#pragma unroll
            for (int i = 0; i < 31; i++) {
                r[i] = w[i];
            }
        }
    }
    for (uint32_t off = 0; off < blocklen; off += 31) {
#pragma unroll
        for (int t = 0; t < 31; t++) {
            r[t] += r[(t + 28) % 31];
            my[lane * 33 + t] = r[t] >> 1;
        }
        __syncwarp();
        /* lanes past the last block hold no words: their runs start at or past nword */
        for (unsigned int L = 0; L < 32; L++) {
            const size_t bL = (size_t)(j0 + L) * blocklen;
            const size_t eL = bL + blocklen < nword ? bL + blocklen : nword;
            const size_t k = bL + off + lane;
            if (lane < 31 && k < eL) {
                out[k] = my[L * 33 + lane];
            }
        }
        __syncwarp();
    }
}
}  // namespace

int mcxg_set_seeds_lfib(mcxg_session* s, const uint32_t* starts, uint32_t nblock, uint32_t blocklen,
                        uint32_t nthread) {
    const uint64_t nword = 4ull * nthread;
    if (!s || !starts || nthread == 0 || nblock == 0 || blocklen == 0 || nword > 0xFFFFFFFFull ||
        (uint64_t)nblock * blocklen < nword || (uint64_t)(nblock - 1) * blocklen >= nword) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    int rc = ensure(&s->d_seeds, &s->seeds_cap, nthread);
    if (!rc) {
        rc = ensure(&s->d_energy, &s->energy_cap, nthread);
    }
    if (!rc) {
        rc = ensure(&s->d_lfib, &s->lfib_cap, 31 * (size_t)nblock);
    }
    if (rc) {
        return rc;
    }
    MCXG_TRY(cudaMemcpyAsync(s->d_lfib, starts, sizeof(uint32_t) * 31 * (size_t)nblock, cudaMemcpyHostToDevice, s->st));
    lfib_words<<<(nblock + 127) / 128, 128, 0, s->st>>>(s->d_lfib, nblock, blocklen, (uint32_t)nword,
                                                         (uint32_t*)s->d_seeds);
    MCXG_TRY(cudaGetLastError());
    MCXG_TRY(cudaStreamSynchronize(s->st));
    s->has_seeds = true;
    return MCXG_OK;
}

int mcxg_set_seeds_window(mcxg_session* s, const uint32_t* window, uint32_t nthread) {
    const uint64_t nword = 4ull * nthread;
    if (!s || !window || nthread == 0 || nword > 0xFFFFFFFFull) {
        return MCXG_ERR_ARG;
    }
    /* blocks of at least 1,024 words, at most 65,536 blocks: a 1e8-photon
       launch's 80 M words in 65,536 blocks of 1,216 */
    const uint32_t blocklen = (uint32_t)std::max<uint64_t>(1024, (nword + 65535) / 65536);
    const uint32_t nblock = (uint32_t)((nword + blocklen - 1) / blocklen);
    uint32_t npow = 0;
    while (npow < 32 && ((uint64_t)1 << npow) < nblock) {
        npow++;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    int rc = ensure(&s->d_seeds, &s->seeds_cap, nthread);
    if (!rc) {
        rc = ensure(&s->d_energy, &s->energy_cap, nthread);
    }
    if (!rc) {
        rc = ensure(&s->d_lfib, &s->lfib_cap, 31 + 31 * 31 * (size_t)std::max<uint32_t>(npow, 1));
    }
    if (rc) {
        return rc;
    }
    MCXG_TRY(cudaMemcpyAsync(s->d_lfib, window, sizeof(uint32_t) * 31, cudaMemcpyHostToDevice, s->st));
    if (npow) {
        lf_powers<<<1, 1024, 0, s->st>>>(blocklen, npow, s->d_lfib + 31);
    }
    lfib_jump_words<<<(nblock + 127) / 128, 128, 0, s->st>>>(s->d_lfib, s->d_lfib + 31, npow, nblock, blocklen,
                                                              (uint32_t)nword, (uint32_t*)s->d_seeds);
    MCXG_TRY(cudaGetLastError());
    MCXG_TRY(cudaStreamSynchronize(s->st));
    s->has_seeds = true;
    return MCXG_OK;
}

int mcxg_get_seeds(mcxg_session* s, uint32_t* out, uint32_t nthread) {
    if (!s || !out || !s->has_seeds || nthread > s->seeds_cap) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    MCXG_TRY(cudaMemcpyAsync(out, s->d_seeds, sizeof(uint4) * nthread, cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_set_trajectory(mcxg_session* s, uint32_t maxrec) {
    if (!s) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    s->maxjump = 0;
    if (maxrec) {
        int rc = ensure(&s->d_jump, &s->jump_cap, 1);
        if (!rc) {
            rc = ensure(&s->d_traj, &s->traj_cap, 6 * (size_t)maxrec);
        }
        if (rc) {
            return rc;
        }
        s->maxjump = maxrec;
    }
    return MCXG_OK;
}

int mcxg_get_trajectory(mcxg_session* s, float* out, uint32_t maxrec, uint32_t* count) {
    if (!s || !count || (maxrec && !out) || !s->maxjump) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    unsigned int n = 0;
    MCXG_TRY(cudaMemcpyAsync(&n, s->d_jump, sizeof(n), cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    *count = n;
    const size_t take = (size_t)(n < s->maxjump ? n : s->maxjump) < maxrec ? (n < s->maxjump ? n : s->maxjump) : maxrec;
    if (take) {
        MCXG_TRY(cudaMemcpyAsync(out, s->d_traj, sizeof(float) * 6 * take, cudaMemcpyDeviceToHost, s->st));
        MCXG_TRY(cudaStreamSynchronize(s->st));
    }
    return MCXG_OK;
}

int mcxg_set_replay(mcxg_session* s, const void* seeds16, const float* weight, const float* tof, const int* detid,
                    uint32_t n) {
    if (!s || (n && (!seeds16 || !weight || !tof || !detid))) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    /* one spare entry so an empty replay still has valid pointers */
    int rc = ensure(&s->d_rseed, &s->rseed_cap, (size_t)n + 1);
    if (!rc) {
        rc = ensure(&s->d_rweight, &s->rweight_cap, (size_t)n + 1);
    }
    if (!rc) {
        rc = ensure(&s->d_rtof, &s->rtof_cap, (size_t)n + 1);
    }
    if (!rc) {
        rc = ensure(&s->d_rdetid, &s->rdetid_cap, (size_t)n + 1);
    }
    if (rc) {
        return rc;
    }
    if (n) {
        MCXG_TRY(cudaMemcpyAsync(s->d_rseed, seeds16, 16 * (size_t)n, cudaMemcpyHostToDevice, s->st));
        MCXG_TRY(cudaMemcpyAsync(s->d_rweight, weight, sizeof(float) * n, cudaMemcpyHostToDevice, s->st));
        MCXG_TRY(cudaMemcpyAsync(s->d_rtof, tof, sizeof(float) * n, cudaMemcpyHostToDevice, s->st));
        MCXG_TRY(cudaMemcpyAsync(s->d_rdetid, detid, sizeof(int) * n, cudaMemcpyHostToDevice, s->st));
    }
    MCXG_TRY(cudaStreamSynchronize(s->st));
    s->nreplay = n;
    return MCXG_OK;
}

int mcxg_set_tile(mcxg_session* s, uint32_t elements) {
    if (!s) {
        return MCXG_ERR_ARG;
    }
    s->tile_req = elements;
    return MCXG_OK;
}

int mcxg_get_tile(mcxg_session* s, uint32_t* box) {
    if (!s || !box) {
        return MCXG_ERR_ARG;
    }
    const KArgs::Tile& t = s->tile_used;
    const uint32_t v[8] = {(uint32_t)t.x0, (uint32_t)t.y0, (uint32_t)t.z0, t.nx, t.ny, t.nz, t.ng,
                           t.nx * t.ny * t.nz * t.ng};
    memcpy(box, v, sizeof(v));
    return MCXG_OK;
}

int mcxg_set_launch(mcxg_session* s, int block, int blocks_per_sm) {
    if (!s || block < 0 || block > 256 || (block % 32) || blocks_per_sm < 0) {
        return MCXG_ERR_ARG;
    }
    s->block_req = block;
    s->bpsm_req = blocks_per_sm;
    return MCXG_OK;
}

int mcxg_simulate(mcxg_session* s, unsigned int flags, float* kernel_ms) {
    if (!s) {
        return MCXG_ERR_ARG;
    }
    if (!s->has_problem || !s->has_seeds || s->seeds_cap < s->kp.nthread || s->energy_cap < s->kp.nthread) {
        return MCXG_ERR_STATE;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    const mcxg_kparams& kp = s->kp;
    const bool exact = (flags & (MCXG_EXACT | MCXG_RNGDUMP)) != 0;

    if (exact && !s->up_exact) {
        MCXG_TRY(mcxg::exact_upload(&kp, s->h_det.data(), kp.detnum, s->h_srcx.data(), kp.extrasrclen, s->st));
        s->up_exact = true;
    }
    if (!exact && !s->up_fast) {
        MCXG_TRY(mcxg::fast_upload(&kp, s->h_det.data(), kp.detnum, s->h_srcx.data(), kp.extrasrclen, s->st));
        s->up_fast = true;
    }
    {
        /* a run that turns on the complex field after mcxg_set_problem */
        const size_t need = kFieldPlanes * (size_t)kp.fieldlen * field_comps(kp);
        if (need > s->field_cap) {
            if (flags & MCXG_KEEP) {
                return MCXG_ERR_STATE;
            }
            const int rc = ensure(&s->d_field, &s->field_cap, need);
            if (rc) {
                return rc;
            }
        }
    }
    if (!(flags & MCXG_KEEP)) {
        MCXG_TRY(cudaMemsetAsync(s->d_field, 0, sizeof(float) * kFieldPlanes * (size_t)kp.fieldlen * field_comps(kp), s->st));
    }
    s->out_valid = false;
    MCXG_TRY(cudaMemsetAsync(s->d_energy, 0, sizeof(float2) * kp.nthread, s->st));
    MCXG_TRY(cudaMemsetAsync(s->d_words, 0, 8 * sizeof(unsigned int), s->st));
    MCXG_TRY(cudaMemsetAsync(s->d_events, 0, 8 * sizeof(unsigned long long), s->st));

    KArgs a;
    memset(&a, 0, sizeof(a));
    a.media8 = (const uint8_t*)s->d_media;
    a.media32 = (const uint32_t*)s->d_media;
    a.gprop = s->d_prop;
    a.invcdf = s->d_tables;
    a.angleinvcdf = s->d_tables + kp.nphase;
    a.srcpattern = s->d_pattern;
    a.seeds = s->d_seeds;
    a.field = s->d_field;
    a.fhi = reinterpret_cast<unsigned long long*>(s->d_field);
    a.flo = s->d_field + 2 * (size_t)kp.fieldlen * field_comps(kp);
    a.smatrix = s->d_smatrix;
    a.s0 = s->pol_s0;
    a.maxpol = s->npol;
    a.jumpctr = s->d_jump;
    a.traj = s->d_traj;
    a.maxjump = s->maxjump;
    if (s->maxjump) {
        MCXG_TRY(cudaMemsetAsync(s->d_jump, 0, sizeof(unsigned int), s->st));
    }
    a.energy = s->d_energy;
    a.detp = s->d_detp;
    a.detseed = s->d_detseed;
    a.detw = kp.savedet ? s->d_detw : nullptr;
    a.detcount = s->d_words + 0;
    a.vtcounter = s->d_words + 1;
    a.status = s->d_words + 2;
    a.counters = s->d_events;
    a.rseed = s->d_rseed;
    a.rweight = s->d_rweight;
    a.rtof = s->d_rtof;
    a.rdetid = s->d_rdetid;
    if (kp.replay && (kp.nreplay > s->nreplay || !s->d_rseed)) {
        return MCXG_ERR_STATE;
    }

    /* deposits go straight to the field unless aggregation is asked for or
       the autotuner found it faster for this problem */
    const bool verify = (flags & MCXG_VERIFY) != 0;
    const unsigned int adjmode = (flags & MCXG_ADJ1) ? 1u : ((flags & MCXG_ADJ2) ? 2u : 0u);
    if (adjmode) {
        /* the two passes of the fluence gradient: flux or fluence output, fast
           kernel, no replay, the loss gradient set for this problem */
        if (exact || verify || kp.replay || (flags & MCXG_KEEP) || !s->adj_ready || kp.is2d ||
                !(kp.outputtype == otFlux || kp.outputtype == otFluence) || kp.omega > 0.f || s->npol ||
                kp.mediaformat == 97 || kp.srcnum > 1 || s->maxjump || kp.minenergy > 0.f ||
                s->adjJ_cap < (size_t)kp.nthread * (kp.threadphoton + 1u)) {
            return MCXG_ERR_ARG;
        }
        a.adjc = s->d_adjc;
        a.adjJ = s->d_adjJ;
        a.adjmode = adjmode;
    }
    const bool noagg = verify || adjmode || (flags & MCXG_NOAGG) || !((flags & MCXG_AGG) || (s->tuned && !s->tuned_noagg));
    const bool rf = kp.omega > 0.f && !kp.replay;
    const bool pol = s->npol > 0;
    const bool svmc = kp.mediaformat == 97;
    const bool xmedia = !rf && !svmc && kp.mediaformat > 4 && kp.mediaformat != 101;
    /* the instantiations that fix the common configuration's parameters */
    const bool common = !rf && !pol && !(flags & MCXG_GENERAL) && kp.mediaformat <= 4 && !kp.is2d && kp.nphase <= 2 &&
                        kp.srcnum <= 1 && !s->maxjump;
    /* launch shape: block threads x blocks per SM.  Shapes of more than 512
       threads per SM take the instantiation whose registers are capped (64
       a thread: 1,024 resident threads, the default), the others the
       uncapped one.  The specialised instantiations exist only capped: the
       fluence-gradient passes at 64 registers, the others at 80 (768
       threads) */
    const int block = s->block_req ? s->block_req : 256;
    const bool special = xmedia || rf || pol || svmc || verify || adjmode;
    const int bpsm_sel = special ? (adjmode ? 1024 : 768) / block : (s->bpsm_req ? s->bpsm_req : 1024 / block);
    const bool capped = special || block * bpsm_sel > 512;
    int lflags = (kp.savedet ? mcxg::LF_DET : 0) | (kp.dorefl_compiled ? mcxg::LF_REFL : 0) |
                 (noagg ? 0 : mcxg::LF_WAGG) | (capped ? mcxg::LF_CAPPED : 0) | (xmedia ? mcxg::LF_XMEDIA : 0) |
                 (common ? mcxg::LF_COMMON : 0) | (rf ? mcxg::LF_RF : 0) | (pol ? mcxg::LF_POL : 0) |
                 (svmc ? mcxg::LF_SVMC : 0) | (verify ? mcxg::LF_ACC64 : 0) | (adjmode ? mcxg::LF_ADJ : 0);
    if (verify) {
        /* the precision check runs the fast common-configuration instantiation */
        if (exact || !common || kp.replay || (flags & MCXG_KEEP)) {
            return MCXG_ERR_ARG;
        }
        const size_t n = kp.fieldlen;
        int rc = ensure(&s->d_acc64, &s->acc64_cap, n);
        if (!rc) {
            rc = ensure(&s->d_accf, &s->accf_cap, n);
        }
        if (!rc) {
            rc = ensure(&s->d_accs, &s->accs_cap, 2 * n);
        }
        if (rc) {
            return rc;
        }
        MCXG_TRY(cudaMemsetAsync(s->d_acc64, 0, sizeof(double) * n, s->st));
        MCXG_TRY(cudaMemsetAsync(s->d_accf, 0, sizeof(float) * n, s->st));
        MCXG_TRY(cudaMemsetAsync(s->d_accs, 0, sizeof(float) * 2 * n, s->st));
        a.acc64 = s->d_acc64;
        a.accf = s->d_accf;
        a.accs = s->d_accs;
    }
    size_t smem = shared_bytes(kp, block);
    s->tile_used = KArgs::Tile{};
    if (s->tile_req && !exact && common && !verify && !adjmode && !kp.replay && !kp.extrasrclen && kp.srcnum <= 1 &&
            kp.save2pt && !(flags & MCXG_RNGDUMP)) {
        /* the hot-voxel tile: what shared memory is left at this shape's
           blocks per SM (1 KB of each block's share is the system's) */
        int smsm = 0;
        MCXG_TRY(cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, s->device));
        const size_t off = (smem + 7) & ~(size_t)7;
        const long long avail = (long long)smsm / bpsm_sel - 1024 - (long long)off;
        const uint32_t maxel = avail > 0 ? (uint32_t)std::min<long long>(avail / 12, (long long)s->tile_req) : 0u;
        KArgs::Tile t;
        if (tile_geometry(kp, maxel, t)) {
            t.smemoff = (uint32_t)off;
            a.tile = t;
            smem = off + 12 * (size_t)t.nx * t.ny * t.nz * t.ng;
            lflags |= mcxg::LF_TILE;
            s->tile_used = t;
        }
    }
    if (smem > s->info.sharedmem_per_block) {
        return MCXG_ERR_LIMIT;
    }
    int bpsm = exact ? 2 : bpsm_sel;
    if (!exact) {
        /* never more blocks than fit at once: a persistent grid must be resident */
        int occ = 0;
        MCXG_TRY(mcxg::fast_occupancy(lflags, block, smem, &occ));
        if (occ >= 1 && bpsm > occ) {
            bpsm = occ;
        }
    }
    if (bpsm < 1) {
        bpsm = 1;
    }
    int grid = s->info.sm * bpsm;
    s->grid = grid;
    s->block = block;
    if (!exact) {
        cudaFuncAttributes fa;
        if (mcxg::fast_attributes(lflags, &fa) == cudaSuccess) {
            s->regs = fa.numRegs;
        }
    }

    l2_window(s, kp, !(flags & MCXG_NOL2WINDOW) && !adjmode);
    MCXG_TRY(cudaEventRecord(s->e0, s->st));
    if (flags & MCXG_RNGDUMP) {
        MCXG_TRY(mcxg::exact_rngdump(a, s->info.sm * 4, 256, s->st));
    } else if (exact) {
        MCXG_TRY(mcxg::exact_launch(a, lflags, grid, block, smem, s->st));
    } else {
        MCXG_TRY(mcxg::fast_launch(a, lflags, grid, block, smem, s->st));
    }
    MCXG_TRY(cudaEventRecord(s->e1, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    MCXG_TRY(cudaGetLastError());
    if (kernel_ms) {
        float ms = 0.f;
        MCXG_TRY(cudaEventElapsedTime(&ms, s->e0, s->e1));
        *kernel_ms = ms;
    }
    return MCXG_OK;
}

int mcxg_autotune(mcxg_session* s, uint32_t sample_photons, int* block, int* blocks_per_sm, int* noagg) {
    if (!s) {
        return MCXG_ERR_ARG;
    }
    if (!s->has_problem || !s->has_seeds) {
        return MCXG_ERR_STATE;
    }
    /* run a sample of the problem: the first sample_photons photons of the
       reference threads (same seeds), with each candidate shape */
    mcxg_kparams full = s->kp;
    mcxg_kparams samp = full;
    unsigned long long total = (unsigned long long)full.threadphoton * full.nthread + (unsigned int)full.oddphoton;
    if (sample_photons && sample_photons < total) {
        samp.threadphoton = sample_photons / full.nthread;
        samp.oddphoton = (int)(sample_photons - samp.threadphoton * full.nthread);
    }
    s->kp = samp;
    s->up_fast = false;
    /* the block sizes 64, 128 and 256 at 1,024 resident threads per SM (64
       registers) and 128 and 256 at 512 (uncapped registers), direct
       deposits; then the fastest with warp-aggregated deposits */
    struct Cand {
        int block, bpsm, noagg;
    } cands[] = {{256, 4, 1}, {128, 8, 1}, {64, 16, 1}, {256, 2, 1}, {128, 4, 1}, {0, 0, 0}};
    const int ncand = (int)(sizeof(cands) / sizeof(cands[0]));
    float best = 1e30f;
    Cand pick = cands[0];
    int keep_block = s->block_req, keep_bpsm = s->bpsm_req;
    int rc = MCXG_OK;
    for (int ci = 0; ci < ncand && !rc; ci++) {
        Cand c = cands[ci];
        if (!c.block) {
            c = pick;            /* the last candidate: the best shape, aggregated */
            c.noagg = 0;
        }
        s->block_req = c.block;
        s->bpsm_req = c.bpsm;
        float ms = 0.f, t = 1e30f;
        for (int rep = 0; rep < 2 && !rc; rep++) {
            rc = mcxg_simulate(s, c.noagg ? MCXG_NOAGG : MCXG_AGG, &ms);
            if (ms < t) {
                t = ms;
            }
        }
        if (!rc && t < best) {
            best = t;
            pick = c;
        }
    }
    s->kp = full;
    s->up_fast = false;
    s->block_req = keep_block;
    s->bpsm_req = keep_bpsm;
    if (rc) {
        return rc;
    }
    if (!keep_block && !keep_bpsm) {
        s->block_req = pick.block;
        s->bpsm_req = pick.bpsm;
    }
    s->tuned = 1;
    s->tuned_noagg = pick.noagg;
    if (block) {
        *block = pick.block;
    }
    if (blocks_per_sm) {
        *blocks_per_sm = pick.bpsm;
    }
    if (noagg) {
        *noagg = pick.noagg;
    }
    return MCXG_OK;
}

int mcxg_get_energy(mcxg_session* s, double* escaped, double* launched) {
    if (!s || !s->has_seeds) {
        return MCXG_ERR_STATE;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    energy_partials<<<kRedBlocks, kRedThreads, 0, s->st>>>(s->d_energy, s->kp.nthread, s->d_red);
    energy_final<<<1, 32, 0, s->st>>>(s->d_red, kRedBlocks);
    double h[2];
    MCXG_TRY(cudaMemcpyAsync(h, s->d_red + 2 * kRedBlocks, sizeof(h), cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    if (escaped) {
        *escaped = h[0];
    }
    if (launched) {
        *launched = h[1];
    }
    return MCXG_OK;
}

int mcxg_get_thread_energy(mcxg_session* s, float* out) {
    if (!s || !out || !s->has_seeds) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    MCXG_TRY(cudaMemcpyAsync(out, s->d_energy, sizeof(float2) * s->kp.nthread, cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_get_field(mcxg_session* s, float* out, double scale) {
    if (!s || !out || !s->has_problem) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    size_t n = s->kp.fieldlen, total = n * field_comps(s->kp);
    int rc = ensure((double**)&s->d_out, &s->out_cap, total);
    if (rc) {
        return rc;
    }
    field_merge_f32<<<grid_for(s, total), 256, 0, s->st>>>(s->d_field, n, total, (double)s->kp.fxunit, scale,
                                                           (float*)s->d_out);
    s->out_valid = true;
    MCXG_TRY(cudaMemcpyAsync(out, s->d_out, sizeof(float) * total, cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_get_field_blocks(mcxg_session* s, float* out, const double* scales, uint32_t nblocks) {
    if (!s || !out || !scales || nblocks == 0 || !s->has_problem || s->kp.fieldlen % nblocks) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    size_t n = s->kp.fieldlen, total = n * field_comps(s->kp);
    int rc = ensure((double**)&s->d_out, &s->out_cap, total);
    if (!rc) {
        rc = ensure(&s->d_scales, &s->scales_cap, nblocks);
    }
    if (rc) {
        return rc;
    }
    MCXG_TRY(cudaMemcpyAsync(s->d_scales, scales, sizeof(double) * nblocks, cudaMemcpyHostToDevice, s->st));
    field_merge_blocks<<<grid_for(s, total), 256, 0, s->st>>>(s->d_field, n, total, (double)s->kp.fxunit, n / nblocks,
                                                              s->d_scales,
                                                              (float*)s->d_out);
    s->out_valid = true;
    MCXG_TRY(cudaMemcpyAsync(out, s->d_out, sizeof(float) * total, cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_get_field_interleaved(mcxg_session* s, float* out, const double* scales, uint32_t nsrc) {
    if (!s || !out || !scales || nsrc == 0 || !s->has_problem || s->kp.fieldlen % nsrc) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    size_t n = s->kp.fieldlen, total = n * field_comps(s->kp);
    int rc = ensure((double**)&s->d_out, &s->out_cap, total);
    if (!rc) {
        rc = ensure(&s->d_scales, &s->scales_cap, nsrc);
    }
    if (rc) {
        return rc;
    }
    MCXG_TRY(cudaMemcpyAsync(s->d_scales, scales, sizeof(double) * nsrc, cudaMemcpyHostToDevice, s->st));
    field_merge_interleaved<<<grid_for(s, total), 256, 0, s->st>>>(s->d_field, n, total, (double)s->kp.fxunit, nsrc,
                                                                   s->d_scales,
                                                                   (float*)s->d_out);
    s->out_valid = true;
    MCXG_TRY(cudaMemcpyAsync(out, s->d_out, sizeof(float) * total, cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_set_polarization(mcxg_session* s, const float* smatrix, uint32_t nmedia, const float* s0) {
    if (!s || (nmedia && (!smatrix || !s0))) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    if (nmedia) {
        int rc = ensure(&s->d_smatrix, &s->smatrix_cap, (size_t)nmedia * MCX_NANGLES);
        if (rc) {
            return rc;
        }
        MCXG_TRY(cudaMemcpyAsync(s->d_smatrix, smatrix, sizeof(float4) * nmedia * MCX_NANGLES, cudaMemcpyHostToDevice,
                                 s->st));
        MCXG_TRY(cudaStreamSynchronize(s->st));
        s->pol_s0 = make_float4(s0[0], s0[1], s0[2], s0[3]);
    }
    s->npol = nmedia;
    return MCXG_OK;
}

static int adjoint_run(mcxg_session* s, int kind, const float* dfield, uint32_t ns, uint32_t nd, uint32_t nx,
                       uint32_t ny, uint32_t nz, uint32_t maxgate, float* out) {
    const unsigned int nvox = nx * ny * nz;
    const size_t len = (size_t)nvox * ns * nd;
    int rc = ensure(&s->d_adj, &s->adj_cap, len);
    if (rc) {
        return rc;
    }
    const int grid = grid_for(s, nvox);
    if (kind == 0) {
        adjoint_mua<<<grid, 256, 0, s->st>>>(dfield, s->d_adj, nvox, maxgate, ns, nd);
    } else {
        adjoint_dcoeff<<<grid, 256, 0, s->st>>>(dfield, s->d_adj, nvox, maxgate, ns, nd, nx, ny);
    }
    MCXG_TRY(cudaMemcpyAsync(out, s->d_adj, sizeof(float) * len, cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    MCXG_TRY(cudaGetLastError());
    return MCXG_OK;
}

int mcxg_adjoint(mcxg_session* s, int kind, uint32_t ns, uint32_t nd, uint32_t nx, uint32_t ny, uint32_t nz,
                 uint32_t maxgate, float* out) {
    if (!s || !out || !s->has_problem || !s->out_valid || ns == 0 || nd == 0 || nx == 0 || ny == 0 || nz == 0 ||
            (unsigned long long)nx * ny * nz * maxgate * (ns + nd) != s->kp.fieldlen) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    return adjoint_run(s, kind, (const float*)s->d_out, ns, nd, nx, ny, nz, maxgate, out);
}

int mcxg_adjoint_field(mcxg_session* s, int kind, const float* field, uint32_t ns, uint32_t nd, uint32_t nx,
                       uint32_t ny, uint32_t nz, uint32_t maxgate, float* out) {
    if (!s || !field || !out || ns == 0 || nd == 0 || nx == 0 || ny == 0 || nz == 0 || maxgate == 0 ||
            (unsigned long long)nx * ny * nz * maxgate * (ns + nd) > 0xFFFFFFFFull) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    const size_t n = (size_t)nx * ny * nz * maxgate * (ns + nd);
    int rc = ensure((float**)&s->d_out, &s->out_cap, n);
    if (rc) {
        return rc;
    }
    s->out_valid = false;
    MCXG_TRY(cudaMemcpyAsync(s->d_out, field, sizeof(float) * n, cudaMemcpyHostToDevice, s->st));
    return adjoint_run(s, kind, (const float*)s->d_out, ns, nd, nx, ny, nz, maxgate, out);
}

int mcxg_get_field_f64(mcxg_session* s, double* out) {
    if (!s || !out || !s->has_problem) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    size_t n = s->kp.fieldlen, total = n * field_comps(s->kp);
    int rc = ensure((double**)&s->d_out, &s->out_cap, total);
    if (rc) {
        return rc;
    }
    field_merge_f64<<<grid_for(s, total), 256, 0, s->st>>>(s->d_field, n, total, (double)s->kp.fxunit,
                                                           (double*)s->d_out);
    s->out_valid = false;
    MCXG_TRY(cudaMemcpyAsync(out, s->d_out, sizeof(double) * total, cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_batch_get_verify(mcxg_session* s, double* f64, double* comp) {
    if (!s || !s->has_batch || !s->d_acc64 || s->acc64_cap < s->totalfield) {
        return MCXG_ERR_STATE;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    const size_t n = s->totalfield;
    if (f64) {
        MCXG_TRY(cudaMemcpyAsync(f64, s->d_acc64, sizeof(double) * n, cudaMemcpyDeviceToHost, s->st));
    }
    if (comp) {
        /* each simulation's elements merged with its own unit, unscaled */
        std::vector<double> ones(s->nsim, 1.0);
        int rc = ensure(&s->d_scales, &s->scales_cap, s->nsim);
        if (!rc) {
            rc = ensure((double**)&s->d_out, &s->out_cap, n);
        }
        if (rc) {
            return rc;
        }
        MCXG_TRY(cudaMemcpyAsync(s->d_scales, ones.data(), sizeof(double) * s->nsim, cudaMemcpyHostToDevice, s->st));
        batch_merge_f64<<<dim3(64, s->nsim), 256, 0, s->st>>>(s->d_bfield, s->totalfield, s->d_sims,
                                                              (double*)s->d_out);
        s->out_valid = false;
        MCXG_TRY(cudaMemcpyAsync(comp, s->d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, s->st));
    }
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_set_adjoint(mcxg_session* s, const float* dloss, uint32_t n) {
    if (!s || !s->has_problem || !dloss || n != s->kp.fieldlen) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    int rc = ensure(&s->d_adjc, &s->adjc_cap, (size_t)n);
    if (!rc) {
        rc = ensure(&s->d_adjJ, &s->adjJ_cap, (size_t)s->kp.nthread * (s->kp.threadphoton + 1u));
    }
    if (rc) {
        return rc;
    }
    MCXG_TRY(cudaMemcpyAsync(s->d_adjc, dloss, sizeof(float) * n, cudaMemcpyHostToDevice, s->st));
    MCXG_TRY(cudaMemsetAsync(s->d_adjJ, 0, sizeof(float) * s->adjJ_cap, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    s->adj_ready = true;
    return MCXG_OK;
}

int mcxg_get_adjoint_grad(mcxg_session* s, float* gmua, float* gmus) {
    if (!s || !s->has_problem || !s->adj_ready) {
        return MCXG_ERR_STATE;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    const size_t nvox = s->kp.nvox, F = s->kp.fieldlen;
    if (gmua) {
        MCXG_TRY(cudaMemcpyAsync(gmua, s->d_field, sizeof(float) * nvox, cudaMemcpyDeviceToHost, s->st));
    }
    if (gmus) {
        MCXG_TRY(cudaMemcpyAsync(gmus, s->d_field + F, sizeof(float) * nvox, cudaMemcpyDeviceToHost, s->st));
    }
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_get_field_planes(mcxg_session* s, int64_t* counts, float* rem) {
    if (!s || !s->has_problem) {
        return MCXG_ERR_STATE;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    const size_t total = (size_t)s->kp.fieldlen * field_comps(s->kp);
    if (counts) {
        MCXG_TRY(cudaMemcpyAsync(counts, s->d_field, sizeof(int64_t) * total, cudaMemcpyDeviceToHost, s->st));
    }
    if (rem) {
        MCXG_TRY(cudaMemcpyAsync(rem, s->d_field + 2 * total, sizeof(float) * total, cudaMemcpyDeviceToHost, s->st));
    }
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_get_verify(mcxg_session* s, double* f64, float* plain, float* spill) {
    if (!s || !s->has_problem || !s->d_acc64 || s->acc64_cap < s->kp.fieldlen) {
        return MCXG_ERR_STATE;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    const size_t n = s->kp.fieldlen;
    if (f64) {
        MCXG_TRY(cudaMemcpyAsync(f64, s->d_acc64, sizeof(double) * n, cudaMemcpyDeviceToHost, s->st));
    }
    if (plain) {
        MCXG_TRY(cudaMemcpyAsync(plain, s->d_accf, sizeof(float) * n, cudaMemcpyDeviceToHost, s->st));
    }
    std::vector<float> raw;
    if (spill) {
        raw.resize(2 * n);
        MCXG_TRY(cudaMemcpyAsync(raw.data(), s->d_accs, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost, s->st));
    }
    MCXG_TRY(cudaStreamSynchronize(s->st));
    if (spill) {
        /* the reference's host merge of the two halves, in float
           (mcx_host.cpp:1252-1257) */
        for (size_t i = 0; i < n; i++) {
            spill[i] = raw[i] + raw[i + n];
        }
    }
    return MCXG_OK;
}

int mcxg_get_detected(mcxg_session* s, float* detp, uint64_t* seeds, uint32_t* detected) {
    if (!s || !s->has_problem) {
        return MCXG_ERR_STATE;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    unsigned int cnt = 0;
    MCXG_TRY(cudaMemcpyAsync(&cnt, s->d_words, sizeof(cnt), cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    if (detected) {
        *detected = cnt;
    }
    if (!s->kp.savedet) {
        return MCXG_OK;
    }
    size_t saved = cnt < s->kp.maxdetphoton ? cnt : s->kp.maxdetphoton;
    if (detp && saved && s->kp.reclen) {
        MCXG_TRY(cudaMemcpyAsync(detp, s->d_detp, sizeof(float) * saved * s->kp.reclen, cudaMemcpyDeviceToHost, s->st));
    }
    if (seeds && saved && s->kp.issaveseed) {
        MCXG_TRY(cudaMemcpyAsync(seeds, s->d_detseed, sizeof(uint64_t) * 2 * saved, cudaMemcpyDeviceToHost, s->st));
    }
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_get_detweight(mcxg_session* s, float* out) {
    if (!s || !out || !s->has_problem) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    unsigned int cnt = 0;
    MCXG_TRY(cudaMemcpyAsync(&cnt, s->d_words, sizeof(cnt), cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    if (!s->kp.savedet) {
        return MCXG_OK;
    }
    size_t saved = cnt < s->kp.maxdetphoton ? cnt : s->kp.maxdetphoton;
    if (saved) {
        MCXG_TRY(cudaMemcpyAsync(out, s->d_detw, sizeof(float2) * saved, cudaMemcpyDeviceToHost, s->st));
        MCXG_TRY(cudaStreamSynchronize(s->st));
    }
    return MCXG_OK;
}

int mcxg_get_counters(mcxg_session* s, uint64_t counters[5], uint32_t status[2]) {
    if (!s) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    unsigned long long ev[8];
    unsigned int w[8];
    MCXG_TRY(cudaMemcpyAsync(ev, s->d_events, sizeof(ev), cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaMemcpyAsync(w, s->d_words, sizeof(w), cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    if (counters) {
        for (int i = 0; i < 5; i++) {
            counters[i] = ev[i];
        }
    }
    if (status) {
        status[0] = w[2];
        status[1] = w[3];
    }
    return MCXG_OK;
}

int mcxg_fp32_peak(mcxg_session* s, double* gops) {
    if (!s || !gops) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    /* ~0.25 s per repetition at full clock: long enough to time, short
       enough that the power limit does not pull the clock down */
    const int block = 256, iters = 1 << 12;
    const int grid = s->info.sm * 8;
    float best = 1e30f;
    for (int rep = 0; rep < 12; rep++) {
        MCXG_TRY(cudaEventRecord(s->e0, s->st));
        fma_peak<<<grid, block, 0, s->st>>>((float*)s->d_red, iters, 0.999999f, 1e-7f);
        MCXG_TRY(cudaEventRecord(s->e1, s->st));
        MCXG_TRY(cudaStreamSynchronize(s->st));
        MCXG_TRY(cudaGetLastError());
        float ms = 0.f;
        MCXG_TRY(cudaEventElapsedTime(&ms, s->e0, s->e1));
        if (rep > 0 && ms < best) {
            best = ms;
        }
    }
    *gops = (double)grid * block * iters * 8.0 / (best * 1e-3) / 1e9;
    return MCXG_OK;
}


/* ---- batch of simulations ---------------------------------------------------
 *
 * Many independent simulations share one persistent launch.  Their volumes,
 * fields and property rows are concatenated; each simulation's descriptor
 * (parameter block + offsets) sits in global memory and the threads claim
 * reference threads from one counter over the concatenated numbering, so a
 * simulation of 1e5 photons does not leave the GPU idle at the end of its
 * own launch, and many small simulations cost one launch.
 */
namespace {

int batch_reset_graph(mcxg_session* s) {
    if (s->bgraph_exec) {
        cudaGraphExecDestroy(s->bgraph_exec);
        s->bgraph_exec = nullptr;
    }
    if (s->bgraph) {
        cudaGraphDestroy(s->bgraph);
        s->bgraph = nullptr;
    }
    return MCXG_OK;
}

/* the work of one batch run, on s->st: clear; per wave of simulations, their
   descriptors into constant memory and the transport launch; per-simulation
   sums */
int batch_enqueue(mcxg_session* s, int lflags) {
    MCXG_TRY(cudaMemsetAsync(s->d_bfield, 0, sizeof(float) * kFieldPlanes * (size_t)s->totalfield, s->st));
    if (lflags & mcxg::LF_ACC64) {
        const size_t n = s->totalfield;
        MCXG_TRY(cudaMemsetAsync(s->d_acc64, 0, sizeof(double) * n, s->st));
        MCXG_TRY(cudaMemsetAsync(s->d_accf, 0, sizeof(float) * n, s->st));
        MCXG_TRY(cudaMemsetAsync(s->d_accs, 0, sizeof(float) * 2 * n, s->st));
    }
    MCXG_TRY(cudaMemsetAsync(s->d_benergy, 0, sizeof(float2) * (size_t)s->totalvt, s->st));
    MCXG_TRY(cudaMemsetAsync(s->d_words, 0, 8 * sizeof(unsigned int), s->st));
    KArgs a;
    memset(&a, 0, sizeof(a));
    a.media8 = s->d_bmedia;
    a.media32 = (const uint32_t*)s->d_bmedia;
    a.field = s->d_bfield;
    a.fhi = reinterpret_cast<unsigned long long*>(s->d_bfield);
    a.flo = s->d_bfield + 2 * (size_t)s->totalfield;
    a.energy = s->d_benergy;
    a.detcount = s->d_words + 0;
    a.vtcounter = s->d_words + 1;
    a.status = s->d_words + 2;
    a.counters = s->d_events;
    a.lo = (unsigned int)s->totalfield;
    if (lflags & mcxg::LF_ACC64) {
        a.acc64 = s->d_acc64;
        a.accf = s->d_accf;
        a.accs = s->d_accs;
    }
    MCXG_TRY(cudaMemsetAsync(s->d_simctr, 0, sizeof(unsigned int) * s->nsim, s->st));
    for (uint32_t w0 = 0; w0 < s->nsim; w0 += mcxg::kBatchWave) {
        const uint32_t n = std::min<uint32_t>(mcxg::kBatchWave, s->nsim - w0);
        MCXG_TRY(mcxg::batch_wave_upload(s->d_sims + w0, n, s->st));
        MCXG_TRY(cudaMemsetAsync(s->d_words + 1, 0, sizeof(unsigned int), s->st));
        a.simctr = s->d_simctr + w0;
        a.nsim = n;
        MCXG_TRY(mcxg::batch_launch(a, lflags, s->bt_grid, s->bt_block, (size_t)s->bt_block * 32, s->st));
    }
    batch_energy<<<s->nsim, 256, 0, s->st>>>(s->d_benergy, s->d_sims, s->d_bsum);
    return MCXG_OK;
}

}  // namespace

namespace {
/* The checks and buffers of a batch (the simulations' reference threads must
   number 0.. contiguously, and every offset must stay inside the buffers
   given), then its upload: the volume as bytes, or as each simulation's
   32-bit label words packed on the device. */
int batch_upload(mcxg_session* s, const mcxg_simdesc* sims, uint32_t nsim, const uint8_t* media,
                 const uint32_t* const* words, uint64_t nmedia) {
    std::vector<unsigned long long> simvt(nsim + 1);
    unsigned long long vt = 0, field = 0;
    for (uint32_t i = 0; i < nsim; i++) {
        const mcxg_simdesc& d = sims[i];
        if (d.vt_off != vt || d.kp.nthread == 0 || d.kp.mediaword != 1 || d.kp.savedet || d.kp.replay ||
                d.kp.extrasrclen || d.kp.nphase || d.kp.nangle || d.kp.npattern || d.kp.mediaformat > 4 ||
                d.kp.medianum > MCXG_BATCH_MAXMEDIA || d.media_off + d.kp.nvox > nmedia ||
                (unsigned long long)d.kp.threadphoton * d.kp.nthread + (unsigned int)d.kp.oddphoton == 0 ||
                (words && !words[i])) {
            return MCXG_ERR_ARG;
        }
        simvt[i] = vt;
        vt += d.kp.nthread;
        field = std::max(field, (unsigned long long)d.field_off + d.kp.fieldlen);
    }
    simvt[nsim] = vt;
    if (vt >= 0xFFFFFFFFull - 65536ull * 1024 || 2 * field >= 0xFFFFFFFFull) {
        return MCXG_ERR_LIMIT;          /* 32-bit thread counter and field indices */
    }
    MCXG_TRY(cudaSetDevice(s->device));
    int rc = ensure(&s->d_sims, &s->sims_cap, nsim);
    if (!rc) {
        rc = ensure(&s->d_simvt, &s->simvt_cap, (size_t)nsim + 1);
    }
    if (!rc) {
        rc = ensure(&s->d_simctr, &s->simctr_cap, (size_t)nsim);
    }
    if (!rc) {
        rc = ensure(&s->d_bmedia, &s->bmedia_cap, (size_t)nmedia);
    }
    if (!rc && words) {
        rc = ensure(&s->d_words32, &s->words32_cap, (size_t)nmedia);
    }
    if (!rc) {
        rc = ensure(&s->d_bfield, &s->bfield_cap, kFieldPlanes * (size_t)field);
    }
    if (!rc) {
        rc = ensure(&s->d_benergy, &s->benergy_cap, (size_t)vt);
    }
    if (!rc) {
        rc = ensure(&s->d_bsum, &s->bsum_cap, 2 * (size_t)nsim);
    }
    if (rc) {
        return rc;
    }
    MCXG_TRY(cudaMemcpyAsync(s->d_sims, sims, sizeof(mcxg_simdesc) * nsim, cudaMemcpyHostToDevice, s->st));
    MCXG_TRY(cudaMemcpyAsync(s->d_simvt, simvt.data(), sizeof(unsigned long long) * (nsim + 1), cudaMemcpyHostToDevice,
                             s->st));
    if (words) {
        for (uint32_t i = 0; i < nsim; i++) {
            MCXG_TRY(cudaMemcpyAsync(s->d_words32 + sims[i].media_off, words[i], sizeof(uint32_t) * (size_t)sims[i].kp.nvox,
                                     cudaMemcpyHostToDevice, s->st));
        }
        /* a batch saves no detected photons: the label alone, as the byte upload takes it */
        pack_labels<<<grid_for(s, (size_t)nmedia), 256, 0, s->st>>>(s->d_words32, (size_t)nmedia, 0x7Fu,
                                                                     (uint8_t*)s->d_bmedia);
        MCXG_TRY(cudaGetLastError());
    } else {
        MCXG_TRY(cudaMemcpyAsync(s->d_bmedia, media, (size_t)nmedia, cudaMemcpyHostToDevice, s->st));
    }
    batch_recip<<<grid_for(s, (size_t)nsim * MCXG_BATCH_MAXMEDIA), 256, 0, s->st>>>(s->d_sims, nsim);
    MCXG_TRY(cudaStreamSynchronize(s->st));
    MCXG_TRY(cudaGetLastError());
    s->h_sims.assign(sims, sims + nsim);
    s->h_simvt = simvt;
    s->nsim = nsim;
    s->totalvt = vt;
    s->totalfield = field;
    s->has_batch = true;
    return batch_reset_graph(s);
}
}  // namespace

int mcxg_batch_set(mcxg_session* s, const void* sims, size_t desc_size, uint32_t nsim, const uint8_t* media,
                   uint64_t nmedia) {
    if (!s || !sims || desc_size != sizeof(mcxg_simdesc) || nsim == 0 || !media) {
        return MCXG_ERR_ARG;
    }
    return batch_upload(s, (const mcxg_simdesc*)sims, nsim, media, nullptr, nmedia);
}

int mcxg_batch_set_words(mcxg_session* s, const void* sims, size_t desc_size, uint32_t nsim,
                         const uint32_t* const* words, uint64_t nmedia) {
    if (!s || !sims || desc_size != sizeof(mcxg_simdesc) || nsim == 0 || !words) {
        return MCXG_ERR_ARG;
    }
    return batch_upload(s, (const mcxg_simdesc*)sims, nsim, nullptr, words, nmedia);
}

int mcxg_batch_simulate(mcxg_session* s, unsigned int flags, float* kernel_ms) {
    if (!s) {
        return MCXG_ERR_ARG;
    }
    if (!s->has_batch) {
        return MCXG_ERR_STATE;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    bool refl = false, common = true;
    for (const mcxg_simdesc& d : s->h_sims) {
        refl = refl || d.kp.dorefl_compiled;
        common = common && !d.kp.is2d && d.kp.mediaformat <= 4 && d.kp.nphase <= 2;
    }
    const bool verify = (flags & MCXG_VERIFY) != 0;
    if (verify) {
        /* the precision check: every deposit also to FP64, plain float and
           spill fields of the whole batch (not captured in a graph) */
        if (flags & MCXG_GRAPH) {
            return MCXG_ERR_ARG;
        }
        const size_t n = s->totalfield;
        int rc = ensure(&s->d_acc64, &s->acc64_cap, n);
        if (!rc) {
            rc = ensure(&s->d_accf, &s->accf_cap, n);
        }
        if (!rc) {
            rc = ensure(&s->d_accs, &s->accs_cap, 2 * n);
        }
        if (rc) {
            return rc;
        }
    }
    const bool agg = (flags & MCXG_AGG) != 0 && !verify;
    /* 4 blocks of 256 a SM on the 64-register instantiation; the precision
       check's instantiation is capped at 80 (3 blocks) */
    const int bpsm_req = verify ? 3 : (s->bpsm_req ? s->bpsm_req : 4);
    int lflags = (refl ? mcxg::LF_REFL : 0) | (agg ? mcxg::LF_WAGG : 0) | (bpsm_req >= 3 ? mcxg::LF_CAPPED : 0) |
                 (common && !(flags & MCXG_GENERAL) ? mcxg::LF_COMMON : 0) | (verify ? mcxg::LF_ACC64 : 0);
    int block = s->block_req ? s->block_req : 256;
    int occ = 0;
    MCXG_TRY(mcxg::batch_occupancy(lflags, block, (size_t)block * 32, &occ));
    int bpsm = std::max(1, std::min(bpsm_req, occ > 0 ? occ : bpsm_req));
    const int grid = s->info.sm * bpsm;
    if (grid != s->bt_grid || block != s->bt_block) {
        batch_reset_graph(s);
    }
    s->bt_grid = grid;
    s->bt_block = block;
    s->grid = grid;
    s->block = block;

    if (flags & MCXG_GRAPH) {
        /* the clear + transport + sums sequence, captured once and replayed */
        if (!s->bgraph_exec) {
            MCXG_TRY(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
            int rc = batch_enqueue(s, lflags);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(s->st, &g);
            if (rc) {
                if (g) {
                    cudaGraphDestroy(g);
                }
                return rc;
            }
            MCXG_TRY(e);
            s->bgraph = g;
            MCXG_TRY(cudaGraphInstantiate(&s->bgraph_exec, g, 0));
        }
        MCXG_TRY(cudaEventRecord(s->e0, s->st));
        MCXG_TRY(cudaGraphLaunch(s->bgraph_exec, s->st));
        MCXG_TRY(cudaEventRecord(s->e1, s->st));
    } else {
        MCXG_TRY(cudaEventRecord(s->e0, s->st));
        int rc = batch_enqueue(s, lflags);
        if (rc) {
            return rc;
        }
        MCXG_TRY(cudaEventRecord(s->e1, s->st));
    }
    MCXG_TRY(cudaStreamSynchronize(s->st));
    MCXG_TRY(cudaGetLastError());
    if (kernel_ms) {
        float ms = 0.f;
        MCXG_TRY(cudaEventElapsedTime(&ms, s->e0, s->e1));
        *kernel_ms = ms;
    }
    return MCXG_OK;
}

int mcxg_batch_get_energy(mcxg_session* s, double* out) {
    if (!s || !out || !s->has_batch) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    MCXG_TRY(cudaMemcpyAsync(out, s->d_bsum, sizeof(double) * 2 * s->nsim, cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    return MCXG_OK;
}

int mcxg_batch_get_field(mcxg_session* s, float* out, const double* scales) {
    if (!s || !out || !scales || !s->has_batch) {
        return MCXG_ERR_ARG;
    }
    MCXG_TRY(cudaSetDevice(s->device));
    int rc = ensure(&s->d_bout, &s->bout_cap, (size_t)s->totalfield);
    if (!rc) {
        rc = ensure(&s->d_scales, &s->scales_cap, s->nsim);
    }
    if (rc) {
        return rc;
    }
    MCXG_TRY(cudaMemcpyAsync(s->d_scales, scales, sizeof(double) * s->nsim, cudaMemcpyHostToDevice, s->st));
    MCXG_TRY(cudaMemsetAsync(s->d_bout, 0, sizeof(float) * (size_t)s->totalfield, s->st));
    batch_merge<<<dim3(64, s->nsim), 256, 0, s->st>>>(s->d_bfield, s->totalfield, s->d_sims, s->d_scales, s->d_bout);
    MCXG_TRY(cudaMemcpyAsync(out, s->d_bout, sizeof(float) * (size_t)s->totalfield, cudaMemcpyDeviceToHost, s->st));
    MCXG_TRY(cudaStreamSynchronize(s->st));
    MCXG_TRY(cudaGetLastError());
    return MCXG_OK;
}

/* ---- allocation-free FP64 energy sum ---------------------------------------
 *
 * For callers that cannot let this library allocate device memory: a service
 * that reserves its whole device budget at start-up, or a host framework that
 * owns every device buffer and only lends the library pointers into them.
 * mcxg_get_energy needs a session, and a session allocates its buffers with
 * cudaMalloc; this entry point reduces a caller-owned array of per-thread
 * {escaped, launched} weights with no allocation at all.  Its scratch -- one
 * {escaped, launched} FP64 pair per block of 2048 threads, plus the result --
 * is the static device array below, sized for MCXG_NOALLOC_MAX_THREADS
 * threads (64 KB on every GPU that loads the library, held until exit).
 */
#define MCXG_NOALLOC_CHUNK        2048u
#define MCXG_NOALLOC_MAX_BLOCKS   4096u
#define MCXG_NOALLOC_MAX_DEVICES  64

static __device__ __align__(256) double g_noalloc_scratch[2 * MCXG_NOALLOC_MAX_BLOCKS + 2];
static double* g_noalloc_scratch_addr[MCXG_NOALLOC_MAX_DEVICES];

static int energy_sum_noalloc_on(int device, const float* d_energy, uint32_t nthread, uint32_t nblocks,
                                 double* d_sums) {
    if (!g_noalloc_scratch_addr[device]) {
        /* once per device, with that device current: the device address of the
           static array (its host-side name is not a device address) */
        void* p = nullptr;
        MCXG_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_scratch_addr[device] = (double*)p;
    }
    double* scratch = g_noalloc_scratch_addr[device];
    /* the array keeps the previous call's contents: clear the part this call uses */
    MCXG_TRY(cudaMemsetAsync(scratch, 0, sizeof(double) * (2 * (size_t)nblocks + 2), 0));
    energy_partials<<<nblocks, kRedThreads, 0, 0>>>((const float2*)d_energy, nthread, scratch);
    MCXG_TRY(cudaGetLastError());
    energy_final<<<1, 32, 0, 0>>>(scratch, (int)nblocks);
    MCXG_TRY(cudaGetLastError());
    MCXG_TRY(cudaMemcpyAsync(d_sums, scratch + 2 * nblocks, 2 * sizeof(double), cudaMemcpyDeviceToDevice, 0));
    MCXG_TRY(cudaStreamSynchronize(0));
    return MCXG_OK;
}

int mcxg_energy_sum_noalloc(int device, const float* d_energy, uint32_t nthread, double* d_sums) {
    if (!d_energy || !d_sums || nthread == 0 || device < 0 || device >= MCXG_NOALLOC_MAX_DEVICES) {
        return MCXG_ERR_ARG;
    }
    uint32_t nblocks = (nthread + MCXG_NOALLOC_CHUNK - 1) / MCXG_NOALLOC_CHUNK;
    if (nblocks > MCXG_NOALLOC_MAX_BLOCKS) {
        return MCXG_ERR_LIMIT;
    }
    /* run on `device`, then give the calling thread its current device back */
    int prev = 0;
    MCXG_TRY(cudaGetDevice(&prev));
    MCXG_TRY(cudaSetDevice(device));
    const int rc = energy_sum_noalloc_on(device, d_energy, nthread, nblocks, d_sums);
    const cudaError_t e = cudaSetDevice(prev);
    return rc != MCXG_OK ? rc : (e == cudaSuccess ? MCXG_OK : MCXG_ERR_CUDA);
}

int mcxg_get_launch(mcxg_session* s, int* grid, int* block, int* regs) {
    if (!s) {
        return MCXG_ERR_ARG;
    }
    if (grid) {
        *grid = s->grid;
    }
    if (block) {
        *block = s->block;
    }
    if (regs) {
        *regs = s->regs;
    }
    return MCXG_OK;
}

}  // extern "C"
