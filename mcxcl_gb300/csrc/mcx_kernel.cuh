/*
 * mcx_kernel.cuh -- the GB300 photon-transport kernel.
 *
 * Replaces the reference's mcx_main_loop (src/mcx_core.cl:2307-3307) and its
 * launchnewphoton (1463-2275).  The physics, its branch structure and the
 * order of floating-point operations follow the reference's OpenCL branch so
 * that, in the exact instantiation, a photon's path is the same bits as in
 * the CPU oracle; the GPU-specific structure is new:
 *
 *  - Persistent threads.  The reference assigns one RNG stream ("reference
 *    thread", vt) per OpenCL work item.  Here each GPU thread repeatedly
 *    claims the next vt from a global counter and runs all of its photons,
 *    so results do not depend on the launch shape and long-lived photons do
 *    not leave the rest of a warp idle at the end of the grid.
 *  - One launch site.  Every photon termination (exit, time-out, roulette,
 *    transmission into air) sets a relaunch request handled at the top of the
 *    step loop, so the large source-sampling code is instantiated once.
 *  - Parameters in constant memory, optical properties and inverse-CDF tables
 *    staged in shared memory (label lookups diverge across a warp), the label
 *    volume as one byte per voxel (label | detector bit << 7) read through
 *    the read-only path.
 *  - Fluence accumulated exactly: each deposit splits into a 64-bit
 *    fixed-point part (integer atomics, exact in any order) and a tiny float
 *    remainder.  Deposits to the same voxel and gate by several lanes of a
 *    warp can be merged first (match, shuffle-sum, one leader commit).
 *  - Detected-photon partial data in shared memory, strided per thread.
 *
 * Template flags: EXACT (IEEE-only math, no contraction: compile this TU with
 * -fmad=false -prec-div=true -prec-sqrt=true -ftz=false), DET (detector
 * bookkeeping compiled in), REFL (Fresnel / boundary-condition block
 * compiled in), WAGG (warp aggregation of deposits), COUNT (event counters),
 * MINB (resident 256-thread blocks per SM the register allocation targets),
 * ACC64 (every deposit also accumulated in FP64, plain float and the
 * reference's spill form, to state the accumulation error), ADJ (the two
 * passes of the fluence gradient instead of the deposits).
 * DET and REFL are upper bounds: the runtime flags in the constant block
 * still decide, so the exact build runs every configuration.
 */
#ifndef MCX_KERNEL_CUH
#define MCX_KERNEL_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include <cuda_fp16.h>

#include <type_traits>

#include "mcx_kparams.h"
#include "mcx_launch.h"
#include "mcx_pmath.cuh"

namespace mcxg {
/* each kernel translation unit gets its own copy (internal linkage): the two
   units are compiled with different floating-point flags */
namespace {

#define K_EPS            1.19209290E-07F
#define K_VERY_BIG       (1.f / K_EPS)
#define K_ONE_PI         3.1415926535897932f
#define K_TWO_PI         6.28318530717959f
#define K_R_PI           0.318309886183791f
#define K_NANGLES        181            /* polar angles of the Mueller tables */
#define K_JUST_BELOW_ONE 0.9998f
#define K_MAX_ACCUM      1000.f
#define K_ROULETTE       10.f
#define K_OUT_MIN        0xFFFFFFFFu
#define K_OUT_MAX        0x7FFFFFFFu
#define K_DET_MASK       0x80000000u
#define K_MED_MASK       0x7FFFFFFFu
#define K_LAUNCH_CAP     (1u << 16)     /* launch attempts per photon before giving up */
#define K_STEP_CAP       (1u << 27)     /* propagation steps per photon before it is dropped */
#define K_CONE_CAP       (1u << 16)     /* rejection draws of the cone source */

enum { bcUnknown, bcReflect, bcAbsorb, bcMirror, bcCyclic };
enum { otFlux, otFluence, otEnergy, otJacobian, otWP, otDCS, otRF, otL, otRFmus, otWLTOF, otWPTOF, otAdjoint };
enum { S_PENCIL, S_ISOTROPIC, S_CONE, S_GAUSSIAN, S_PLANAR, S_PATTERN, S_FOURIER, S_ARCSINE,
       S_DISK, S_FOURIERX, S_FOURIERX2D, S_ZGAUSSIAN, S_LINE, S_SLIT, S_PENCILARRAY, S_PATTERN3D,
       S_HYPERBOLOID, S_RING };

#define SAVE_DETID(a) ((a) & 0x1)
#define SAVE_NSCAT(a) ((a) >> 1 & 0x1)
#define SAVE_PPATH(a) ((a) >> 2 & 0x1)
#define SAVE_MOM(a)   ((a) >> 3 & 0x1)
#define SAVE_PEXIT(a) ((a) >> 4 & 0x1)
#define SAVE_VEXIT(a) ((a) >> 5 & 0x1)
#define SAVE_W0(a)    ((a) >> 6 & 0x1)
#define SAVE_IQUV(a)  ((a) >> 7 & 0x1)

/* status words written by the kernel */
#define ST_FAILED_LAUNCH 0   /* reference threads whose launch failed (NO_LAUNCH) */
#define ST_GUARD         1   /* photons stopped by a safety cap (steps, cone draws) or an index guard */

__constant__ mcxg_kparams c_p;
#ifdef MCXG_BATCH_TU
/* the batch translation unit spends its constant bank on the descriptors of
   the simulations of one wave; batches have no detectors or extra sources */
#define MCXG_BATCH_WAVE 136
__constant__ float4 c_det[1];
__constant__ float4 c_srcx[4];
__constant__ mcxg_simdesc c_sims[MCXG_BATCH_WAVE];
#else
__constant__ float4 c_det[MCXG_MAX_DET];
__constant__ float4 c_srcx[MCXG_MAX_EXTRASRC * 4];
__constant__ mcxg_simdesc c_sims[1];
#endif



/* Per-thread state written at a launch and read only at a detection or at
   the end of the reference thread: kept in shared memory, out of the
   registers of the step loop. */
struct ColdState {
    unsigned long long ps0, ps1;   /* RNG state at launch, saved with detected photons */
    float esc, launched, w0init, srcsel;   /* reference ppath[partialdata .. +3] */
};

/* Per-thread view of the tables.  A single simulation stages them in shared
   memory at fixed offsets, so their addresses are recomputed where used
   instead of held in registers; a batch reads the rows of the thread's
   current simulation from global memory through these two pointers. */
struct Shared {
    const float4* bprop;           /* batch: property rows of the current simulation */
    const float4* brecip;          /* batch: their reciprocals */
};


extern __shared__ float4 mcxg_smem[];

/* --------------------------------------------------------- parameter source
 *
 * Where the kernel reads its parameters.  One simulation keeps them in
 * constant memory (ConstPS).  A batch of simulations (BatchPST) keeps one
 * descriptor per simulation in constant memory -- the parameter block, the
 * simulation's offsets into the batch's volume, field and reference-thread
 * numbering, its seed and property rows -- and each thread follows the
 * descriptor of the reference thread it is running.  Every device function that reads a
 * parameter takes the source and binds `c_p` to it locally, so the physics
 * code is the same text for both.
 */
template <bool XMEDIA, bool COMMON = false>
struct ConstPST {
    static constexpr bool kBatch = false;
    static constexpr bool kXMedia = XMEDIA;   /* decode the encodings beyond labels and float mua */
    static constexpr bool kCommon = COMMON;   /* the common configuration (KP_* below) */
    __device__ __forceinline__ void init(const KArgs&) {}
    __device__ __forceinline__ const mcxg_kparams& p() const { return c_p; }
    __device__ __forceinline__ const float4* det() const { return c_det; }
    __device__ __forceinline__ const float4* srcx() const { return c_srcx; }
    __device__ __forceinline__ unsigned long long media_off() const { return 0ull; }
    __device__ __forceinline__ unsigned int field_off() const { return 0u; }
    __device__ __forceinline__ unsigned int lo_plane() const { return c_p.fieldlen; }
    __device__ __forceinline__ unsigned long long vt_off() const { return 0ull; }
    __device__ __forceinline__ unsigned int prop_off() const { return 0u; }
    __device__ __forceinline__ unsigned long long seed() const { return 0ull; }
    /* shared layout: prop[medianum], recip[medianum] (float4), ColdState[blockDim],
       invcdf[nphase], angleinvcdf[nangle], partial data[partialdata][blockDim] */
    __device__ __forceinline__ const float4& prop(const Shared&, unsigned int i) const { return mcxg_smem[i]; }
    __device__ __forceinline__ const float4& recip(const Shared&, unsigned int i) const {
        return mcxg_smem[c_p.medianum + i];
    }
    __device__ __forceinline__ ColdState* cold() const {
        return (ColdState*)(mcxg_smem + 2 * c_p.medianum) + threadIdx.x;
    }
    __device__ __forceinline__ float* tables() const {
        return (float*)((ColdState*)(mcxg_smem + 2 * c_p.medianum) + blockDim.x);
    }
    __device__ __forceinline__ float invcdf(unsigned int i) const { return tables()[i]; }
    __device__ __forceinline__ float angle(unsigned int i) const { return tables()[c_p.nphase + i]; }
    __device__ __forceinline__ float& pp(unsigned int slot) const {
        return tables()[c_p.nphase + c_p.nangle + slot * blockDim.x + threadIdx.x];
    }
};

using ConstPS = ConstPST<false>;

template <bool COMMON>
struct BatchPST {
    static constexpr bool kBatch = true;
    static constexpr bool kXMedia = false;
    static constexpr bool kCommon = COMMON;   /* every simulation of the wave is 3-D */
    unsigned int sid;              /* the simulation of this wave the thread is running */
    unsigned int lo;               /* low-plane offset: the batch's total field length */
    __device__ __forceinline__ void init(const KArgs& a) {
        sid = 0;
        lo = a.lo;
    }
    __device__ __forceinline__ const mcxg_kparams& p() const { return c_sims[sid].kp; }
    __device__ __forceinline__ const float4* det() const { return c_det; }   /* batches save no detectors */
    __device__ __forceinline__ const float4* srcx() const { return c_srcx; } /* nor use extra sources */
    __device__ __forceinline__ unsigned long long media_off() const { return c_sims[sid].media_off; }
    __device__ __forceinline__ unsigned int field_off() const { return (unsigned int)c_sims[sid].field_off; }
    __device__ __forceinline__ unsigned int lo_plane() const { return lo; }
    __device__ __forceinline__ unsigned long long vt_off() const { return c_sims[sid].vt_off; }
    __device__ __forceinline__ unsigned int prop_off() const { return 0u; }
    __device__ __forceinline__ unsigned long long seed() const { return c_sims[sid].seed; }
    /* shared layout: ColdState[blockDim]; batches have no phase tables or detectors */
    __device__ __forceinline__ float4 prop(const Shared&, unsigned int i) const {
        const mcxg_float4& q = c_sims[sid].prop[i];
        return make_float4(q.x, q.y, q.z, q.w);
    }
    __device__ __forceinline__ float4 recip(const Shared&, unsigned int i) const {
        const mcxg_float4& q = c_sims[sid].recip[i];
        return make_float4(q.x, q.y, q.z, q.w);
    }
    __device__ __forceinline__ ColdState* cold() const { return (ColdState*)mcxg_smem + threadIdx.x; }
    __device__ __forceinline__ float* tables() const { return (float*)((ColdState*)mcxg_smem + blockDim.x); }
    __device__ __forceinline__ float invcdf(unsigned int i) const { return tables()[i]; }
    __device__ __forceinline__ float angle(unsigned int i) const { return tables()[i]; }
    __device__ __forceinline__ float& pp(unsigned int slot) const { return tables()[slot * blockDim.x + threadIdx.x]; }
};

/* Parameters that the common-configuration instantiations fix at compile
   time: label volumes (media format 1, 2 or 4), a 3-D domain and the
   Henyey-Greenstein phase function.  These describe the medium, so a run and
   the replay of its detected photons always take the same instantiation and
   follow the same arithmetic.  The host selects the common instantiations
   only for a configuration that has all three; the others read the parameter
   block.  Used inside functions templated on the parameter source `PS` that
   bind `c_p`. */
#define KP_IS2D (PS::kCommon ? 0u : c_p.is2d)
#define KP_NPHASE_GT2 (!PS::kCommon && c_p.nphase > 2)
#define KP_MEDIAFORMAT (PS::kCommon ? 1u : c_p.mediaformat)
#define KP_SHARING (!PS::kCommon && c_p.srcnum > 1)
/* frequency-domain transport (complex photon weights) in the instantiations
   compiled with it; the rf / rfmus replay outputs in every one that replays */
#define KP_RFFWD (RF && c_p.omega > 0.f && !c_p.replay)
#define KP_RFREPLAY (c_p.replay && (c_p.outputtype == otRF || c_p.outputtype == otRFmus))
/* polarised transport in the instantiations compiled with it */
#define KP_POL (POL && a.maxpol > 0u)
/* split-voxel volumes (MEDIA_2LABEL_SPLIT) in the instantiations compiled with them */
#define KP_SVMC (SVMC && c_p.mediaformat == 97u)

/* ------------------------------------------------------------------ math */

template <bool EXACT> struct Mth;

template <> struct Mth<true> {
    static __device__ __forceinline__ float log(float x) { return pm_logf(x); }
    static __device__ __forceinline__ float exp(float x) { return pm_expf(x); }
    static __device__ __forceinline__ void sincos(float x, float* s, float* c) { pm_sincosf(x, s, c); }
    static __device__ __forceinline__ float sin(float x) { return pm_sinf(x); }
    static __device__ __forceinline__ float cos(float x) { return pm_cosf(x); }
    static __device__ __forceinline__ float acos(float x) { return pm_acosf(x); }
    static __device__ __forceinline__ float rsqrt(float x) { return 1.f / sqrtf(x); }
    static __device__ __forceinline__ float div(float a, float b) { return a / b; }
    static __device__ __forceinline__ float sqrt(float x) { return sqrtf(x); }
};

template <> struct Mth<false> {
    static __device__ __forceinline__ float log(float x) { return __logf(x); }
    static __device__ __forceinline__ float exp(float x) { return __expf(x); }
    static __device__ __forceinline__ void sincos(float x, float* s, float* c) { __sincosf(x, s, c); }
    static __device__ __forceinline__ float sin(float x) { return __sinf(x); }
    static __device__ __forceinline__ float cos(float x) { return __cosf(x); }
    static __device__ __forceinline__ float acos(float x) { return acosf(x); }
    static __device__ __forceinline__ float rsqrt(float x) { return rsqrtf(x); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
    static __device__ __forceinline__ float sqrt(float x) { return sqrtf(x); }
};

/* xorshift128+ (mcx_core.cl:684-698): 64-bit state pair, the low word of the
   sum fills a float mantissa in [1,2) */
struct Rng {
    unsigned long long a, b;
};

__device__ __forceinline__ float rnd(Rng& t) {
    unsigned long long s1 = t.a;
    const unsigned long long s0 = t.b;
    t.a = s0;
    s1 ^= s1 << 23;
    t.b = s1 ^ s0 ^ (s1 >> 18) ^ (s0 >> 5);
    unsigned int r = (unsigned int)(t.b + s0);
    return __fsub_rn(__uint_as_float(0x3F800000u | (r >> 9)), 1.0f);
}

template <bool EXACT>
__device__ __forceinline__ float rnd_scatlen(Rng& t) {
    return -Mth<EXACT>::log(rnd(t) + K_EPS);
}

/* mcx_core.cl:965-973 */
__device__ __forceinline__ float nextafter_ref(float a, int dir) {
    unsigned int i = __float_as_uint(a + 1000.f);
    i += (unsigned int)dir ^ (i & 0x80000000U);
    return __uint_as_float(i) - 1000.f;
}

__device__ __forceinline__ float4 f4(const mcxg_float4& q) {
    return make_float4(q.x, q.y, q.z, q.w);
}

/* ----------------------------------------------------------- photon state */

struct Photon {
    float4 p, v, f, prop;
    int fx, fy, fz, fw;            /* voxel index and last crossed face (the reference's short4 flipdir) */
    unsigned int idx1d, mediaid, isdet;
    float w0, Lmove, pathlen, n1;
    Rng t;
    float wre, wim, w0re, w0im;    /* RF transport: complex weight now and at the last voxel change */
    float4 st;                     /* polarised transport: Stokes vector {I, Q, U, V} */
    float3 nv;                     /* split voxel: plane normal, pointing away from the photon's side */
    float pd;                      /* and the plane's offset along it */
    unsigned int sv;               /* lower and upper label, split and side bits */
};

/* split-voxel state (mcx_core.cl:577-587) */
#define SV_LOWER(sv)     ((sv) & 0xFFu)
#define SV_UPPER(sv)     (((sv) >> 8) & 0xFFu)
#define SV_ISSPLIT(sv)   (((sv) >> 16) & 1u)
#define SV_ISUPPER(sv)   (((sv) >> 17) & 1u)
#define SV_CURLABEL(sv)  (SV_ISUPPER(sv) ? SV_UPPER(sv) : SV_LOWER(sv))

template <class PS>
__device__ __forceinline__ unsigned int media_at(const KArgs& a, const PS& ps, unsigned int idx) {
    const mcxg_kparams& c_p = ps.p();
    const unsigned long long i = ps.media_off() + idx;
    if (c_p.mediaword == 1) {
        unsigned int m = __ldg(a.media8 + i);
        return (m & 0x7Fu) | ((m & 0x80u) << 24);
    }
    return __ldg(a.media32 + i);
}

/* the less common encodings of updateproperty (mcx_core.cl:1099-1187),
   compiled only into the instantiations that take them */
template <class PS>
__device__ __forceinline__ void media_other(const PS& ps, const Shared& S, float4& prop, unsigned int w) {
    const mcxg_kparams& c_p = ps.p();
    if (c_p.mediaformat == 100 || c_p.mediaformat == 102) {
        prop.x = fabsf(__half2float(__ushort_as_half((unsigned short)(w & 0xFFFFu))));
        prop.y = fabsf(__half2float(__ushort_as_half((unsigned short)(w >> 16))));
        prop.w = ps.prop(S, (!w) == 0).w;
    } else if (c_p.mediaformat == 99) {
        prop = ps.prop(S, w & 0x3FFFu);
        const float v = fabsf(__half2float(__ushort_as_half((unsigned short)(w >> 16))));
        const unsigned int k = (w & 0xC000u) >> 14;
        prop.x = (k == 0) ? v : prop.x;
        prop.y = (k == 1) ? v : prop.y;
        prop.z = (k == 2) ? v : prop.z;
        prop.w = (k == 3) ? v : prop.w;
    } else if (c_p.mediaformat == 103) {
        const float4 a = ps.prop(S, 1), b = ps.prop(S, 2);
        prop.x = (float)(w & 0xFFu) * (1.f / 255.f) * (b.x - a.x) + a.x;
        prop.y = (float)((w >> 8) & 0xFFu) * (1.f / 255.f) * (b.y - a.y) + a.y;
        prop.z = (float)((w >> 16) & 0xFFu) * (1.f / 255.f) * (b.z - a.z) + a.z;
        prop.w = (float)(w >> 24) * (1.f / 127.f) * (b.w - a.w) + a.w;
    } else if (c_p.mediaformat == 104) {
        const float4 a = ps.prop(S, 1), b = ps.prop(S, 2);
        prop.x = (float)(w & 0xFFFFu) * (1.f / 65535.f) * (b.x - a.x) + a.x;
        prop.y = (float)(w >> 16) * (1.f / 65535.f) * (b.y - a.y) + a.y;
        prop.w = ps.prop(S, (!w) == 0).w;
    }
}

/* updateproperty, mcx_core.cl:1079-1187: labels, float mua, half mua/mus,
   label + one half-precision property, byte and short mixtures of rows 1-2 */
template <class PS>
__device__ __forceinline__ void updateprop(const PS& ps, const Shared& S, float4& prop, unsigned int mediaid) {
    const mcxg_kparams& c_p = ps.p();
    const unsigned int w = mediaid & K_MED_MASK;
    if (KP_MEDIAFORMAT <= 4) {
        prop = ps.prop(S, w);
    } else if (KP_MEDIAFORMAT == 101) {
        prop.x = fabsf(__uint_as_float(mediaid));
        prop.w = ps.prop(S, (!w) == 0).w;
    } else {
        if (PS::kXMedia) {
            media_other(ps, S, prop, w);
        }
    }
}

/* the reference's (ushort)flipdir < maxidx test (mcx_core.cl:2803) in
   integers: the voxel index wrapped to 16 bits against the extent */
template <class PS>
__device__ __forceinline__ bool inside_u(const PS& ps, int x, int y, int z) {
    const mcxg_kparams& c_p = ps.p();
    return ((unsigned int)x & 0xFFFFu) < c_p.dimx && ((unsigned int)y & 0xFFFFu) < c_p.dimy &&
           ((unsigned int)z & 0xFFFFu) < c_p.dimz;
}

template <class PS>
__device__ __forceinline__ unsigned int vox_index(const PS& ps, int x, int y, int z) {
    const mcxg_kparams& c_p = ps.p();
    return (unsigned int)(z * (int)c_p.dimxy + y * (int)c_p.dimx + x);
}

/* hitgrid, OpenCL branch (mcx_core.cl:988-993): distance to the next voxel
   face along v, face id into fw */
template <bool EXACT>
__device__ __forceinline__ float hitgrid(const float4& p, const float4& v, int fx, int fy, int fz, int& fw) {
    float hx = fabsf((float)fx - (v.x > 0.f ? -1.f : 0.f) - p.x);
    float hy = fabsf((float)fy - (v.y > 0.f ? -1.f : 0.f) - p.y);
    float hz = fabsf((float)fz - (v.z > 0.f ? -1.f : 0.f) - p.z);
    hx = fabsf(Mth<EXACT>::div(hx + K_EPS, v.x));
    hy = fabsf(Mth<EXACT>::div(hy + K_EPS, v.y));
    hz = fabsf(Mth<EXACT>::div(hz + K_EPS, v.z));
    float dist = fminf(fminf(hx, hy), hz);
    fw = (dist == hx ? 0 : (dist == hy ? 1 : 2));
    return dist;
}

/* hitgrid of the fast kernel with the direction's reciprocals cached:
   __fdividef(h, v) == h * rcp(v), so the result is the same bits */
__device__ __forceinline__ float hitgrid_rcp(const float4& p, const float4& v, const float3& rv, int fx, int fy, int fz,
                                             int& fw) {
    float hx = fabsf((float)fx - (v.x > 0.f ? -1.f : 0.f) - p.x);
    float hy = fabsf((float)fy - (v.y > 0.f ? -1.f : 0.f) - p.y);
    float hz = fabsf((float)fz - (v.z > 0.f ? -1.f : 0.f) - p.z);
    hx = fabsf((hx + K_EPS) * rv.x);
    hy = fabsf((hy + K_EPS) * rv.y);
    hz = fabsf((hz + K_EPS) * rv.z);
    float dist = fminf(fminf(hx, hy), hz);
    fw = (dist == hx ? 0 : (dist == hy ? 1 : 2));
    return dist;
}

/* rotatevector, mcx_core.cl:1025-1042 */
template <bool EXACT>
__device__ __forceinline__ void rotatevector(float4& v, float st, float ct, float sp, float cp) {
    if (v.z > -1.f + K_EPS && v.z < 1.f - K_EPS) {
        float tmp0 = 1.f - v.z * v.z;
        float tmp1 = st * Mth<EXACT>::rsqrt(tmp0);
        float nx = tmp1 * (v.x * v.z * cp - v.y * sp) + v.x * ct;
        float ny = tmp1 * (v.y * v.z * cp + v.x * sp) + v.y * ct;
        float nz = -tmp1 * tmp0 * cp + v.z * ct;
        v.x = nx;
        v.y = ny;
        v.z = nz;
    } else {
        v.x = st * cp;
        v.y = st * sp;
        v.z = (v.z > 0.f) ? ct : -ct;
    }
    if (EXACT) {
        /* the reference renormalises component by component */
        v.x *= Mth<EXACT>::rsqrt(v.x * v.x + v.y * v.y + v.z * v.z);
        v.y *= Mth<EXACT>::rsqrt(v.x * v.x + v.y * v.y + v.z * v.z);
        v.z *= Mth<EXACT>::rsqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    } else {
        float r = Mth<EXACT>::rsqrt(v.x * v.x + v.y * v.y + v.z * v.z);
        v.x *= r;
        v.y *= r;
        v.z *= r;
    }
}

/* updateproperty_svmc (mcx_core.cl:1231-1280): the properties of the side of
   the voxel's plane the photon is on; the plane's reference point (in the
   voxel) and normal decode from the second volume plane.  A voxel outside the
   volume takes row 0 and leaves the split state as it was. */
template <bool EXACT, class PS>
__device__ __forceinline__ void updateprop_svmc(const KArgs& a, const PS& ps, const Shared& S, float4& prop,
                                                unsigned int mediaid, unsigned int idx1d, const float4& p, int fx,
                                                int fy, int fz, Photon& s) {
    const mcxg_kparams& c_p = ps.p();
    if (idx1d == K_OUT_MIN || idx1d == K_OUT_MAX) {
        prop = ps.prop(S, 0);
        return;
    }
    const unsigned int i0 = __ldg(a.media32 + ps.media_off() + c_p.nvox + idx1d);
    const unsigned int i1 = mediaid & K_MED_MASK;
    unsigned int sv = (i1 >> 24) | (((i1 >> 16) & 0xFFu) << 8);
    if ((i1 >> 16) & 0xFFu) {
        const float rx = (float)((i1 >> 8) & 0xFFu) * (1.f / 255.f) + (float)(short)fx;
        const float ry = (float)(i1 & 0xFFu) * (1.f / 255.f) + (float)(short)fy;
        const float rz = (float)(i0 >> 24) * (1.f / 255.f) + (float)(short)fz;
        float nx = (float)((i0 >> 16) & 0xFFu) * (2.f / 255.f) - 1.f;
        float ny = (float)((i0 >> 8) & 0xFFu) * (2.f / 255.f) - 1.f;
        float nz = (float)(i0 & 0xFFu) * (2.f / 255.f) - 1.f;
        const float r = Mth<EXACT>::rsqrt(nx * nx + ny * ny + nz * nz);
        nx = nx * r, ny = ny * r, nz = nz * r;
        float pd = rx * nx + ry * ny + rz * nz;
        if (p.x * nx + p.y * ny + p.z * nz > pd) {
            prop = ps.prop(S, SV_UPPER(sv));
            sv |= 1u << 17;
            nx = -nx, ny = -ny, nz = -nz;
            pd = -pd;
        } else {
            prop = ps.prop(S, SV_LOWER(sv));
        }
        s.nv = make_float3(nx, ny, nz);
        s.pd = pd;
        sv |= 1u << 16;
    } else {
        prop = ps.prop(S, i1 >> 24);
    }
    s.sv = sv;
}

/* ray_plane_intersect (mcx_core.cl:1282-1303): clip the step at the voxel's
   plane when the photon moves towards it and crosses it within the step */
template <bool EXACT>
__device__ __forceinline__ bool ray_plane_intersect(const Photon& s, float gscat, float& len, float& slen) {
    const float vdotn = s.v.x * s.nv.x + s.v.y * s.nv.y + s.v.z * s.nv.z;
    if (vdotn <= 0.f) {
        return false;
    }
    const float d0 = s.p.x * s.nv.x + s.p.y * s.nv.y + s.p.z * s.nv.z - s.pd;
    const float d1 = d0 + len * vdotn;
    if (d0 * d1 > 0.f) {
        return false;
    }
    const float len0 = Mth<EXACT>::div(len * d0, d0 - d1);
    len = (len0 > 0.f) ? len0 : len;
    slen = len * s.prop.y * (s.v.w + 1.f > gscat ? (1.f - s.prop.z) : 1.f);
    return true;
}

/* reflectray_svmc (mcx_core.cl:1305-1343): Fresnel reflection or refraction
   of direction c at a split voxel's plane (s.nv faces the side the photon
   comes from); true when the photon refracts into a background half */
template <bool EXACT, class PS>
__device__ __forceinline__ bool reflectray_svmc(const PS& ps, const Shared& S, Photon& s, float n1, float3& c) {
    typedef Mth<EXACT> M;
    const float Icos = fabsf(c.x * s.nv.x + c.y * s.nv.y + c.z * s.nv.z);
    const float n2 = ps.prop(S, SV_ISUPPER(s.sv) ? SV_UPPER(s.sv) : SV_LOWER(s.sv)).w;
    const float tmp0 = n1 * n1, tmp1 = n2 * n2;
    float tmp2 = 1.f - M::div(tmp0, tmp1) * (1.f - Icos * Icos);
    if (tmp2 > 0.f) {
        float Re = tmp0 * Icos * Icos + tmp1 * tmp2;
        tmp2 = M::sqrt(tmp2);
        const float Im = 2.f * n1 * n2 * Icos * tmp2;
        float Rtotal = M::div(Re - Im, Re + Im);
        Re = tmp1 * Icos * Icos + tmp0 * tmp2 * tmp2;
        Rtotal = (Rtotal + M::div(Re - Im, Re + Im)) * 0.5f;
        if (rnd(s.t) <= Rtotal) {
            const float k = -2.f * Icos;
            c.x += k * s.nv.x, c.y += k * s.nv.y, c.z += k * s.nv.z;
            s.sv ^= 1u << 17;
        } else {
            const float k = -Icos, r = M::div(n1, n2);
            c.x += k * s.nv.x, c.y += k * s.nv.y, c.z += k * s.nv.z;
            c.x = tmp2 * s.nv.x + r * c.x;
            c.y = tmp2 * s.nv.y + r * c.y;
            c.z = tmp2 * s.nv.z + r * c.z;
            s.nv = make_float3(-s.nv.x, -s.nv.y, -s.nv.z);
            s.pd = -s.pd;
            if (SV_CURLABEL(s.sv) == 0) {
                return true;
            }
            s.prop = ps.prop(S, SV_CURLABEL(s.sv));
        }
    } else {
        const float k = -2.f * Icos;
        c.x += k * s.nv.x, c.y += k * s.nv.y, c.z += k * s.nv.z;
        s.sv ^= 1u << 17;
    }
    const float r = M::rsqrt(c.x * c.x + c.y * c.y + c.z * c.z);
    c.x = c.x * r, c.y = c.y * r, c.z = c.z * r;
    return false;
}

/* Polarised scattering angles (mcx_core.cl:2454-2469): theta uniform in cos,
   phi uniform, accepted with the probability the Mueller matrix of the
   medium gives the photon's Stokes vector at theta against the forward
   direction; the draws are capped (a guard count records a cap hit) */
template <bool EXACT>
__device__ __forceinline__ void pol_angles(const KArgs& a, Photon& s, float& theta, float& phi) {
    typedef Mth<EXACT> M;
    const unsigned int ipol = K_NANGLES * (((s.mediaid & K_MED_MASK) - 1u) < a.maxpol ? (s.mediaid & K_MED_MASK) - 1u : 0u);
    const float4 m0 = __ldg(a.smatrix + ipol);
    unsigned int tries = 0;
    for (;;) {
        float sin2phi, cos2phi;
        theta = M::acos(2.f * rnd(s.t) - 1.f);
        phi = K_TWO_PI * rnd(s.t);
        M::sincos(2.f * phi, &sin2phi, &cos2phi);
        const float i0 = m0.x * s.st.x + m0.y * (s.st.y * cos2phi + s.st.z * sin2phi);
        unsigned int ith = (unsigned int)(theta * K_NANGLES * (K_R_PI - K_EPS));
        ith = ith < K_NANGLES ? ith : K_NANGLES - 1;
        const float4 mt = __ldg(a.smatrix + ipol + ith);
        const float i1 = mt.x * s.st.x + mt.y * (s.st.y * cos2phi + s.st.z * sin2phi);
        if (!(rnd(s.t) * i0 >= i1)) {
            return;
        }
        if (++tries >= K_CONE_CAP) {
            atomicAdd(a.status + ST_GUARD, 1u);
            return;
        }
    }
}

/* updatestokes (mcx_core.cl:792-835): rotate the Stokes vector into the
   scattering plane, apply the Mueller matrix at theta, rotate back to the
   new meridian plane and normalise to I = 1 */
template <bool EXACT>
__device__ __forceinline__ void update_stokes(const KArgs& a, Photon& s, float theta, float phi, const float3& u,
                                              const float4& u2) {
    typedef Mth<EXACT> M;
    const float costheta = M::cos(theta);
    float sin2phi, cos2phi;
    M::sincos(2.f * phi, &sin2phi, &cos2phi);
    float4 s2 = make_float4(s.st.x, s.st.y * cos2phi + s.st.z * sin2phi, -s.st.y * sin2phi + s.st.z * cos2phi, s.st.w);
    const unsigned int imed = ((s.mediaid & K_MED_MASK) - 1u) < a.maxpol ? (s.mediaid & K_MED_MASK) - 1u : 0u;
    unsigned int ith = (unsigned int)(theta * K_NANGLES * (K_R_PI - K_EPS));
    ith = ith < K_NANGLES ? ith : K_NANGLES - 1;
    const float4 m = __ldg(a.smatrix + K_NANGLES * imed + ith);
    s.st.x = m.x * s2.x + m.y * s2.y;
    s.st.y = m.y * s2.x + m.x * s2.y;
    s.st.z = m.z * s2.z + m.w * s2.w;
    s.st.w = -m.w * s2.z + m.z * s2.w;
    float temp = (u2.z > -1.f && u2.z < 1.f) ? M::rsqrt((1.f - costheta * costheta) * (1.f - u2.z * u2.z)) : 0.f;
    float cosi = (temp == 0.f) ? 0.f : (((phi > K_ONE_PI && phi < K_TWO_PI) ? 1.f : -1.f) * (u2.z * costheta - u.z) * temp);
    cosi = fmaxf(-1.f, fminf(cosi, 1.f));
    const float sini = M::sqrt(1.f - cosi * cosi);
    const float cos22 = 2.f * cosi * cosi - 1.f;
    const float sin22 = 2.f * sini * cosi;
    s2 = make_float4(s.st.x, s.st.y * cos22 - s.st.z * sin22, s.st.y * sin22 + s.st.z * cos22, s.st.w);
    temp = M::div(1.f, s2.x);
    s.st = make_float4(1.f, s2.y * temp, s2.z * temp, s2.w * temp);
}

/* rotatevector2d, mcx_core.cl:1008-1023 */
template <bool EXACT>
__device__ __forceinline__ void rotatevector2d(float4& v, float st, float ct, unsigned int is2d) {
    float nx = v.x, ny = v.y, nz = v.z;
    if (is2d == 1) {
        nx = 0.f;
        ny = v.y * ct - v.z * st;
        nz = v.y * st + v.z * ct;
    } else if (is2d == 2) {
        nx = v.x * ct - v.z * st;
        ny = 0.f;
        nz = v.x * st + v.z * ct;
    } else if (is2d == 3) {
        nx = v.x * ct - v.y * st;
        ny = v.x * st + v.y * ct;
        nz = 0.f;
    }
    float tmp0 = Mth<EXACT>::rsqrt(nx * nx + ny * ny + nz * nz);
    v.x = nx * tmp0;
    v.y = ny * tmp0;
    v.z = nz * tmp0;
}

__device__ __forceinline__ float vcomp(const float4& v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : v.z);
}

/* transmit, mcx_core.cl:1044-1055 */
template <bool EXACT>
__device__ __forceinline__ void transmit(float4& v, float n1, float n2, int fw) {
    float tmp0 = Mth<EXACT>::div(n1, n2);
    v.x *= tmp0;
    v.y *= tmp0;
    v.z *= tmp0;
    if (fw == 0) {
        v.x = Mth<EXACT>::sqrt(1.f - v.y * v.y - v.z * v.z) * (float)((v.x > 0.f) - (v.x < 0.f));
    } else if (fw == 1) {
        v.y = Mth<EXACT>::sqrt(1.f - v.x * v.x - v.z * v.z) * (float)((v.y > 0.f) - (v.y < 0.f));
    } else {
        v.z = Mth<EXACT>::sqrt(1.f - v.x * v.x - v.y * v.y) * (float)((v.z > 0.f) - (v.z < 0.f));
    }
}

/* reflectcoeff, mcx_core.cl:1057-1075 */
template <bool EXACT>
__device__ float reflectcoeff(const float4& v, float n1, float n2, int fw) {
    float Icos = fabsf(vcomp(v, fw));
    float tmp0 = n1 * n1;
    float tmp1 = n2 * n2;
    float tmp2 = 1.f - tmp0 / tmp1 * (1.f - Icos * Icos);
    if (tmp2 > 0.f) {
        float Re = tmp0 * Icos * Icos + tmp1 * tmp2;
        tmp2 = sqrtf(tmp2);
        float Im = 2.f * n1 * n2 * Icos * tmp2;
        float Rtotal = (Re - Im) / (Re + Im);
        Re = tmp1 * Icos * Icos + tmp0 * tmp2 * tmp2;
        Rtotal = (Rtotal + (Re - Im) / (Re + Im)) * 0.5f;
        return Rtotal;
    }
    return 1.f;
}

/* skipvoid, mcx_core.cl:1350-1455: march through background voxels to the
   first labelled voxel on the ray */
template <bool EXACT, bool SVMC, class PS>
__device__ int skipvoid(const KArgs& a, const PS& ps, const Shared& S, float4& p, float4& v, float4& f, int& fx,
                        int& fy, int& fz, int& fw) {
    const mcxg_kparams& c_p = ps.p();
    int count = 1;
    fx = (int)(short)floorf(p.x);
    fy = (int)(short)floorf(p.y);
    fz = (int)(short)floorf(p.z);
    fw = -1;
    for (;;) {
        if (inside_u(ps, fx, fy, fz)) {
            int idx1d = (int)vox_index(ps, fx, fy, fz);
            if (media_at(a, ps, idx1d) & K_MED_MASK) {
                p.x -= v.x;
                p.y -= v.y;
                p.z -= v.z;
                fx = (int)(short)floorf(p.x);
                fy = (int)(short)floorf(p.y);
                fz = (int)(short)floorf(p.z);
                f.y -= c_p.minaccumtime;
                idx1d = (int)vox_index(ps, fx, fy, fz);
                count = 0;
                while (!inside_u(ps, fx, fy, fz) || !(media_at(a, ps, idx1d) & K_MED_MASK)) {
                    float dist = hitgrid<EXACT>(p, v, fx, fy, fz, fw);
                    f.y += c_p.minaccumtime * dist;
                    p.x = p.x + dist * v.x;
                    p.y = p.y + dist * v.y;
                    p.z = p.z + dist * v.z;
                    if (fw == 0) {
                        fx += (v.x > 0.f ? 1 : -1);
                    }
                    if (fw == 1) {
                        fy += (v.y > 0.f ? 1 : -1);
                    }
                    if (fw == 2) {
                        fz += (v.z > 0.f ? 1 : -1);
                    }
                    idx1d = (int)vox_index(ps, fx, fy, fz);
                    if (count++ > 3) {
                        break;
                    }
                }
                f.y = (c_p.voidtime) ? f.y : 0.f;
                {
                    unsigned int m = media_at(a, ps, idx1d);
                    float4 ht = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (KP_SVMC) {
                        /* the side of the entry voxel's plane (1404-1420); the launch sets
                           the photon's split state again, and the specular test uses that
                           side's index where the reference reads the table at the voxel word */
                        Photon tmp;
                        updateprop_svmc<EXACT>(a, ps, S, ht, m, (unsigned int)idx1d, p, fx, fy, fz, tmp);
                    } else {
                        updateprop(ps, S, ht, m);
                    }
                    /* ht.w is the entry voxel's index of refraction; the reference reads
                       gproperty[label].w, the same value for label volumes and an index past
                       the table for float-mua volumes */
                    if (c_p.isspecular && ht.w != ps.prop(S, 0).w) {
                        p.w *= 1.f - reflectcoeff<EXACT>(v, ps.prop(S, 0).w, ht.w, fw);
                        if (p.w > K_EPS) {
                            transmit<EXACT>(v, ps.prop(S, 0).w, ht.w, fw);
                        }
                    }
                }
                return idx1d;
            }
        }
        if (((p.x < 0.f) && (v.x <= 0.f)) || ((p.x >= c_p.maxidx.x) && (v.x >= 0.f)) ||
            ((p.y < 0.f) && (v.y <= 0.f)) || ((p.y >= c_p.maxidx.y) && (v.y >= 0.f)) ||
            ((p.z < 0.f) && (v.z <= 0.f)) || ((p.z >= c_p.maxidx.z) && (v.z >= 0.f))) {
            return -1;
        }
        p.x = p.x + v.x;
        p.y = p.y + v.y;
        p.z = p.z + v.z;
        fx = (int)(short)floorf(p.x);
        fy = (int)(short)floorf(p.y);
        fz = (int)(short)floorf(p.z);
        f.y += c_p.minaccumtime;
        if ((unsigned int)count++ > c_p.maxvoidstep) {
            return -1;
        }
    }
}

/* finddetector, mcx_core.cl:838-850 */
template <class PS>
__device__ __forceinline__ unsigned int finddetector(const PS& ps, const float4& p) {
    const mcxg_kparams& c_p = ps.p();
    const float4* c_det = ps.det();
    for (unsigned int i = 0; i < c_p.detnum; i++) {
        float4 d = c_det[i];
        if ((d.x - p.x) * (d.x - p.x) + (d.y - p.y) * (d.y - p.y) + (d.z - p.z) * (d.z - p.z) < d.w * d.w) {
            return i + 1;
        }
    }
    return 0;
}

/* savedetphoton, mcx_core.cl:867-926 */
template <bool POL, class PS>
__device__ void savedetphoton(const KArgs& a, const PS& ps, const Shared& S, Photon& s, unsigned int isdet) {
    const mcxg_kparams& c_p = ps.p();
    int detid = (isdet == K_OUT_MIN) ? -1 : (int)finddetector(ps, s.p);
    if (!detid) {
        return;
    }
    unsigned int slot = atomicAdd(a.detcount, 1u);
    if (slot < c_p.maxdetphoton) {
        if (c_p.issaveseed) {
            a.detseed[slot * 2] = ps.cold()->ps0;
            a.detseed[slot * 2 + 1] = ps.cold()->ps1;
        }
        float* rec = a.detp + (size_t)slot * c_p.reclen;
        unsigned int k = 0;
        if (SAVE_DETID(c_p.savedetflag)) {
            if (c_p.extrasrclen && (c_p.srcid <= 0)) {
                detid |= (((int)ps.cold()->srcsel) << 16);
            }
            rec[k++] = (float)detid;
        }
        for (unsigned int i = 0; i < c_p.partialdata; i++) {
            rec[k++] = ps.pp(i);
        }
        if (SAVE_PEXIT(c_p.savedetflag)) {
            rec[k++] = s.p.x;
            rec[k++] = s.p.y;
            rec[k++] = s.p.z;
        }
        if (SAVE_VEXIT(c_p.savedetflag)) {
            rec[k++] = s.v.x;
            rec[k++] = s.v.y;
            rec[k++] = s.v.z;
        }
        if (SAVE_W0(c_p.savedetflag)) {
            rec[k++] = ps.cold()->w0init;
        }
        if (POL && SAVE_IQUV(c_p.savedetflag)) {
            rec[k++] = s.st.x;
            rec[k++] = s.st.y;
            rec[k++] = s.st.z;
            rec[k++] = s.st.w;
        }
        if (a.detw) {
            a.detw[slot] = make_float2(s.p.w, s.f.y);
        }
    } else if (c_p.savedet == 3) {
        atomicSub(a.detcount, 1u);
    }
}

/* ---------------------------------------------------------------- deposit */

/* Compensated accumulation: each field component is a plane of signed
   64-bit fixed-point counts of 2^-S and a plane of float remainders.  A
   deposit w is split exactly into k = round(w 2^S) and r = w - k 2^-S
   (|r| <= 2^-(S+1)); k goes to the integer plane, r to the float plane, both
   with fire-and-forget atomics.  Integer adds are exact in any order -- also
   when the memory system merges the adds of several lanes to one address --
   so the bulk of an element carries no rounding at all, and the remainders
   are too small for the float plane's rounding to matter: an element is
   count x 2^-S + remainder, summed in FP64.  The host picks S per problem so
   that no element can reach 2^62 units (mcx_host.c, field_scale).  A float
   running sum, or float high and low planes compensated by the value an
   atomic returns (TwoSum), loses the low-order deposits of the hottest
   voxels at 1e8-1e9 photons. */
struct Field {
    unsigned long long* hi;        /* fixed-point counts */
    float* lo;                     /* remainders */
    float sc, unit;                /* 2^S, 2^-S */
};

/* component comp of the field (0 real, 1 imaginary); the planes of the
   components follow one another, plane length ps.lo_plane() */
template <class PS>
__device__ __forceinline__ Field field_of(const KArgs& a, const PS& ps, unsigned int comp) {
    const mcxg_kparams& c_p = ps.p();
    const size_t F = ps.lo_plane();
    Field f;
    f.hi = a.fhi + comp * F;
    f.lo = a.flo + comp * F;
    f.sc = c_p.fxscale;
    f.unit = c_p.fxunit;
    return f;
}

/* w = k 2^-S + r exactly: k is w 2^S rounded to an integer (a float integer,
   so exact in float), r the part below the grid */
__device__ __forceinline__ void field_split(const Field& f, float w, long long& k, float& r) {
    k = __float2ll_rn(__fmul_rn(w, f.sc));
    r = __fsub_rn(w, __fmul_rn((float)k, f.unit));
}

__device__ __forceinline__ void field_commit(const Field& f, size_t i, long long k, float r) {
    if (k) {
        atomicAdd(f.hi + i, (unsigned long long)k);
    }
    if (r != 0.f) {
        atomicAdd(f.lo + i, r);
    }
}

__device__ __forceinline__ void field_add(const Field& f, size_t i, float w) {
    long long k;
    float r;
    field_split(f, w, k, r);
    field_commit(f, i, k, r);
}

/* Deposit from every lane that has one; with WAGG, lanes of the warp hitting
   the same field element add their integer parts (exactly) and their
   remainders first and one leader commits. */
template <bool WAGG>
__device__ __forceinline__ void deposit(const Field& f, bool doit, unsigned int key, float w) {
    if (!WAGG) {
        if (doit) {
            field_add(f, key, w);
        }
        return;
    }
    unsigned int act = __activemask();
    unsigned int m = __ballot_sync(act, doit);
    if (!doit) {
        return;
    }
    long long k;
    float r;
    field_split(f, w, k, r);
    unsigned int peers = __match_any_sync(m, key);
    unsigned int lane = threadIdx.x & 31u;
    if (peers == (1u << lane)) {
        field_commit(f, key, k, r);
        return;
    }
    long long ksum = 0;
    float rsum = 0.f;
    unsigned int rest = peers;
    while (rest) {
        int src = __ffs(rest) - 1;
        rest &= rest - 1;
        ksum += __shfl_sync(peers, k, src);
        rsum += __shfl_sync(peers, r, src);
    }
    if ((int)lane == __ffs(peers) - 1) {
        field_commit(f, key, ksum, rsum);
    }
}

/* rf replay output (mcx_core.cl:2853-2877): the real part (no spill) and,
   with omega > 0, the imaginary part in the planes after the real ones; the
   gate shift and its fold follow the deposit in the transport loop */
template <class PS>
__device__ __forceinline__ void rf_replay_deposit(const KArgs& a, const PS& ps, unsigned int idx, int tshift, float wre,
                                                  float wim) {
    const mcxg_kparams& c_p = ps.p();
    if (c_p.extrasrclen && (c_p.srcid < 0)) {
        tshift += ((int)ps.cold()->srcsel - 1) * ((c_p.replaydet == -1) ? (int)c_p.detnum : 1) * (int)c_p.maxgate;
    }
    unsigned int key = idx + (unsigned int)tshift * c_p.nvox;
    if (key >= c_p.fieldlen) {
        key -= c_p.fieldlen;
    }
    field_add(field_of(a, ps, 0), key, wre);
    if (c_p.omega > 0.f) {
        field_add(field_of(a, ps, 1), key, wim);
    }
}

/* Photon sharing (mcx_core.cl:1527-1538, 2902-2911): a deposit goes to every
   pattern with a non-zero weight, element (voxel + gate * nvox) * srcnum +
   pattern, scaled by that weight.  An element one gate past the last folds
   into the low plane at gate 0, as the single-pattern deposit does. */
template <class PS>
__device__ __forceinline__ void share_deposit(const KArgs& a, const PS& ps, unsigned int key, float w) {
    const mcxg_kparams& c_p = ps.p();
    const unsigned int n = c_p.srcnum;
    for (unsigned int i = 0; i < n; i++) {
        const float pw = ps.pp(c_p.partialdata + i);
        if (fabsf(pw) > 0.f) {
            unsigned int k = key * n + i;
            if (k >= c_p.fieldlen) {
                k -= c_p.fieldlen;
            }
            field_add(field_of(a, ps, 0), k, w * pw);
        }
    }
}

/* ------------------------------------------------------------------ replay */

/* index of the photon a replay quantity belongs to: the reference's
   vt*threadphoton + min(vt, oddphoton-1) + offset (mcx_core.cl:1591, 2571, 2847) */
template <class PS>
__device__ __forceinline__ long long replay_index(const PS& ps, unsigned int vt, long long offset) {
    const mcxg_kparams& c_p = ps.p();
    long long m = (long long)c_p.oddphoton - 1;
    long long t = (long long)vt;
    return t * (long long)c_p.threadphoton + (t < m ? t : m) + offset;
}

/* replay deposit at a scattering site (mcx_core.cl:2567-2604): the detected
   weight (x (1 - cos theta) for the momentum-transfer output, x time of
   flight for wptof) into the gate of the photon's detected time of flight */
template <class PS>
__device__ void replay_site_deposit(const KArgs& a, const PS& ps, const Shared& S, const Photon& s, unsigned int vt,
                                    float ctheta) {
    const mcxg_kparams& c_p = ps.p();
    long long k = replay_index(ps, vt, (long long)(int)s.f.w - 1 + (long long)c_p.siteshift);
    if (k < 0 || k >= (long long)c_p.nreplay) {
        return;        /* the reference reads one photon past its arrays here */
    }
    float rt = __ldg(a.rtof + k);
    float rw = __ldg(a.rweight + k);
    float tmp0 = (c_p.outputtype == otDCS) ? (1.f - ctheta) : 1.f;
    float tim = 0.f;
    if (c_p.outputtype == otRFmus) {
        /* 2572-2576: the launch phase's cos / sin (the reference's imaginary
           part goes to a quarter of the field it never allocated) */
        tmp0 = rw * ps.pp(c_p.partialdata);
        tim = rw * ps.pp(c_p.partialdata + 1);
    } else if (c_p.outputtype == otWPTOF) {
        tmp0 = rt;
        tmp0 *= rw;
    } else {
        tmp0 *= rw;
    }
    int tshift = (int)(floorf((rt - c_p.twin0) * c_p.Rtstep)) +
                 ((c_p.replaydet == -1) ? (((__ldg(a.rdetid + k) & 0xFFFF) - 1) * (int)c_p.maxgate) : 0);
    if (c_p.extrasrclen && (c_p.srcid < 0)) {
        tshift += ((int)ps.cold()->srcsel - 1) * ((c_p.replaydet == -1) ? (int)c_p.detnum : 1) * (int)c_p.maxgate;
    }
    tshift = ((int)c_p.maxgate - 1 < tshift) ? (int)c_p.maxgate - 1 : tshift;
    long long key = (long long)s.idx1d + (long long)tshift * c_p.nvox;
    if (key < 0 || key >= (long long)c_p.fieldlen) {
        atomicAdd(a.status + ST_GUARD, 1u);
        return;
    }
    field_add(field_of(a, ps, 0), ps.field_off() + (unsigned int)key, tmp0);
    if (c_p.outputtype == otRFmus) {
        field_add(field_of(a, ps, 1), (unsigned int)key, tim);
    }
}

/* ------------------------------------------------------------------ launch */

template <class PS>
__device__ __forceinline__ void set_launch_voxel(const KArgs& a, const PS& ps, Photon& s) {
    const mcxg_kparams& c_p = ps.p();
    s.idx1d = (unsigned int)((int)(floorf(s.p.z)) * (int)c_p.dimxy + (int)(floorf(s.p.y)) * (int)c_p.dimx +
                             (int)(floorf(s.p.x)));
    if (s.p.x < 0.f || s.p.y < 0.f || s.p.z < 0.f || s.p.x >= c_p.maxidx.x || s.p.y >= c_p.maxidx.y ||
            s.p.z >= c_p.maxidx.z) {
        s.mediaid = 0;
    } else {
        s.mediaid = media_at(a, ps, s.idx1d);
    }
}

/* savedebugdata (mcx_core.cl:929-948): one trajectory record {photon id
   (uint bits), x, y, z, w, source id} at a slot from a global counter.  The
   id is the reference thread's launch counter plus its photon offset, which
   the close record computes with min(tid, oddphoton) (1501) and the launch
   and scattering records with min(tid, (tid < oddphoton) tid) (2247, 2630). */
__device__ __forceinline__ void save_traj(const KArgs& a, const mcxg_kparams& c_p, const Photon& s, float srcsel,
                                          unsigned int vt, bool closing) {
    const int tid = (int)vt, odd = c_p.oddphoton, x = (tid < odd) * tid;
    const int off = closing ? min(tid, odd) : min(tid, x);
    const unsigned int id = (unsigned int)s.f.w + (unsigned int)(tid * (int)c_p.threadphoton) + (unsigned int)off;
    const unsigned int pos = atomicAdd(a.jumpctr, 1u);
    if (pos < a.maxjump) {
        float* r = a.traj + (size_t)pos * 6;
        r[0] = __uint_as_float(id);
        r[1] = s.p.x;
        r[2] = s.p.y;
        r[3] = s.p.z;
        r[4] = s.p.w;
        r[5] = (float)(int)srcsel;
    }
}

/*
 * launchnewphoton (mcx_core.cl:1463-2275): close the current photon (escaped
 * weight, saved reflectance, detection) and launch the next one of this
 * reference thread.  Returns 0 on launch, 1 when the thread's quota is done,
 * -1 when no launch position was found.
 */
template <bool EXACT, bool DET, bool RF, bool POL, bool SVMC, class PS>
__device__ int launchnewphoton(const KArgs& a, const PS& ps, const Shared& S, Photon& s, unsigned int isdet,
                               unsigned int vt, unsigned long long* nfailed) {
    const mcxg_kparams& c_p = ps.p();
    const float4* c_srcx = ps.srcx();
    typedef Mth<EXACT> M;
    s.w0 = 1.f;
    s.Lmove = -1.f;

    if (DET && c_p.savedet == 3 && *(volatile unsigned int*)a.detcount >= c_p.maxdetphoton) {
        return 1;
    }

    if (fabsf(s.p.w) >= 0.f) {
        ps.cold()->esc += s.p.w;
        if (!PS::kCommon && !PS::kBatch && a.maxjump) {
            save_traj(a, ps.p(), s, ps.cold()->srcsel, vt, true);
        }
        if (s.mediaid == 0 && s.idx1d != K_OUT_MIN && s.idx1d != K_OUT_MAX && c_p.issaveref && s.p.w > 0.f) {
            int tshift = (int)floorf((s.f.y - c_p.twin0) * c_p.Rtstep);
            if ((int)c_p.maxgate - 1 < tshift) {
                tshift = (int)c_p.maxgate - 1;
            }
            if (c_p.extrasrclen && (c_p.srcid < 0)) {
                tshift += ((int)ps.cold()->srcsel - 1) * (int)c_p.maxgate;
            }
            const unsigned int key = ps.field_off() + s.idx1d + (unsigned int)tshift * c_p.nvox;
            if (KP_SHARING) {
                share_deposit(a, ps, key, -s.p.w);
            } else {
                field_add(field_of(a, ps, 0), key, -s.p.w);
            }
        }
        if (DET && c_p.savedet && (isdet & K_DET_MASK) == K_DET_MASK &&
                (s.mediaid == 0 || (KP_SVMC && SV_CURLABEL(s.sv) == 0)) && c_p.issaveref < 2) {
            savedetphoton<POL>(a, ps, S, s, isdet);
        }
    }
    if (DET) {
        for (unsigned int i = 0; i < c_p.partialdata; i++) {
            ps.pp(i) = 0.f;
        }
    }

    if (s.f.w >= (float)(c_p.threadphoton + (vt < (unsigned int)c_p.oddphoton))) {
        return 1;
    }

    if (c_p.replay) {
        /* the saved launch state of this photon (mcx_core.cl:1590-1596) */
        long long k = replay_index(ps, vt, (long long)((int)s.f.w > 0 ? (int)s.f.w : 0));
        if (k < 0 || k >= (long long)c_p.nreplay) {
            atomicAdd(a.status + ST_GUARD, 1u);
            return 1;
        }
        ulonglong2 st = a.rseed[k];
        s.t.a = st.x;
        s.t.b = st.y;
    }

    if (DET && c_p.issaveseed) {
        ps.cold()->ps0 = s.t.a;
        ps.cold()->ps1 = s.t.b;
    }

    float4 lpos = f4(c_p.srcpos), ldir = f4(c_p.srcdir), lp1 = f4(c_p.srcparam1), lp2 = f4(c_p.srcparam2);
    if (c_p.extrasrclen && (c_p.srcid != 1)) {
        int sel = -1;
        if (c_p.srcid > 1) {
            sel = c_p.srcid - 2;
        } else {
            ps.cold()->srcsel = (float)((int)(rnd(s.t) * K_JUST_BELOW_ONE * (float)(c_p.extrasrclen + 1)) + 1);
            if ((int)ps.cold()->srcsel > 1) {
                sel = (int)(ps.cold()->srcsel - 2);
            }
        }
        if (sel >= 0) {
            lpos = c_srcx[sel * 4];
            ldir = c_srcx[sel * 4 + 1];
            lp1 = c_srcx[sel * 4 + 2];
            lp2 = c_srcx[sel * 4 + 3];
        }
    }

    if (c_p.replay && c_p.srcid >= 1) {
        rnd(s.t);      /* keeps the stream in step with a run that picked a source (1614-1616) */
    }

    unsigned int attempts = 0;
    for (;;) {
        if (++attempts > K_LAUNCH_CAP) {
            return -1;
        }
        s.p = lpos;
        s.v = ldir;
        if (KP_SVMC) {
            s.sv = 0u;        /* 1640-1642 */
        }
        s.f.x = 0.f;
        s.f.y = 0.f;
        s.f.z = c_p.minaccumtime;
        if (KP_POL) {
            s.st = a.s0;      /* 1633-1638 */
        }
        s.idx1d = __float_as_uint(lp2.z);
        s.mediaid = __float_as_uint(lp2.w);
        s.prop = make_float4(lpos.x, lpos.y, lpos.z, 0.f);

        const unsigned int st = c_p.srctype;
        if (st == S_PENCIL) {
            /* position and direction already set */
        } else if (st == S_PLANAR || st == S_PATTERN || st == S_PATTERN3D || st == S_FOURIER || st == S_PENCILARRAY) {
            float rx = rnd(s.t);
            float ry = rnd(s.t);
            float rz = 0.f;
            if (st == S_PATTERN3D) {
                rz = rnd(s.t);
                s.p.x = s.p.x + rx * lp1.x;
                s.p.y = s.p.y + ry * lp1.y;
                s.p.z = s.p.z + rz * lp1.z;
            } else {
                s.p.x = s.p.x + rx * lp1.x + ry * lp2.x;
                s.p.y = s.p.y + rx * lp1.y + ry * lp2.y;
                s.p.z = s.p.z + rx * lp1.z + ry * lp2.z;
            }
            if (st == S_PATTERN || st == S_PATTERN3D) {
                unsigned int pi;
                if (st == S_PATTERN) {
                    pi = (unsigned int)((int)(ry * K_JUST_BELOW_ONE * lp2.w) * (int)(lp1.w) +
                                        (int)(rx * K_JUST_BELOW_ONE * lp1.w));
                } else {
                    pi = (unsigned int)((int)(rz * K_JUST_BELOW_ONE * lp1.z) * (int)(lp1.y) * (int)(lp1.x) +
                                        (int)(ry * K_JUST_BELOW_ONE * lp1.y) * (int)(lp1.x) +
                                        (int)(rx * K_JUST_BELOW_ONE * lp1.x));
                }
                if (KP_SHARING) {
                    /* photon sharing (mcx_core.cl:1697-1704, 1718-1726): the photon
                       carries weight 1 and one weight per pattern; the pixel index
                       takes the initial-weight slot */
                    const unsigned int n = c_p.srcnum;
                    for (unsigned int i = 0; i < n; i++) {
                        ps.pp(c_p.partialdata + i) = a.srcpattern[min(pi * n + i, c_p.npattern - 1)];
                    }
                    ps.cold()->w0init = __uint_as_float(pi);
                    s.p.w = 1.f;
                } else {
                    s.p.w = lpos.w * a.srcpattern[min(pi, c_p.npattern - 1)];
                }
            } else if (st == S_FOURIER) {
                s.p.w = lpos.w * (M::cos((floorf(lp1.w) * rx + floorf(lp2.w) * ry + lp1.w - floorf(lp1.w)) * K_TWO_PI) *
                                  (1.f - lp2.w + floorf(lp2.w)) + 1.f) * 0.5f;
            } else if (st == S_PENCILARRAY) {
                s.p.x = lpos.x + floorf(rx * lp1.w) * lp1.x / (lp1.w - 1.f) + floorf(ry * lp2.w) * lp2.x / (lp2.w - 1.f);
                s.p.y = lpos.y + floorf(rx * lp1.w) * lp1.y / (lp1.w - 1.f) + floorf(ry * lp2.w) * lp2.y / (lp2.w - 1.f);
                s.p.z = lpos.z + floorf(rx * lp1.w) * lp1.z / (lp1.w - 1.f) + floorf(ry * lp2.w) * lp2.z / (lp2.w - 1.f);
            }
            set_launch_voxel(a, ps, s);
            s.prop.x = s.prop.x + (lp1.x + lp2.x) * 0.5f;
            s.prop.y = s.prop.y + (lp1.y + lp2.y) * 0.5f;
            s.prop.z = s.prop.z + (lp1.z + lp2.z) * 0.5f;
            s.prop.w = 0.f;
        } else if (st == S_FOURIERX || st == S_FOURIERX2D) {
            float rx = rnd(s.t);
            float ry = rnd(s.t);
            float4 v2 = lp1;
            v2.w *= M::rsqrt(lp1.x * lp1.x + lp1.y * lp1.y + lp1.z * lp1.z);
            v2.x = v2.w * (ldir.y * lp1.z - ldir.z * lp1.y);
            v2.y = v2.w * (ldir.z * lp1.x - ldir.x * lp1.z);
            v2.z = v2.w * (ldir.x * lp1.y - ldir.y * lp1.x);
            s.p.x = s.p.x + rx * lp1.x + ry * v2.x;
            s.p.y = s.p.y + rx * lp1.y + ry * v2.y;
            s.p.z = s.p.z + rx * lp1.z + ry * v2.z;
            if (st == S_FOURIERX2D) {
                s.p.w = lpos.w * (M::sin((lp2.x * rx + lp2.z) * K_TWO_PI) * M::sin((lp2.y * ry + lp2.w) * K_TWO_PI) + 1.f) * 0.5f;
            } else {
                s.p.w = lpos.w * (M::cos((lp2.x * rx + lp2.y * ry + lp2.z) * K_TWO_PI) * (1.f - lp2.w) + 1.f) * 0.5f;
            }
            set_launch_voxel(a, ps, s);
            s.prop.x = s.prop.x + (lp1.x + v2.x) * 0.5f;
            s.prop.y = s.prop.y + (lp1.y + v2.y) * 0.5f;
            s.prop.z = s.prop.z + (lp1.z + v2.z) * 0.5f;
            s.prop.w = 0.f;
        } else if (st == S_HYPERBOLOID) {
            float sphi, cphi, r;
            r = K_TWO_PI * rnd(s.t);
            M::sincos(r, &sphi, &cphi);
            r = M::sqrt(0.5f * rnd_scatlen<EXACT>(s.t)) * lp1.x;
            s.prop.x = -lp1.y / lp1.z;
            s.prop.y = M::rsqrt(r * r + lp1.z * lp1.z);
            s.p.x = r * (cphi - s.prop.x * sphi);
            s.p.y = r * (sphi + s.prop.x * cphi);
            s.p.z = 0.f;
            {
                float4 np;
                np.x = -r * sphi * s.prop.y;
                np.y = r * cphi * s.prop.y;
                np.z = lp1.z * s.prop.y;
                np.w = 0.f;
                s.prop = np;
            }
            if (s.v.z > -1.f + K_EPS && s.v.z < 1.f - K_EPS) {
                r = 1.f - s.v.z * s.v.z;
                float sth = M::sqrt(r);
                r = M::rsqrt(r);
                cphi = s.v.x * r;
                sphi = s.v.y * r;
                float px = s.p.x * cphi * s.v.z - s.p.y * sphi;
                float py = s.p.x * sphi * s.v.z + s.p.y * cphi;
                float pz = -s.p.x * sth;
                s.p.x = px;
                s.p.y = py;
                s.p.z = pz;
                float vx = s.prop.x * cphi * s.v.z - s.prop.y * sphi + s.prop.z * cphi * sth;
                float vy = s.prop.x * sphi * s.v.z + s.prop.y * cphi + s.prop.z * sphi * sth;
                float vz = -s.prop.x * sth + s.prop.z * s.v.z;
                s.v.x = vx;
                s.v.y = vy;
                s.v.z = vz;
            } else {
                s.v.x = s.prop.x;
                s.v.y = s.prop.y;
                s.v.z = (s.v.z > 0.f) ? s.prop.z : -s.prop.z;
            }
            s.p.x = s.p.x + lpos.x;
            s.p.y = s.p.y + lpos.y;
            s.p.z = s.p.z + lpos.z;
            s.prop = make_float4(lpos.x, lpos.y, lpos.z, 0.f);
            s.Lmove = 0.f;
        } else if (st == S_DISK || st == S_GAUSSIAN || st == S_RING) {
            float sphi, cphi, phi, r;
            if (st == S_DISK || st == S_RING) {
                if (lp1.z > 0.f || lp1.w > 0.f) {
                    phi = fabsf(lp1.z - lp1.w) * rnd(s.t) + fminf(lp1.z, lp1.w);
                } else {
                    phi = K_TWO_PI * rnd(s.t);
                }
            } else {
                phi = K_TWO_PI * rnd(s.t);
            }
            M::sincos(phi, &sphi, &cphi);
            if (st == S_DISK || st == S_RING) {
                r = M::sqrt(rnd(s.t) * fabsf(lp1.x * lp1.x - lp1.y * lp1.y) + lp1.y * lp1.y);
            } else {
                if (fabsf(ldir.w) < 1e-5f || fabsf(lp1.y) < 1e-5f) {
                    r = M::sqrt(-0.5f * M::log(rnd(s.t))) * lp1.x;
                } else {
                    r = lp1.x * lp1.x * K_ONE_PI / lp1.y;
                    r = M::sqrt(-0.5f * M::log(rnd(s.t)) * (1.f + (ldir.w * ldir.w / (r * r)))) * lp1.x;
                }
            }
            if (s.v.z > -1.f + K_EPS && s.v.z < 1.f - K_EPS) {
                float tmp0 = 1.f - s.v.z * s.v.z;
                float tmp1 = r * M::rsqrt(tmp0);
                s.p.x = s.p.x + tmp1 * (s.v.x * s.v.z * cphi - s.v.y * sphi);
                s.p.y = s.p.y + tmp1 * (s.v.y * s.v.z * cphi + s.v.x * sphi);
                s.p.z = s.p.z - tmp1 * tmp0 * cphi;
            } else {
                s.p.x += r * cphi;
                s.p.y += r * sphi;
            }
            set_launch_voxel(a, ps, s);
        } else if (st == S_CONE || st == S_ISOTROPIC || st == S_ARCSINE) {
            float ang, sth, cth, sphi, cphi;
            ang = K_TWO_PI * rnd(s.t);
            M::sincos(ang, &sphi, &cphi);
            if (st == S_CONE) {
                /* the reference loops until a draw falls inside the cone; a cone
                   of zero half-angle would never end, so the draws are capped */
                unsigned int tries = 0;
                do {
                    ang = (lp1.y > 0) ? K_TWO_PI * rnd(s.t) : M::acos(2.f * rnd(s.t) - 1.f);
                } while (ang > lp1.x && ++tries < K_CONE_CAP);
            } else if (st == S_ISOTROPIC) {
                ang = M::acos(2.f * rnd(s.t) - 1.f);
            } else {
                ang = K_ONE_PI * rnd(s.t);
            }
            M::sincos(ang, &sth, &cth);
            rotatevector<EXACT>(s.v, sth, cth, sphi, cphi);
            s.Lmove = 0.f;
        } else if (st == S_ZGAUSSIAN) {
            float ang, sth, cth, sphi, cphi;
            ang = K_TWO_PI * rnd(s.t);
            M::sincos(ang, &sphi, &cphi);
            ang = M::sqrt(-2.f * M::log(rnd(s.t))) * (1.f - 2.f * rnd(s.t)) * lp1.x;
            M::sincos(ang, &sth, &cth);
            rotatevector<EXACT>(s.v, sth, cth, sphi, cphi);
            s.Lmove = 0.f;
        } else if (st == S_LINE || st == S_SLIT) {
            float r_l = rnd(s.t);
            s.p.x = s.p.x + r_l * lp1.x;
            s.p.y = s.p.y + r_l * lp1.y;
            s.p.z = s.p.z + r_l * lp1.z;
            if (st == S_LINE) {
                float sphi_l, cphi_l;
                r_l = M::rsqrt(lp1.x * lp1.x + lp1.y * lp1.y + lp1.z * lp1.z);
                if (lp2.x > 0.f) {
                    float lx = lp1.x * r_l, ly = lp1.y * r_l, lz = lp1.z * r_l;
                    float vd = s.v.x * lx + s.v.y * ly + s.v.z * lz;
                    s.v.x = s.v.x - vd * lx;
                    s.v.y = s.v.y - vd * ly;
                    s.v.z = s.v.z - vd * lz;
                    float vn = M::rsqrt(s.v.x * s.v.x + s.v.y * s.v.y + s.v.z * s.v.z);
                    s.v.x = s.v.x * vn;
                    s.v.y = s.v.y * vn;
                    s.v.z = s.v.z * vn;
                    r_l = lp2.x * (2.f * rnd(s.t) - 1.f);
                    M::sincos(r_l, &sphi_l, &cphi_l);
                    /* rotate_perpendicular_vector, mcx_core.cl:997-1006 */
                    float cx = ly * s.v.z - lz * s.v.y;
                    float cy = lz * s.v.x - lx * s.v.z;
                    float cz = lx * s.v.y - ly * s.v.x;
                    s.v.x = s.v.x * cphi_l + cx * sphi_l;
                    s.v.y = s.v.y * cphi_l + cy * sphi_l;
                    s.v.z = s.v.z * cphi_l + cz * sphi_l;
                } else {
                    s.v.x = lp1.x * r_l;
                    s.v.y = lp1.y * r_l;
                    s.v.z = lp1.z * r_l;
                    r_l = K_TWO_PI * rnd(s.t);
                    M::sincos(r_l, &sphi_l, &cphi_l);
                    rotatevector<EXACT>(s.v, 1.f, 0.f, sphi_l, cphi_l);
                }
            } else {
                if (lp2.x > 0.f || lp2.y > 0.f) {
                    float sphi_s, cphi_s;
                    r_l = K_TWO_PI * rnd(s.t);
                    M::sincos(r_l, &sphi_s, &cphi_s);
                    r_l = M::sqrt(2.f * rnd_scatlen<EXACT>(s.t));
                    cphi_s *= lp2.x * r_l;
                    sphi_s *= lp2.y * r_l;
                    sphi_s *= M::rsqrt(lp1.x * lp1.x + lp1.y * lp1.y + lp1.z * lp1.z);
                    s.prop.x = lp1.y * s.v.z - lp1.z * s.v.y;
                    s.prop.y = lp1.z * s.v.x - lp1.x * s.v.z;
                    s.prop.z = lp1.x * s.v.y - lp1.y * s.v.x;
                    s.prop.w = 0.f;
                    cphi_s *= M::rsqrt(s.prop.x * s.prop.x + s.prop.y * s.prop.y + s.prop.z * s.prop.z);
                    s.v.x += cphi_s * s.prop.x + sphi_s * lp1.x;
                    s.v.y += cphi_s * s.prop.y + sphi_s * lp1.y;
                    s.v.z += cphi_s * s.prop.z + sphi_s * lp1.z;
                    r_l = M::rsqrt(s.v.x * s.v.x + s.v.y * s.v.y + s.v.z * s.v.z);
                    s.v.x *= r_l;
                    s.v.y *= r_l;
                    s.v.z *= r_l;
                }
            }
            set_launch_voxel(a, ps, s);
            s.prop = make_float4(lpos.x + (lp1.x) * 0.5f, lpos.y + (lp1.y) * 0.5f, lpos.z + (lp1.z) * 0.5f, 0.f);
            s.Lmove = -1.f;
        }

        if (fabsf(s.p.w) <= c_p.minenergy) {
            continue;
        }

        if (c_p.nangle) {
            float ang, sth, cth, sphi, cphi;
            unsigned int na = c_p.nangle;
            if (ldir.w > 0.f) {
                ang = fminf(rnd(s.t) * (float)na, (float)na - K_EPS);
                cphi = ps.angle((int)(ang));
            } else {
                ang = fminf(rnd(s.t) * (float)(na - 1), (float)(na - 1) - K_EPS);
                sphi = ang - (float)((int)ang);
                unsigned int a0 = ((unsigned int)ang >= na - 1 ? na - 1 : (unsigned int)(int)(ang));
                unsigned int a1 = ((unsigned int)ang + 1 >= na - 1 ? na - 1 : (unsigned int)((int)(ang) + 1));
                cphi = ((1.f - sphi) * ps.angle(a0) + sphi * ps.angle(a1));
            }
            cphi *= K_ONE_PI;
            M::sincos(cphi, &sth, &cth);
            ang = K_TWO_PI * rnd(s.t);
            M::sincos(ang, &sphi, &cphi);
            if (ldir.w < 1.5f && ldir.w >= 0.f) {
                s.v = ldir;
            }
            rotatevector<EXACT>(s.v, sth, cth, sphi, cphi);
        } else if (s.Lmove < 0.f) {
            if (isnan(ldir.w)) {
                float ang, sth, cth, sphi, cphi;
                ang = K_TWO_PI * rnd(s.t);
                M::sincos(ang, &sphi, &cphi);
                ang = M::acos(2.f * rnd(s.t) - 1.f);
                M::sincos(ang, &sth, &cth);
                rotatevector<EXACT>(s.v, sth, cth, sphi, cphi);
            } else if (ldir.w < 0.f && isinf(ldir.w)) {
                float ang, sth, cth, sphi, cphi;
                ang = K_TWO_PI * rnd(s.t);
                M::sincos(ang, &sphi, &cphi);
                sth = M::sqrt(rnd(s.t));
                cth = M::sqrt(1.f - sth * sth);
                rotatevector<EXACT>(s.v, sth, cth, sphi, cphi);
            } else if (ldir.w != 0.f) {
                float Rn2 = (float)((ldir.w > 0.f) - (ldir.w < 0.f));
                s.prop.x += ldir.w * s.v.x;
                s.prop.y += ldir.w * s.v.y;
                s.prop.z += ldir.w * s.v.z;
                s.v.x = Rn2 * (s.prop.x - s.p.x);
                s.v.y = Rn2 * (s.prop.y - s.p.y);
                s.v.z = Rn2 * (s.prop.z - s.p.z);
                Rn2 = M::rsqrt(s.v.x * s.v.x + s.v.y * s.v.y + s.v.z * s.v.z);
                s.v.x *= Rn2;
                s.v.y *= Rn2;
                s.v.z *= Rn2;
            }
        }

        if ((s.mediaid & K_MED_MASK) == 0) {
            int idx = skipvoid<EXACT, SVMC>(a, ps, S, s.p, s.v, s.f, s.fx, s.fy, s.fz, s.fw);
            if (idx >= 0) {
                s.idx1d = (unsigned int)idx;
                s.mediaid = media_at(a, ps, s.idx1d);
            }
        }
        s.fx = (int)(short)floorf(s.p.x);
        s.fy = (int)(short)floorf(s.p.y);
        s.fz = (int)(short)floorf(s.p.z);

        s.w0 += 1.f;
        if (s.w0 > (float)c_p.maxvoidstep) {
            (*nfailed)++;
            return -1;
        }
        if (!((s.mediaid & K_MED_MASK) == 0 || fabsf(s.p.w) <= c_p.minenergy)) {
            break;
        }
    }

    s.f.w += 1.f;
    s.prop = ps.prop(S, 1);
    if (KP_SVMC) {
        updateprop_svmc<EXACT>(a, ps, S, s.prop, s.mediaid, s.idx1d, s.p, s.fx, s.fy, s.fz, s);
    } else {
        updateprop(ps, S, s.prop, s.mediaid);
    }
    if (!PS::kCommon && !PS::kBatch && a.maxjump) {
        save_traj(a, ps.p(), s, ps.cold()->srcsel, vt, false);      /* 2243-2249 */
    }
    ps.cold()->launched += s.p.w;
    s.w0 = s.p.w;
    if (!KP_SHARING) {
        ps.cold()->w0init = s.p.w;
    }
    s.v.w = K_EPS;
    s.Lmove = 0.f;
    if (KP_RFFWD) {
        /* the complex weight restarts with every launch (mcx_core.cl:2427-2430, 3011, 3054, ...) */
        s.wre = s.w0re = s.p.w;
        s.wim = s.w0im = 0.f;
    } else if (KP_RFREPLAY) {
        /* rf / rfmus replay (2257-2262): cos and sin of omega times the detected
           time of flight, read with the launch counter itself (the next photon,
           as the scattering-site outputs do: siteshift 1); the last photon reads
           the start time.  The reference stores them through its launch's
           partial-data-shifted pointer (1621), past the slots its deposits read,
           so its rf outputs come out zero; here they go where they are read. */
        long long k = replay_index(ps, vt, (long long)(int)s.f.w - 1 + (long long)c_p.siteshift);
        const float tof = (k >= 0 && k < (long long)c_p.nreplay) ? __ldg(a.rtof + k) : c_p.twin0;
        float rs, rc;
        M::sincos(c_p.omega * tof, &rs, &rc);
        ps.pp(c_p.partialdata) = rc;
        ps.pp(c_p.partialdata + 1) = rs;
    }
    return 0;
}

/* ------------------------------------------------------------------ kernel */

/* exit flag of a relaunch through a detecting face (mcx_core.cl:3001, 3181) */
template <class PS>
__device__ __forceinline__ unsigned int exit_detflag(const PS& ps, const Photon& s, unsigned int mediaidold) {
    const mcxg_kparams& c_p = ps.p();
    return (((s.idx1d == K_OUT_MAX && c_p.bc[9 + s.fw]) || (s.idx1d == K_OUT_MIN && c_p.bc[6 + s.fw]))
            ? K_OUT_MIN : (mediaidold & K_DET_MASK));
}

/* splitmix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number
   generators", OOPSLA 2014): seeds of a batch's reference threads */
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

template <class PS>
__device__ __forceinline__ void vt_begin(const KArgs& a, const PS& ps, const Shared& S, Photon& s, unsigned int vt) {
    const mcxg_kparams& c_p = ps.p();
    s.p = make_float4(0.f, 0.f, 0.f, __int_as_float(0x7fffffff));
    s.v = make_float4(0.f, 0.f, 0.f, 0.f);
    s.f = make_float4(0.f, 0.f, 0.f, 0.f);
    s.mediaid = __float_as_uint(c_p.srcparam2.w);
    s.isdet = 0;
    s.idx1d = 0;
    s.pathlen = 0.f;
    s.fx = s.fy = s.fz = 0;
    s.fw = -1;
    ps.cold()->esc = 0.f;
    ps.cold()->launched = 0.f;
    ps.cold()->w0init = 0.f;
    ps.cold()->srcsel = 0.f;
    if (PS::kBatch) {
        const unsigned long long k = ps.seed() ^ ((unsigned long long)vt << 1);
        s.t.a = splitmix64(k);
        s.t.b = splitmix64(k ^ 0xD1B54A32D192ED03ull);
    } else {
        uint4 sd = __ldg(a.seeds + vt);
        s.t.a = (unsigned long long)sd.x << 32 | sd.y;
        s.t.b = (unsigned long long)sd.z << 32 | sd.w;
    }
}

/* Next reference thread for this GPU thread: a global counter over the
   single simulation's threads, or over the concatenated threads of a batch
   (the simulation found by binary search in the prefix of thread counts). */
template <bool X, bool C>
__device__ __forceinline__ bool claim_vt(const KArgs& a, ConstPST<X, C>&, unsigned int& vt) {
    vt = atomicAdd(a.vtcounter, 1u);
    return vt < c_p.nthread;
}

/* A batch thread keeps claiming reference threads of the simulation it is
   in (one counter per simulation) and moves to the next open simulation only
   when that one is exhausted, so the lanes of a warp stay in the same
   simulation and read the same constant-memory descriptor.  A simulation is
   left only once its counter has run out, so every reference thread is
   claimed; `open` (the shared counter word) is one past the highest
   simulation found exhausted. */
template <bool C>
__device__ __forceinline__ bool claim_vt(const KArgs& a, BatchPST<C>& ps, unsigned int& vt) {
    for (;;) {
        if (ps.sid < a.nsim) {
            const unsigned int v = atomicAdd(a.simctr + ps.sid, 1u);
            if (v < c_sims[ps.sid].kp.nthread) {
                vt = v;
                return true;
            }
            atomicMax(a.vtcounter, ps.sid + 1);
        }
        const unsigned int open = *(volatile unsigned int*)a.vtcounter;
        const unsigned int next = open > ps.sid + 1 ? open : ps.sid + 1;
        if (next >= a.nsim) {
            return false;
        }
        ps.sid = next;
    }
}

/* Precision check: the same deposit into an FP64 field (the accumulation the
   two-plane field is measured against), a plain float field, and a float
   field with the reference's +-1000 spill into a shadow plane
   (mcx_core.cl:2880-2886), so all three see exactly the photons of the run. */
__device__ __forceinline__ void acc_verify(const KArgs& a, unsigned int planelen, unsigned int k, float w) {
    atomicAdd(a.acc64 + k, (double)w);
    atomicAdd(a.accf + k, w);
    const float o = atomicAdd(a.accs + k, w);
    if (fabsf(o) > K_MAX_ACCUM) {
        atomicAdd(a.accs + k, o > 0.f ? -K_MAX_ACCUM : K_MAX_ACCUM);
        atomicAdd(a.accs + planelen + k, o > 0.f ? K_MAX_ACCUM : -K_MAX_ACCUM);
    }
}

/* Fluence gradient.  For a loss L = sum_e c_e Phi_e of the raw field
   (c_e = dL/dPhi_e, Phi_e = sum of the flux deposits D_k = w0_k (1 -
   exp(-mua l_k)) / mua into element e), a photon's path does not depend on
   mua, and the weight entering voxel visit k carries exp(-sum_{j<k} mua_j
   l_j), so

     dL/dmua_u = sum_{visits k in u} [ c_k dD_k/dmua  -  l_k (J - P_k) ]

   with J = sum_k c_k D_k over the whole photon and P_k the same sum up to
   and including visit k (dD/dmua = (w l - D) / mua, or -w0 l^2 / 2 when mua
   is below EPS).  By the likelihood ratio of the free paths (density mus
   exp(-mus l) per scattering), the later deposits of a scattering in u gain
   1/mus_u and every path length in u costs -l:

     dL/dmus_u = sum_{scatterings in u} (J - P_before) / mus_u
                 - sum_{visits k in u} l_k (J - P_{k-1}).

   J is known only when the photon ends, so the photons run twice with the
   same random numbers: pass 1 stores each photon's J, pass 2 reads it at the
   launch and accumulates the gradients. */
/* Hot-voxel tile: the element of the box that voxel idx of gate tshift falls
   in, or 0xFFFFFFFF (the divisions are the host's exact multiply-shift pairs) */
__device__ __forceinline__ unsigned int tile_element(const KArgs& a, const mcxg_kparams& c_p, unsigned int idx,
                                                     int tshift) {
    const KArgs::Tile& t = a.tile;
    if (idx - t.lo >= t.span || (unsigned int)tshift >= t.ng) {
        return 0xFFFFFFFFu;
    }
    const unsigned int z = __umulhi(idx, t.mxy) >> t.sxy;
    const unsigned int r = idx - z * c_p.dimxy;
    const unsigned int y = __umulhi(r, t.mx) >> t.sx;
    const unsigned int x = r - y * c_p.dimx;
    const unsigned int ty = y - (unsigned int)t.y0, tx = x - (unsigned int)t.x0;
    if (ty >= t.ny || tx >= t.nx) {
        return 0xFFFFFFFFu;
    }
    return (((unsigned int)tshift * t.nz + (z - (unsigned int)t.z0)) * t.ny + ty) * t.nx + tx;
}

/* the block's tile: fixed-point counts, then remainders, in shared memory */
__device__ __forceinline__ unsigned long long* tile_counts(const KArgs& a) {
    return (unsigned long long*)((char*)mcxg_smem + a.tile.smemoff);
}

__device__ __forceinline__ unsigned int tile_size(const KArgs& a) {
    return a.tile.nx * a.tile.ny * a.tile.nz * a.tile.ng;
}

__device__ __forceinline__ size_t adj_slot(const mcxg_kparams& c_p, unsigned int vt, float fw) {
    return (size_t)vt * (c_p.threadphoton + 1u) + (unsigned int)((int)fw - 1);
}

template <bool EXACT, bool DET, bool REFL, bool WAGG, bool COUNT, int MINB, bool BATCH = false, bool XMEDIA = false,
          bool COMMON = false, bool RF = false, bool POL = false, bool SVMC = false, bool ACC64 = false,
          bool ADJ = false, bool TILE = false>
__global__ void __launch_bounds__(256, MINB) mcx_transport(const KArgs a) {
    typedef Mth<EXACT> M;
    typedef typename std::conditional<BATCH, BatchPST<COMMON>, ConstPST<XMEDIA, COMMON>>::type PS;
    PS ps;
    ps.init(a);
    Shared S;
    S.bprop = S.brecip = a.gprop;
    if (!BATCH) {
        /* stage the property table, its reciprocals and the inverse-CDF tables */
        for (unsigned int i = threadIdx.x; i < c_p.medianum; i += blockDim.x) {
            float4 q = a.gprop[i];
            mcxg_smem[i] = q;
            /* __fdividef(x, y) is x * rcp(y): keeping rcp(y) per medium gives the
               fast kernel the same bits with one MUFU op fewer per use */
            mcxg_smem[c_p.medianum + i] = make_float4(__fdividef(1.f, q.y), __fdividef(1.f, q.y * (1.f - q.z)),
                                                      __fdividef(1.f, q.x), __fdividef(1.f, 2.f * q.z));
        }
        float* tab = ps.tables();
        for (unsigned int i = threadIdx.x; i < c_p.nphase; i += blockDim.x) {
            tab[i] = a.invcdf[i];
        }
        for (unsigned int i = threadIdx.x; i < c_p.nangle; i += blockDim.x) {
            tab[c_p.nphase + i] = a.angleinvcdf[i];
        }
        __syncthreads();
    }

    unsigned long long cnt_step = 0, cnt_scat = 0, cnt_launch = 0, cnt_refl = 0, cnt_fail = 0;

    Photon s;
    unsigned int vt = 0;
    bool claimed = claim_vt(a, ps, vt);
    bool relaunch = false;         /* a relaunch request from the previous step */
    unsigned int relaunch_isdet = 0;
    bool fresh = true;             /* vt just claimed: initial launch */
    unsigned int mediaidold = 0, idx1dold = 0;
    unsigned int nsteps = 0;       /* steps of the current photon, against K_STEP_CAP */
    bool testint = false, hitintf = false;    /* split voxels: test the plane this step / the step ended on it */
    float adjJ = 0.f, adjP = 0.f;             /* fluence gradient: the photon's loss total and its running part */
    if (TILE) {
        /* the hot-voxel tile starts empty in every block */
        unsigned long long* tc = tile_counts(a);
        float* tr = (float*)(tc + tile_size(a));
        for (unsigned int i = threadIdx.x; i < tile_size(a); i += blockDim.x) {
            tc[i] = 0ull;
            tr[i] = 0.f;
        }
        __syncthreads();
    }

    while (claimed) {
        const mcxg_kparams& c_p = ps.p();
        const float gscat = (float)c_p.gscatter;
        if (fresh || relaunch) {
            int r;
            if (fresh) {
                vt_begin(a, ps, S, s, vt);
                testint = false;     /* each reference thread starts untested (2342) */
            }
            if (ADJ && !fresh && a.adjmode == 1u) {
                a.adjJ[adj_slot(c_p, vt, s.f.w)] = adjJ;        /* the photon that just ended */
            }
            /* one call site for the first and every later launch keeps the hot loop small */
            if (fresh && (unsigned long long)vt >= (unsigned long long)c_p.threadphoton * c_p.nthread + (unsigned int)c_p.oddphoton) {
                r = 1;
            } else {
                r = launchnewphoton<EXACT, DET, RF, POL, SVMC>(a, ps, S, s, fresh ? 0u : relaunch_isdet, vt, &cnt_fail);
                if (r && fresh) {
                    atomicAdd(a.status + ST_FAILED_LAUNCH, 1u);
                    r = 2;       /* NO_LAUNCH: the reference returns without writing energies */
                }
            }
            fresh = false;
            relaunch = false;
            if (r) {
                if (r != 2) {
                    a.energy[ps.vt_off() + vt] = make_float2(ps.cold()->esc, ps.cold()->launched);
                }
                claimed = claim_vt(a, ps, vt);
                fresh = true;
                continue;
            }
            if (COUNT) {
                cnt_launch++;
            }
            if (ADJ) {
                adjP = 0.f;
                adjJ = (a.adjmode == 2u) ? a.adjJ[adj_slot(c_p, vt, s.f.w)] : 0.f;
            }
            nsteps = 0;
            s.isdet = s.mediaid & K_DET_MASK;
            s.mediaid &= K_MED_MASK;
        }
        if (++nsteps > K_STEP_CAP) {
            atomicAdd(a.status + ST_GUARD, 1u);
            relaunch = true;
            relaunch_isdet = 0;
            continue;
        }

        if (COUNT) {
            cnt_step++;
        }
        /* ---- scattering (mcx_core.cl:2446-2649) */
        if (s.f.x <= 0.f) {
            s.f.x = rnd_scatlen<EXACT>(s.t);
            if (s.v.w != K_EPS) {
                float cphi = 1.f, sphi = 0.f, theta, stheta, ctheta, tmp0 = 0.f;
                if (COUNT) {
                    cnt_scat++;
                }
                float polphi = 0.f;
                if (KP_POL) {
                    /* polarised: angles from the Mueller matrix (2454-2469) */
                    pol_angles<EXACT>(a, s, theta, polphi);
                    M::sincos(polphi, &sphi, &cphi);
                    M::sincos(theta, &stheta, &ctheta);
                } else {
                if (!KP_IS2D) {
                    tmp0 = K_TWO_PI * rnd(s.t);
                    M::sincos(tmp0, &sphi, &cphi);
                }
                if (KP_NPHASE_GT2) {
                    unsigned int np = c_p.nphase;
                    tmp0 = rnd(s.t) * (float)(np - 1);
                    theta = tmp0 - (float)((int)tmp0);
                    unsigned int i0 = (unsigned int)tmp0 >= np ? np - 1 : (unsigned int)(int)(tmp0);
                    unsigned int i1 = (unsigned int)tmp0 + 1 >= np ? np - 1 : (unsigned int)((int)(tmp0) + 1);
                    tmp0 = (1.f - theta) * ps.invcdf(i0) + theta * ps.invcdf(i1);
                    if (EXACT) {
                        theta = M::acos(tmp0);
                        stheta = M::sin(theta);
                    } else {
                        stheta = M::sqrt(fmaxf(0.f, 1.f - tmp0 * tmp0));
                    }
                    ctheta = tmp0;
                } else {
                    tmp0 = (s.v.w > (float)c_p.gscatter) ? 0.f : s.prop.z;
                    if (fabsf(tmp0) > K_EPS) {
                        /* Henyey-Greenstein, mcx_core.cl:2487-2493 */
                        tmp0 = (1.f - s.prop.z * s.prop.z) / (1.f - s.prop.z + 2.f * s.prop.z * rnd(s.t));
                        tmp0 *= tmp0;
                        if (EXACT || KP_MEDIAFORMAT > 4) {
                            tmp0 = M::div(1.f + s.prop.z * s.prop.z - tmp0, 2.f * s.prop.z);
                        } else {
                            /* __fdividef(a, 2g) == a * rcp(2g): the label's rcp(2g) is staged */
                            tmp0 = (1.f + s.prop.z * s.prop.z - tmp0) * ps.recip(S, s.mediaid & K_MED_MASK).w;
                        }
                        tmp0 = fmaxf(-1.f, fminf(1.f, tmp0));
                        if (EXACT) {
                            theta = M::acos(tmp0);
                            stheta = M::sin(theta);
                        } else {
                            stheta = M::sqrt(1.f - tmp0 * tmp0);
                        }
                        ctheta = tmp0;
                    } else {
                        if (EXACT) {
                            theta = M::acos(2.f * rnd(s.t) - 1.f);
                            M::sincos(theta, &stheta, &ctheta);
                        } else {
                            ctheta = 2.f * rnd(s.t) - 1.f;
                            stheta = M::sqrt(1.f - ctheta * ctheta);
                        }
                    }
                }
                }
                /* a split voxel records under the label of the photon's side (2507-2535) */
                const unsigned int slab = KP_SVMC ? SV_CURLABEL(s.sv) : (s.mediaid & K_MED_MASK);
                if (DET && c_p.savedet && slab - 1u < c_p.maxmedia) {
                    unsigned int med = slab - 1;
                    if (SAVE_NSCAT(c_p.savedetflag)) {
                        float* q = &ps.pp(med);
                        *q = __uint_as_float(__float_as_uint(*q) + 1u);
                    }
                    if (SAVE_MOM(c_p.savedetflag)) {
                        ps.pp(c_p.maxmedia * (SAVE_NSCAT(c_p.savedetflag) + SAVE_PPATH(c_p.savedetflag)) + med) += 1.f - ctheta;
                    }
                }
                const float3 olddir = make_float3(s.v.x, s.v.y, s.v.z);
                if (KP_IS2D) {
                    rotatevector2d<EXACT>(s.v, (rnd(s.t) > 0.5f ? stheta : -stheta), ctheta, KP_IS2D);
                } else {
                    rotatevector<EXACT>(s.v, stheta, ctheta, sphi, cphi);
                }
                s.v.w += 1.f;
                if (ADJ && a.adjmode == 2u && s.idx1d < c_p.nvox) {
                    /* a scattering in this voxel: 1/mus on every later deposit */
                    atomicAdd(a.field + c_p.fieldlen + s.idx1d, (adjJ - adjP) * __fdividef(1.f, s.prop.y));
                }
                if (KP_POL) {
                    update_stokes<EXACT>(a, s, theta, polphi, olddir, s.v);
                }
                if (c_p.replay && (c_p.outputtype == otWP || c_p.outputtype == otDCS || c_p.outputtype == otWPTOF ||
                                   c_p.outputtype == otRFmus)) {
                    replay_site_deposit(a, ps, S, s, vt, ctheta);
                }
                if (!PS::kCommon && !PS::kBatch && a.maxjump) {
                    save_traj(a, c_p, s, ps.cold()->srcsel, vt, false);      /* 2625-2634 */
                }
            }
            s.v.w = (float)(int)s.v.w;
            if (KP_SVMC) {
                testint = true;      /* 2641-2647 */
            }
        }

        s.n1 = s.prop.w;
        if (KP_SVMC) {
            updateprop_svmc<EXACT>(a, ps, S, s.prop, s.mediaid, s.idx1d, s.p, s.fx, s.fy, s.fz, s);
        } else {
            updateprop(ps, S, s.prop, s.mediaid);
        }

        /* ---- move to the next voxel face or the end of the free path */
        if (EXACT) {
            s.f.z = hitgrid<EXACT>(s.p, s.v, s.fx, s.fy, s.fz, s.fw);
        } else {
            /* the reciprocals of the direction, every step: three MUFU ops are
               cheaper than the four registers a cache of them held across the
               loop (cube + sphere 3 %, head 4 % faster at the 64-register cap) */
            const float3 rv = make_float3(__fdividef(1.f, s.v.x), __fdividef(1.f, s.v.y), __fdividef(1.f, s.v.z));
            s.f.z = hitgrid_rcp(s.p, s.v, rv, s.fx, s.fy, s.fz, s.fw);
        }
        {
            const bool reduced = s.v.w + 1.f > gscat;
            float slen = s.f.z * s.prop.y * (reduced ? (1.f - s.prop.z) : 1.f);
            slen = fminf(slen, s.f.x);
            if (EXACT || KP_MEDIAFORMAT > 4) {
                s.f.z = M::div(slen, s.prop.y * (reduced ? (1.f - s.prop.z) : 1.f));
            } else {
                const float4 rc = ps.recip(S, s.mediaid & K_MED_MASK);
                s.f.z = slen * (reduced ? rc.y : rc.x);
            }
            hitintf = false;
            if (KP_SVMC && SV_ISSPLIT(s.sv) && testint) {
                /* the voxel's plane cuts the step short (2687-2702) */
                hitintf = ray_plane_intersect<EXACT>(s, gscat, s.f.z, slen);
            }
            s.pathlen += s.f.z;
            s.p.x = s.p.x + s.f.z * s.v.x;
            s.p.y = s.p.y + s.f.z * s.v.y;
            s.p.z = s.p.z + s.f.z * s.v.z;
            bool scat_here = (slen == s.f.x) || hitintf;
            if (s.fw == 0) {
                s.fx += scat_here ? 0 : (s.v.x > 0.f ? 1 : -1);
            }
            if (s.fw == 1) {
                s.fy += scat_here ? 0 : (s.v.y > 0.f ? 1 : -1);
            }
            if (s.fw == 2) {
                s.fz += scat_here ? 0 : (s.v.z > 0.f ? 1 : -1);
            }
            if (KP_RFFWD) {
                /* RF transport (mcx_core.cl:2750-2760): w <- w exp(-(mua + i omega n / c0) ds) */
                const float att = M::exp(-s.prop.x * s.f.z);
                float rs, rc;
                M::sincos(c_p.omega * s.prop.w * c_p.oneoverc0 * s.f.z, &rs, &rc);
                const float tre = att * (s.wre * rc + s.wim * rs);
                const float tim = att * (-s.wre * rs + s.wim * rc);
                s.wre = tre;
                s.wim = tim;
                s.p.w = M::sqrt(s.wre * s.wre + s.wim * s.wim);
            } else {
                s.p.w *= M::exp(-s.prop.x * s.f.z);
            }
            s.f.x -= slen;
            s.f.y += s.f.z * s.prop.w * c_p.oneoverc0;
        }
        /* a photon in a label-0 voxel (entered from a medium of the same index)
           has no partial-path slot; the reference writes one slot early there */
        {
            const unsigned int plab = KP_SVMC ? SV_CURLABEL(s.sv) : (s.mediaid & K_MED_MASK);
            if (DET && c_p.savedet && SAVE_PPATH(c_p.savedetflag) && plab - 1u < c_p.maxmedia) {
                ps.pp(c_p.maxmedia * SAVE_NSCAT(c_p.savedetflag) + plab - 1) += s.f.z;
            }
        }

        /* ---- new voxel (mcx_core.cl:2795-2811) */
        mediaidold = s.mediaid | s.isdet;
        idx1dold = s.idx1d;
        s.idx1d = vox_index(ps, s.fx, s.fy, s.fz);
        if (!inside_u(ps, s.fx, s.fy, s.fz)) {
            s.mediaid = 0;
            s.idx1d = (s.fx < 0 || s.fy < 0 || s.fz < 0) ? K_OUT_MIN : K_OUT_MAX;
            s.isdet = c_p.bc[(s.idx1d == K_OUT_MAX) * 3 + s.fw];
            s.isdet = ((s.isdet & 0xF) == bcUnknown) ? (c_p.doreflect ? bcReflect : bcAbsorb) : s.isdet;
        } else {
            s.mediaid = media_at(a, ps, s.idx1d);
            s.isdet = s.mediaid & K_DET_MASK;
            s.mediaid &= K_MED_MASK;
        }

        /* ---- deposit on a voxel change (mcx_core.cl:2816-2929) */
        {
            bool dep = false, depim = false;
            unsigned int key = 0;
            float weight = 0.f, weight_im = 0.f;
            if ((s.idx1d != idx1dold || hitintf) && idx1dold < c_p.nvox && mediaidold) {
                if (c_p.save2pt && s.f.y >= c_p.twin0 && s.f.y < c_p.twin1) {
                    int tshift = (int)(floorf((s.f.y - c_p.twin0) * c_p.Rtstep));
                    if (KP_RFFWD) {
                        /* RF transport (2833-2840): (w0 - w) / (mua + i omega n / c0) */
                        const float dre = s.w0re - s.wre, dim = s.w0im - s.wim;
                        const float aim = c_p.omega * s.prop.w * c_p.oneoverc0;
                        const float am2 = s.prop.x * s.prop.x + aim * aim;
                        weight = (am2 < K_EPS) ? (s.w0re * s.pathlen) : M::div(dre * s.prop.x + dim * aim, am2);
                        weight_im = (am2 < K_EPS) ? (s.w0im * s.pathlen) : M::div(dim * s.prop.x - dre * aim, am2);
                        depim = fabsf(weight) > 0.f;
                    } else if (c_p.outputtype == otEnergy) {
                        weight = s.w0 - s.p.w;
                    } else if (c_p.outputtype == otFluence || c_p.outputtype == otFlux || c_p.outputtype >= otAdjoint) {
                        if (EXACT || KP_MEDIAFORMAT > 4) {
                            weight = (s.prop.x < K_EPS) ? (s.w0 * s.pathlen) : M::div(s.w0 - s.p.w, s.prop.x);
                        } else {
                            /* prop still holds the medium the photon deposited in */
                            weight = (s.prop.x < K_EPS) ? (s.w0 * s.pathlen)
                                     : (s.w0 - s.p.w) * ps.recip(S, mediaidold & K_MED_MASK).z;
                        }
                    } else if (c_p.replay) {
                        /* replay Jacobian (mcx_core.cl:2845-2858): detected weight times
                           the path length in the voxel, gated by the detected time of flight */
                        if (c_p.outputtype == otJacobian || c_p.outputtype == otRF || c_p.outputtype == otWLTOF) {
                            long long k = replay_index(ps, vt, (long long)(int)s.f.w - 1);
                            if (k >= 0 && k < (long long)c_p.nreplay) {
                                float rt = __ldg(a.rtof + k);
                                int d = __ldg(a.rdetid + k) & 0xFFFF;
                                weight = __ldg(a.rweight + k) * s.pathlen;
                                tshift = (int)(floorf((rt - c_p.twin0) * c_p.Rtstep)) +
                                         ((c_p.replaydet == -1) ? ((d - 1) * (int)c_p.maxgate) : 0);
                                if (c_p.outputtype == otWLTOF) {
                                    weight = weight * rt;
                                }
                                if (tshift < 0 || (c_p.replaydet == -1 && (d < 1 || d > (int)c_p.detnum))) {
                                    /* the host filters these out; never index with them */
                                    atomicAdd(a.status + ST_GUARD, 1u);
                                    weight = 0.f;
                                    tshift = 0;
                                } else if (c_p.outputtype == otRF) {
                                    /* 2853-2855, 2875-2877: times cos / sin of the launch phase,
                                       deposited here (even when zero, as the reference does) */
                                    rf_replay_deposit(a, ps, idx1dold, tshift, -weight * ps.pp(c_p.partialdata),
                                                      -__ldg(a.rweight + k) * s.pathlen * ps.pp(c_p.partialdata + 1));
                                    weight = 0.f;
                                }
                            }
                        }
                    } else if (c_p.outputtype == otL) {
                        weight = s.w0 * s.pathlen;
                    }
                    if (c_p.extrasrclen && (c_p.srcid < 0)) {
                        tshift += ((int)ps.cold()->srcsel - 1) * ((c_p.replay && c_p.replaydet == -1) ? (int)c_p.detnum : 1) *
                                  (int)c_p.maxgate;
                    }
                    dep = fabsf(weight) > 0.f;
                    key = idx1dold + (unsigned int)tshift * c_p.nvox;
                    /* a time of flight a rounding below twin1 can give tshift == maxgate;
                       the reference then writes into its shadow half, which its host adds
                       to gate 0 -- the low plane here plays that role */
                    if (key >= c_p.fieldlen) {
                        key -= c_p.fieldlen;
                    }
                    if (TILE && dep) {
                        /* an element of the hot-voxel tile: the same split, into shared memory */
                        const unsigned int te = tile_element(a, c_p, idx1dold, tshift);
                        if (te != 0xFFFFFFFFu) {
                            long long k;
                            float r;
                            field_split(field_of(a, ps, 0), weight, k, r);
                            unsigned long long* tc = tile_counts(a);
                            if (k) {
                                atomicAdd(tc + te, (unsigned long long)k);
                            }
                            if (r != 0.f) {
                                atomicAdd((float*)(tc + tile_size(a)) + te, r);
                            }
                            dep = false;
                        }
                    }
                }
                if (ADJ) {
                    /* the visit that just ended, in voxel idx1dold */
                    const float c = dep ? __ldg(a.adjc + key) : 0.f;
                    const float cD = c * weight;
                    if (a.adjmode == 1u) {
                        adjJ += cD;
                    } else {
                        const float l = s.pathlen, rest = adjJ - adjP;
                        float own = 0.f;
                        if (dep) {
                            own = (s.prop.x < K_EPS) ? -0.5f * c * s.w0 * l * l
                                                     : c * (s.p.w * l - weight) * __fdividef(1.f, s.prop.x);
                        }
                        atomicAdd(a.field + idx1dold, own - l * (rest - cD));
                        atomicAdd(a.field + c_p.fieldlen + idx1dold, -l * rest);
                        adjP += cD;
                    }
                    dep = false;
                }
                s.w0 = s.p.w;
                if (KP_RFFWD) {
                    s.w0re = s.wre;
                    s.w0im = s.wim;
                }
                s.pathlen = 0.f;
            } else {
                s.mediaid = mediaidold;
            }
            if (KP_SHARING) {
                if (dep) {
                    share_deposit(a, ps, key, weight);
                }
            } else {
                deposit<WAGG>(field_of(a, ps, 0), dep, ps.field_off() + key, weight);
                if (ACC64 && dep) {
                    acc_verify(a, ps.lo_plane(), ps.field_off() + key, weight);
                }
            }
            if (RF && depim) {
                /* the imaginary component's planes follow the real one's: [3F, 6F) */
                field_add(field_of(a, ps, 1), key, weight_im);
            }
        }
        if (KP_SVMC) {
            /* the side of the plane after a voxel change or a plane crossing (2934-2950) */
            if (s.idx1d != idx1dold) {
                updateprop_svmc<EXACT>(a, ps, S, s.prop, s.mediaid, s.idx1d, s.p, s.fx, s.fy, s.fz, s);
                testint = true;
            } else if (hitintf) {
                s.nv = make_float3(-s.nv.x, -s.nv.y, -s.nv.z);
                s.pd = -s.pd;
                s.sv ^= 1u << 17;
                testint = false;
            }
        }

        /* ---- exit, time-out or cyclic boundary, or a background half of a split
           voxel (mcx_core.cl:2958-3028) */
        if ((s.mediaid == 0 && ((s.isdet & 0xF) == bcAbsorb || (s.isdet & 0xF) == bcCyclic ||
                                ((s.isdet & 0xF) == bcReflect && s.n1 == ps.prop(S, 0).w))) ||
                (KP_SVMC && (s.idx1d != idx1dold || hitintf) && !SV_ISUPPER(s.sv) && !SV_LOWER(s.sv) &&
                 (!c_p.doreflect || s.n1 == ps.prop(S, 0).w)) ||
                s.f.y > c_p.twin1) {
            if (s.isdet == bcCyclic) {
                if (s.fw == 0) {
                    s.p.x = nextafter_ref(rintf(((s.idx1d == K_OUT_MIN) ? c_p.maxidx.x : 0)), (s.v.x > 0.f) - (s.v.x < 0.f));
                    s.fx = (int)(short)floorf(s.p.x);
                }
                if (s.fw == 1) {
                    s.p.y = nextafter_ref(rintf(((s.idx1d == K_OUT_MIN) ? c_p.maxidx.y : 0)), (s.v.y > 0.f) - (s.v.y < 0.f));
                    s.fy = (int)(short)floorf(s.p.y);
                }
                if (s.fw == 2) {
                    s.p.z = nextafter_ref(rintf(((s.idx1d == K_OUT_MIN) ? c_p.maxidx.z : 0)), (s.v.z > 0.f) - (s.v.z < 0.f));
                    s.fz = (int)(short)floorf(s.p.z);
                }
                if (inside_u(ps, s.fx, s.fy, s.fz)) {
                    s.idx1d = vox_index(ps, s.fx, s.fy, s.fz);
                    s.mediaid = media_at(a, ps, s.idx1d);
                    s.isdet = s.mediaid & K_DET_MASK;
                    s.mediaid &= K_MED_MASK;
                    continue;
                }
            }
            relaunch = true;
            relaunch_isdet = exit_detflag(ps, s, mediaidold);
            if (KP_SVMC) {
                testint = true;      /* 3019-3023 */
            }
            continue;
        }

        /* ---- Russian roulette (mcx_core.cl:3031-3061) */
        if (fabsf(s.p.w) < c_p.minenergy) {
            if (rnd(s.t) * K_ROULETTE <= 1.f) {
                s.p.w *= K_ROULETTE;
                if (KP_RFFWD) {
                    s.wre *= K_ROULETTE;
                    s.wim *= K_ROULETTE;
                    s.w0re *= K_ROULETTE;
                    s.w0im *= K_ROULETTE;
                }
            } else {
                relaunch = true;
                relaunch_isdet = mediaidold & K_DET_MASK;
                continue;
            }
        }

        /* ---- Fresnel reflection / refraction (mcx_core.cl:3126-3278) */
        /* within the same voxel the medium and index are unchanged, so the test
           below cannot fire -- except for the encodings from 100 on, whose test
           compares with row 1's index rather than the voxel's */
        if (REFL && KP_SVMC && c_p.dorefl_compiled && hitintf) {
            /* Fresnel at a split voxel's plane (mcx_core.cl:3065-3115) */
            if (ps.prop(S, SV_LOWER(s.sv)).w != ps.prop(S, SV_UPPER(s.sv)).w) {
                float3 c0 = make_float3(s.v.x, s.v.y, s.v.z);
                s.nv = make_float3(-s.nv.x, -s.nv.y, -s.nv.z);
                s.pd = -s.pd;
                if (reflectray_svmc<EXACT>(ps, S, s, s.n1, c0)) {
                    relaunch = true;
                    relaunch_isdet = mediaidold & K_DET_MASK;
                    testint = true;
                    continue;
                }
                s.v.x = c0.x, s.v.y = c0.y, s.v.z = c0.z;
            } else {
                s.prop = ps.prop(S, SV_CURLABEL(s.sv));
            }
        } else if (REFL && c_p.dorefl_compiled &&
                   (KP_SVMC || s.idx1d != idx1dold || (PS::kXMedia && KP_MEDIAFORMAT >= 100))) {
            /* a split voxel's side already holds its properties (the OpenCL
               kernel's update of the label is empty for that encoding); the side
               is recomputed from the position every step, so the index can change
               without a voxel change and the test runs every step there */
            if (!KP_SVMC) {
                updateprop(ps, S, s.prop, s.mediaid);
            }
            if (((s.mediaid && c_p.doreflect) ||
                 (s.mediaid == 0 && (((s.isdet & 0xF) == bcUnknown && c_p.doreflect) ||
                                     ((s.isdet & 0xF) == bcReflect || (s.isdet & 0xF) == bcMirror)))) &&
                (((s.isdet & 0xF) == bcMirror) ||
                 s.n1 != ((KP_MEDIAFORMAT < 100) ? (s.prop.w)
                          : (ps.prop(S, (s.mediaid > 0 && KP_MEDIAFORMAT >= 100) ? 1 : s.mediaid).w)))) {
                float Rtotal = 1.f;
                if (COUNT) {
                    cnt_refl++;
                }
                float tmp0 = s.n1 * s.n1;
                float tmp1 = s.prop.w * s.prop.w;
                float cphi = fabsf(vcomp(s.v, s.fw));
                float sphi = 1.f - cphi * cphi;
                s.f.z = 1.f - M::div(tmp0, tmp1) * sphi;
                if (s.f.z > 0.f && (s.isdet & 0xF) != bcMirror) {
                    float ctheta = tmp0 * cphi * cphi + tmp1 * s.f.z;
                    float stheta = 2.f * s.n1 * s.prop.w * cphi * M::sqrt(s.f.z);
                    Rtotal = M::div(ctheta - stheta, ctheta + stheta);
                    ctheta = tmp1 * cphi * cphi + tmp0 * s.f.z;
                    Rtotal = (Rtotal + M::div(ctheta - stheta, ctheta + stheta)) * 0.5f;
                }
                if (Rtotal < 1.f && (!(s.mediaid == 0 && ((s.isdet & 0xF) == bcMirror))) && rnd(s.t) > Rtotal) {
                    transmit<EXACT>(s.v, s.n1, s.prop.w, s.fw);
                    if (s.mediaid == 0) {
                        relaunch = true;
                        relaunch_isdet = exit_detflag(ps, s, mediaidold);
                        continue;
                    }
                } else {
                    if (s.fw == 0) {
                        s.v.x = -s.v.x;
                        s.p.x = nextafter_ref(rintf(s.p.x), (int)((float)(s.v.x > 0.f) - 0.5f));
                        s.fx = (int)(short)rintf(s.p.x);
                    } else if (s.fw == 1) {
                        s.v.y = -s.v.y;
                        s.p.y = nextafter_ref(rintf(s.p.y), (int)((float)(s.v.y > 0.f) - 0.5f));
                        s.fy = (int)(short)rintf(s.p.y);
                    } else {
                        s.v.z = -s.v.z;
                        s.p.z = nextafter_ref(rintf(s.p.z), (int)((float)(s.v.z > 0.f) - 0.5f));
                        s.fz = (int)(short)rintf(s.p.z);
                    }
                    if (idx1dold >= c_p.nvox) {
                        /* unreachable for a photon that came from inside the volume */
                        atomicAdd(a.status + ST_GUARD, 1u);
                        relaunch = true;
                        relaunch_isdet = 0;
                        continue;
                    }
                    s.idx1d = idx1dold;
                    unsigned int m = media_at(a, ps, s.idx1d);
                    s.mediaid = m & K_MED_MASK;
                    /* take the detector bit of the voxel the photon is back in (the
                       reference keeps the face code here, which mcx_core.cl:2796 then
                       ORs into the medium index) */
                    s.isdet = m & K_DET_MASK;
                    if (KP_SVMC) {
                        /* back in the voxel it came from: its side of the plane
                           (mcx_core.cl:3218-3236, the OpenCL kernel keeps testint) */
                        updateprop_svmc<EXACT>(a, ps, S, s.prop, s.mediaid, s.idx1d, s.p, s.fx, s.fy, s.fz, s);
                        if (SV_CURLABEL(s.sv) == 0) {
                            relaunch = true;
                            relaunch_isdet = mediaidold & K_DET_MASK;
                            continue;
                        }
                    } else {
                        updateprop(ps, S, s.prop, s.mediaid);
                    }
                    s.n1 = s.prop.w;
                }
            }
        }
    }

    if (TILE) {
        /* the block's tile into the field: one pair of atomics per touched element */
        __syncthreads();
        const mcxg_kparams& kp = ps.p();
        const Field f = field_of(a, ps, 0);
        const unsigned long long* tc = tile_counts(a);
        const float* tr = (const float*)(tc + tile_size(a));
        const KArgs::Tile& t = a.tile;
        for (unsigned int i = threadIdx.x; i < tile_size(a); i += blockDim.x) {
            const unsigned long long c = tc[i];
            const float r = tr[i];
            if (c || r != 0.f) {
                unsigned int j = i;
                const unsigned int x = j % t.nx;
                j /= t.nx;
                const unsigned int y = j % t.ny;
                j /= t.ny;
                const unsigned int z = j % t.nz;
                const unsigned int g = j / t.nz;
                const size_t key = ps.field_off() + (size_t)((unsigned int)t.z0 + z) * kp.dimxy +
                                   ((unsigned int)t.y0 + y) * kp.dimx + ((unsigned int)t.x0 + x) + (size_t)g * kp.nvox;
                field_commit(f, key, (long long)c, r);
            }
        }
    }

    if (COUNT) {
        atomicAdd(a.counters + 0, cnt_step);
        atomicAdd(a.counters + 1, cnt_scat);
        atomicAdd(a.counters + 2, cnt_launch);
        atomicAdd(a.counters + 3, cnt_refl);
        atomicAdd(a.counters + 4, cnt_fail);
    }
}

/* -D R: each reference thread writes its RNG stream into the field
   (mcx_core.cl:2408-2414) */
__global__ void mcx_rng_dump(const KArgs a) {
    for (unsigned int vt = blockIdx.x * blockDim.x + threadIdx.x; vt < c_p.nthread; vt += gridDim.x * blockDim.x) {
        if ((unsigned long long)vt >= (unsigned long long)c_p.threadphoton * c_p.nthread + (unsigned int)c_p.oddphoton) {
            continue;
        }
        uint4 sd = a.seeds[vt];
        Rng t;
        t.a = (unsigned long long)sd.x << 32 | sd.y;
        t.b = (unsigned long long)sd.z << 32 | sd.w;
        for (unsigned int j = vt; j < c_p.fieldlen; j += c_p.nthread) {
            a.flo[j] = rnd(t);
        }
    }
}

}  // namespace
}  // namespace mcxg

#undef KP_IS2D
#undef KP_NPHASE_GT2
#undef KP_MEDIAFORMAT
#undef KP_SHARING
#undef KP_RFFWD
#undef KP_RFREPLAY
#undef KP_POL
#undef KP_SVMC

#endif
