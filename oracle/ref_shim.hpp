/*
 * ref_shim.hpp -- host C++ environment for compiling the reference kernel
 * source (src/mcx_core.cl, its __NVCC__ branch) unmodified on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  Used by oracle/ref_harness.cpp, built by
 * oracle/Makefile into oracle/_ref/ (never committed, never shipped).  The
 * reference source is read where it lies; nothing from it is copied here.
 *
 * The __NVCC__ branch expects CUDA's vector types, a handful of device
 * intrinsics, the CUDA thread-index built-ins and a constant parameter block
 * `gcfg_const`; this header supplies host equivalents.  The struct and enum
 * names below are interface names the kernel source refers to (its MCXParam
 * fields are listed in mcx_core.cl:611-663 / mcx_host.h:106-166).
 */
#ifndef MCX_REF_SHIM_HPP
#define MCX_REF_SHIM_HPP

#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <math.h>
#include <sys/types.h>

#include <vector_types.h>
#include <vector_functions.h>
#include <cuda_fp16.h>

#define __global__
#define __device__
#define __shared__
#define __constant__

typedef unsigned long long RandType;

/* CUDA thread-index built-ins and the dynamic shared-memory block, set by the
   harness before each call.  Plain globals: the harness runs one reference
   thread at a time (a thread_local here would make g++ emit an unguarded
   call to a weak TLS initialiser for the kernel's block-scope extern
   declaration of an incomplete array). */
uint3 threadIdx;
uint3 blockIdx;
uint3 blockDim;
uint3 gridDim;
char sharedmem_raw[1 << 17];

static inline void __syncthreads(void) {}

static inline float rsqrtf(float x) { return 1.f / sqrtf(x); }
static inline float __fdividef(float a, float b) { return a / b; }
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }

static inline float atomicAdd(float* addr, float val) {
    return std::atomic_ref<float>(*addr).fetch_add(val);
}
static inline unsigned int atomicAdd(unsigned int* addr, unsigned int val) {
    return std::atomic_ref<unsigned int>(*addr).fetch_add(val);
}
static inline unsigned int atomicSub(unsigned int* addr, unsigned int val) {
    return std::atomic_ref<unsigned int>(*addr).fetch_sub(val);
}

/* Source-type ids (mcx_const.h:62-80) as enum constants, not macros: the
   kernel source also tests `#if defined(MCX_SRC_PATTERN)` as the OpenCL JIT
   flag for the pattern-source deposit path (mcx_core.cl:1513, 2881).  With
   the ids as macros (as mcx_const.h has them) the __NVCC__ branch would always
   take that path and deposit nothing for other sources; as enum constants the
   host build follows the OpenCL build for every non-pattern source.  The
   build for pattern sources (MCXREF_PATTERN_BUILD) makes the two pattern ids
   macros, as the OpenCL JIT flags them for a pattern source, so the kernel
   takes its photon-sharing deposit path. */
enum {
    MCX_SRC_PENCIL = 0, MCX_SRC_ISOTROPIC = 1, MCX_SRC_CONE = 2, MCX_SRC_GAUSSIAN = 3, MCX_SRC_PLANAR = 4,
#ifndef MCXREF_PATTERN_BUILD
    MCX_SRC_PATTERN = 5,
    MCX_SRC_PATTERN3D = 15,
#endif
    MCX_SRC_FOURIER = 6, MCX_SRC_ARCSINE = 7, MCX_SRC_DISK = 8, MCX_SRC_FOURIERX = 9,
    MCX_SRC_FOURIERX2D = 10, MCX_SRC_ZGAUSSIAN = 11, MCX_SRC_LINE = 12, MCX_SRC_SLIT = 13,
    MCX_SRC_PENCILARRAY = 14, MCX_SRC_HYPERBOLOID_GAUSSIAN = 16, MCX_SRC_RING = 17
};
#ifdef MCXREF_PATTERN_BUILD
#define MCX_SRC_PATTERN 5
#define MCX_SRC_PATTERN3D 15
#endif

enum TBoundary {bcUnknown, bcReflect, bcAbsorb, bcMirror, bcCyclic};
enum TOutputType {otFlux, otFluence, otEnergy, otJacobian, otWP, otDCS, otRF, otL, otRFmus, otWLTOF, otWPTOF,
                  otAdjoint, otAdjointDcoeff, otAdjointMus, otAdjointMusp, otAdjointMuaD, otAdjointMuaMusp
                 };
#define MCX_IS_ADJOINT_TYPE(t)      ((int)(t) >= (int)otAdjoint)

typedef struct StokesVector {
    float i, q, u, v;
} Stokes;

typedef struct MCXSource {
    float4 pos, dir, param1, param2;
} MCXSrc;

typedef struct KernelParams {
    MCXSrc src;
    unsigned int extrasrclen;
    int srcid;
    float4 maxidx;
    uint4 dimlen, cp0, cp1;
    uint2 cachebox;
    float minstep;
    float twin0, twin1, tmax;
    float oneoverc0;
    unsigned int isrowmajor, save2pt, doreflect, dorefint, savedet;
    float Rtstep;
    float minenergy;
    float skipradius2;
    float minaccumtime;
    unsigned int maxdetphoton;
    unsigned int maxmedia;
    unsigned int detnum;
    unsigned int blockphoton;
    unsigned int blockextra;
    int voidtime;
    int srctype;
    unsigned int maxvoidstep;
    unsigned int issaveexit;
    unsigned int issaveseed;
    unsigned int issaveref;
    unsigned int isspecular;
    unsigned int maxgate;
    int seed;
    unsigned int outputtype;
    unsigned int threadphoton;
    int oddphoton;
    unsigned int debuglevel;
    unsigned int savedetflag;
    unsigned int reclen;
    unsigned int partialdata;
    unsigned int w0offset;
    unsigned int mediaformat;
    unsigned int maxjumpdebug;
    unsigned int gscatter;
    unsigned int is2d;
    int replaydet;
    unsigned int srcnum;
    unsigned int nphase;
    unsigned int nphaselen;
    unsigned int nangle;
    unsigned int nanglelen;
    unsigned int maxpolmedia;
    unsigned int istrajstokes;
    float4 s0;
    float omega;
    unsigned char bc[12];
} MCXParam;

MCXParam gcfg_const[1];

/* JIT flags the reference host passes for this configuration
   (mcx_host.cpp:886-892): atomic float deposits and detector capture */
#define USE_ATOMIC 1
#define MCX_SAVE_DETECTORS 1

#define __NVCC__ 1

#endif
