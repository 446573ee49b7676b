/*
 * mcx_kparams.h -- the transport kernel's constant parameter block.
 *
 * Plain C so the C host driver and the CUDA translation units share one
 * definition.  Field meanings follow the reference's MCXParam
 * (src/mcx_host.h:106-166); fields the GB300 kernel does not read (cache box,
 * polarisation, trajectory debug) are left out, and a few are added for
 * the persistent work queue and the uint8 volume.
 */
#ifndef MCX_KPARAMS_H
#define MCX_KPARAMS_H

#include <stdint.h>

#define MCXG_MAX_DET       1024   /* detectors held in constant memory */
#define MCXG_MAX_EXTRASRC  64     /* additional sources held in constant memory */
#define MCXG_MAX_MEDIA     1024   /* property rows staged in shared memory */

typedef struct mcxg_float4 {
    float x, y, z, w;
} mcxg_float4;

typedef struct mcxg_kparams {
    mcxg_float4 srcpos, srcdir, srcparam1, srcparam2; /* launch source; param2.z/.w carry the
                                                          launch voxel / medium bits of a point source */
    mcxg_float4 maxidx;            /* volume extent (x, y, z) as floats, for bounds tests */
    uint32_t dimx, dimxy, nvox;    /* strides: x fastest, then y, then z */
    uint32_t fieldlen;             /* gates x voxels (x sources when srcid < 0) */
    float twin0, twin1;            /* time window of this launch (s) */
    float oneoverc0;               /* 1/c0 in s per grid unit */
    float Rtstep;                  /* 1/tstep */
    float minenergy;               /* Russian-roulette threshold */
    float minaccumtime;            /* time per void step in skipvoid */
    uint32_t doreflect;            /* Fresnel at label boundaries */
    uint32_t dorefl_compiled;      /* reflection block active (isreflect or an r/m face) */
    uint32_t save2pt;              /* deposit into the field */
    uint32_t savedet;              /* 0 off, 1 on, 3 stop when the record buffer fills */
    uint32_t maxdetphoton;
    uint32_t maxmedia;             /* medianum - 1 */
    uint32_t medianum;
    uint32_t detnum;
    uint32_t voidtime;
    uint32_t srctype;
    uint32_t maxvoidstep;
    uint32_t issaveseed;
    uint32_t issaveref;
    uint32_t isspecular;
    uint32_t maxgate;
    uint32_t outputtype;
    uint32_t threadphoton;         /* photons per reference thread */
    int32_t  oddphoton;            /* the first oddphoton threads run one more */
    uint32_t savedetflag;
    uint32_t reclen;               /* floats per detected-photon record */
    uint32_t partialdata;          /* per-medium record floats */
    uint32_t mediaformat;          /* 1/2/4 labels, 101 float mua */
    uint32_t gscatter;
    uint32_t is2d;
    uint32_t nphase, nangle;       /* inverse-CDF table lengths */
    uint32_t extrasrclen;
    int32_t  srcid;
    uint32_t nthread;              /* reference threads = independent RNG streams */
    uint32_t mediaword;            /* bytes per voxel in device memory: 1 (label | det<<7) or 4 */
    uint32_t npattern;             /* source pattern length, for index clamping */
    uint8_t  bc[12];               /* face conditions then detector flags, as small integers */
    uint32_t replay;               /* 1: photons start from saved RNG states (the reference's SEED_FROM_FILE) */
    uint32_t nreplay;              /* replayed photons */
    int32_t  replaydet;            /* 0 all detectors, -1 one gate block per detector, k detector k */
    uint32_t siteshift;            /* scattering-site replay deposits read photon k+siteshift (the reference: 1) */
    uint32_t dimy, dimz;           /* voxel counts along y and z */
    uint32_t srcnum;               /* patterns sharing each photon (pattern sources), else 1 */
    float omega;                   /* modulation angular frequency (rad/s); > 0 without replay: RF transport */
    float fxscale, fxunit;         /* field accumulator: 2^S and 2^-S (the fixed-point plane counts units of 2^-S) */
} mcxg_kparams;

/* One simulation of a batch: its parameter block (nthread = its reference
   threads, fieldlen = its own field) and where its data sit in the batch's
   concatenated buffers. */
#define MCXG_BATCH_MAXMEDIA 4   /* property rows a batch simulation may have */

typedef struct mcxg_simdesc {
    mcxg_kparams kp;
    uint64_t media_off;            /* first voxel in the batch volume */
    uint64_t field_off;            /* first element in the batch field planes */
    uint64_t vt_off;               /* first reference thread in the batch numbering */
    uint64_t seed;                 /* seeds of its reference threads: splitmix64 of seed ^ (vt << 1) */
    uint64_t pad;
    mcxg_float4 prop[MCXG_BATCH_MAXMEDIA];   /* {mua, mus, g, n} per label */
    mcxg_float4 recip[MCXG_BATCH_MAXMEDIA];  /* filled on the device: 1/mus, 1/(mus (1-g)), 1/mua, 1/(2g) */
} mcxg_simdesc;

#endif
