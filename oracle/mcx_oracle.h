/*
 * mcx_oracle.h -- CPU oracle for the MCX-CL photon-transport path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load this library; the product never links
 * it and has no CPU fallback.
 *
 * The oracle restates, in plain C, the reference's per-thread transport loop
 * (mcx_core.cl:2307-3307, launchnewphoton 1463-2275, skipvoid 1350-1455,
 * hitgrid 975-995, savedetphoton 867-926) together with the host-side steps
 * that shape its inputs and outputs in mcx_run_simulation
 * (mcx_host.cpp:494-524 parameter packing, 696-700/759-768 seeding,
 * 1011-1012/1099-1104 work split, 1242-1306 field/energy merge, 1382-1465
 * normalisation) and the preprocessing of mcx_validatecfg/mcx_preprocess
 * (mcx_utils.c:1822-1964, 1521-1809) and mcx_maskdet (mcx_utils.c:4085-4198).
 *
 * The oracle is pinned bit for bit against the reference kernel itself,
 * compiled as host C++ from the reference sources (oracle/Makefile ->
 * oracle/_ref), and against the reference's own known answers (absorbed
 * fractions of the cube60/cube60b/planar benchmarks).
 */
#ifndef MCX_ORACLE_H
#define MCX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* math providers */
#define MCXO_MATH_LIBM   0   /* C library logf/expf/sincosf/acosf (matches the reference compiled on the host) */
#define MCXO_MATH_PMATH  1   /* oracle_pmath.h: bit-identical to the GPU kernel's exact instantiation */

/* semantics variants: the reference ships one kernel source with two branches */
#define MCXO_VARIANT_OPENCL 0  /* the OpenCL branch that mcxcl actually runs (hitgrid adds EPS) */
#define MCXO_VARIANT_NVCC   1  /* the never-launched __NVCC__ branch (hitgrid without EPS, arcsine==isotropic) */

/* fluence accumulators */
#define MCXO_FIELD_FLOAT_SPILL 0 /* float atomics with the +-1000 spill half, as mcx_core.cl:2880-2886 */
#define MCXO_FIELD_DOUBLE      1 /* FP64 accumulation of the same deposits */

#define MCXO_SEED_FROM_FILE  (-999) /* seed value that selects replay, mcx_core.cl:503-505 */

typedef struct mcxo_input {
    /* domain: vol holds one 32-bit word per voxel, x fastest (the layout
       mcx_preprocess leaves in cfg->vol); labels for mediabyte 1/2/4, float
       bits of mua for mediabyte 101 */
    unsigned int dimx, dimy, dimz;
    const uint32_t* vol;
    int mediabyte;
    const float* prop;          /* medianum rows of {mua, mus, g, n}, per mm */
    unsigned int medianum;
    float unitinmm;

    /* sources */
    int srctype;
    float srcpos[4], srcdir[4], srcparam1[4], srcparam2[4];
    const float* srcpattern;
    unsigned int srcnum;
    unsigned int extrasrclen;
    const float* srcdata;       /* extrasrclen x {pos[4], dir[4], param1[4], param2[4]} */
    int srcid;

    /* detectors */
    const float* detpos;        /* detnum x {x, y, z, r} */
    unsigned int detnum;
    unsigned int maxdetphoton;
    int issavedet;
    unsigned int savedetflag;
    int issaveseed;
    int issaveref;
    int issaveexit;
    int ismomentum;

    /* time gates */
    float tstart, tstep, tend;

    /* physics and output flags */
    int isreflect;
    char bc[12];                /* 6 face conditions ('_','r','a','m','c') + 6 detector flags ('0','1') */
    float minenergy;
    unsigned int gscatter;
    int voidtime;
    int isspecular;
    int maxvoidstep;
    int outputtype;             /* 0 flux, 1 fluence, 2 energy, 3 jacobian, 4 wp, 5 dcs, 7 length, 9 wltof, 10 wptof */
    int isnormalized;
    int issrcfrom0;
    const float* invcdf;
    unsigned int nphase;
    const float* angleinvcdf;
    unsigned int nangle;

    /* run */
    double nphoton;
    unsigned int nthread;       /* reference "autothread": number of RNG streams */
    unsigned int core;          /* device core count (workload weight of the split) */
    int seed;
    int debugrng;               /* 1: fill the field with each thread's RNG stream (-D R) */

    /* oracle options */
    int mathmode;
    int variant;
    int fieldmode;
    int nworkers;               /* OpenMP workers (0 = library default); FLOAT_SPILL always runs serially */

    /* replay (the reference's seed = SEED_FROM_FILE): each photon is launched
       from a saved xorshift128+ state; nphoton must equal nreplay.  The
       per-photon arrays come from mcxo_replayinit. */
    const uint64_t* replayseed; /* nreplay x 2 words */
    const float* replayweight;  /* nreplay */
    const float* replaytof;     /* nreplay, seconds */
    const int* replaydetid;     /* nreplay */
    unsigned int nreplay;
    int replaydet;              /* 0 all detectors into one field, -1 one field per detector, k detector k */
    int replaysiteown;          /* 1: scattering-site replay outputs read the replayed photon's own entries */

    /* optional output: weight and time of flight of each saved detected photon
       when it was detected (maxdetphoton x 2 floats), or NULL */
    float* detweight_out;

    /* modulation angular frequency (rad/s): with omega > 0 a forward run
       carries complex photon weights (RF forward), and the replay outputs
       'rf' and 'rfmus' are complex */
    float omega;

    /* polarised transport: polmedianum x 181 Mueller rows {S11, S12, S33, S34}
       (as mcx_prep_polarized leaves them in cfg->smatrix) and the launch
       Stokes vector; prop must already hold the Mie-derived mus and g */
    const float* smatrix;
    unsigned int polmedianum;
    float s0[4];

    /* rand() words drawn and discarded before the per-thread seed words: a
       later repetition of a respin run draws after the earlier ones'
       4 x nthread words each (mcx_host.cpp:759-768 inside the respin loop) */
    unsigned int seedskip;

    /* trajectory capture (-D M, mcx_core.cl:929-948): records of 6 floats
       {photon id (uint bits), x, y, z, w, source id} at every photon close,
       launch and scattering site; at most maxtraj stored, *ntraj counts all */
    int debugmove;
    unsigned int maxtraj;
    float* traj_out;
    unsigned int* ntraj_out;
} mcxo_input;

typedef struct mcxo_stats {
    double energytot, energyesc, energyabs, normalizer;
    unsigned int detected;      /* detections (may exceed maxdetphoton) */
    unsigned int saved;         /* records written */
    unsigned int threadphoton;
    int oddphoton;
    unsigned int reclen;
    unsigned int fieldlen;      /* gates x voxels */
    unsigned int maxgate;
    uint64_t nstep, nscatter, nlaunch, nreflect, nfailed;
} mcxo_stats;

/* Size queries so the caller can allocate outputs. */
/*
 * mcx_replayinit (mcx_utils.c:1355-1421): select the detected photons to
 * replay and compute each one's detected weight and time of flight from its
 * record.  detp: ndet records of reclen floats (host layout); seeds: ndet x 2
 * words.  Writes up to ndet entries of seed_out/weight/tof/detid and returns
 * the number kept, or a negative error code.
 */
int mcxo_replayinit(const mcxo_input* in, const float* detp, unsigned int reclen, unsigned int ndet,
                    const uint64_t* seeds, uint64_t* seed_out, float* weight, float* tof, int* detid);

unsigned int mcxo_reclen(const mcxo_input* in);
unsigned int mcxo_fieldlen(const mcxo_input* in);
/* 2 when the field is complex (RF forward, RF replay outputs): the outputs
   then hold fieldlen real values followed by fieldlen imaginary values */
unsigned int mcxo_fieldcomp(const mcxo_input* in);

/*
 * Run the simulation.  Outputs (caller-allocated, may be NULL when unused):
 *   field     fieldlen doubles (x mcxo_fieldcomp): the merged raw field
 *   fieldnorm fieldlen floats (x mcxo_fieldcomp): normalised as mcx_run_simulation does
 *   energy    2*nthread floats: per-thread {escaped, launched} weight
 *   detp      maxdetphoton*reclen floats, in the host record layout
 *   seeds     maxdetphoton*2 uint64 (launch RNG state of each record)
 *   masked    dimx*dimy*dimz words: the volume after detector masking
 * Returns 0 on success, a negative error code otherwise.
 */
int mcxo_run(const mcxo_input* in, double* field, float* fieldnorm, float* energy,
             float* detp, uint64_t* seeds, uint32_t* masked, mcxo_stats* stats);

/* Prepared kernel constants and buffers, for driving the reference kernel
   (compiled on the host from the reference sources) with identical inputs.
   Field names follow the reference's MCXParam (mcx_host.h:106-166). */
typedef struct mcxo_refprep {
    float srcpos[4], srcdir[4], srcparam1[4], srcparam2[4];
    unsigned int extrasrclen;
    int srcid;
    float maxidx[4];
    unsigned int dimlen[4];
    float twin0, twin1, oneoverc0, Rtstep, minenergy, minaccumtime;
    unsigned int save2pt, doreflect, savedet, maxdetphoton, maxmedia, detnum, voidtime;
    unsigned int srctype, maxvoidstep, issaveseed, issaveref, isspecular, maxgate, outputtype;
    unsigned int threadphoton;
    int oddphoton;
    unsigned int savedetflag, reclen, partialdata, w0offset, mediaformat, gscatter, is2d, srcnum;
    unsigned int nphase, nangle;
    char bc[12];
    int dorefl_compiled;
    unsigned int nprop;         /* float4 rows in gprop */
    float* gprop;
    float* gdet;
    uint32_t* media;            /* masked volume */
    uint32_t* seedwords;        /* 4 per thread */
    unsigned int nvox, fieldlen;
    float omega;
    int rfmode;                 /* 0 real, 1 RF forward, 2 RF replay output */
    unsigned int maxpolmedia;   /* polarised transport */
    float s0[4];
    const float* smatrix;
} mcxo_refprep;

int  mcxo_prepare_ref(const mcxo_input* in, mcxo_refprep* out);
void mcxo_free_ref(mcxo_refprep* r);

/* Math providers exposed for the cross-implementation bit test. */
float mcxo_pm_logf(float x);
float mcxo_pm_expf(float x);
void  mcxo_pm_sincosf(float x, float* s, float* c);
float mcxo_pm_acosf(float x);

#ifdef __cplusplus
}
#endif

#endif
