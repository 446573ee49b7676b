/*
 * mcx_gb300.h -- C ABI of the GB300 photon-transport path.
 *
 * Two layers, both plain C (no CUDA or torch types in any signature):
 *
 *  1. The drop-in host interface of the reference's simulation driver.
 *     `Config` keeps the field names, types and meanings of the reference's
 *     MCXConfig (src/mcx_utils.h:165-281) for every field the transport path
 *     reads or writes; fields that only serve subsystems outside this path
 *     (MATLAB/NIfTI/JNIfTI writers, shapes parser, polarisation, trajectory
 *     debug, adjoint post-processing) are not carried.  Callers fill a
 *     Config the way they fill the reference's, call mcx_validatecfg() and
 *     mcx_run_simulation(), and read the same output fields.
 *
 *  2. The thin device layer (mcxg_*) that the C host driver calls: a session
 *     owning device memory on one GPU, uploads, a kernel launch, FP64
 *     reductions and readback.  Every call returns an int status
 *     (MCXG_OK == 0); mcxg_error_string() names it.  It replaces the OpenCL
 *     launch and readback code in mcx_run_simulation
 *     (src/mcx_host.cpp:739-1345).
 *
 * One GPU per call.  Not re-entrant across threads that share a Config.
 */
#ifndef MCX_GB300_H
#define MCX_GB300_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCX_GB300_VERSION   "v2025.10-gb300"
#define MAX_SESSION_LENGTH  64
#define MAX_PATH_LENGTH     1024
#define MAX_DEVICE          256

/* ---- constants (src/mcx_const.h) ---------------------------------------- */
#define MCX_SRC_PENCIL       0
#define MCX_SRC_ISOTROPIC    1
#define MCX_SRC_CONE         2
#define MCX_SRC_GAUSSIAN     3
#define MCX_SRC_PLANAR       4
#define MCX_SRC_PATTERN      5
#define MCX_SRC_FOURIER      6
#define MCX_SRC_ARCSINE      7
#define MCX_SRC_DISK         8
#define MCX_SRC_FOURIERX     9
#define MCX_SRC_FOURIERX2D   10
#define MCX_SRC_ZGAUSSIAN    11
#define MCX_SRC_LINE         12
#define MCX_SRC_SLIT         13
#define MCX_SRC_PENCILARRAY  14
#define MCX_SRC_PATTERN3D    15
#define MCX_SRC_HYPERBOLOID_GAUSSIAN 16
#define MCX_SRC_RING         17

#define MEDIA_MUA_FLOAT      101
#define SEED_FROM_FILE       -999
#define FILL_MAXDETPHOTON    3

enum TOutputType {otFlux, otFluence, otEnergy, otJacobian, otWP, otDCS, otRF, otL, otRFmus, otWLTOF, otWPTOF, otAdjoint,
                  otAdjointDcoeff, otAdjointMus, otAdjointMusp, otAdjointMuaD, otAdjointMuaMusp};
#define MCX_IS_ADJOINT_TYPE(t)      ((int)(t) >= (int)otAdjoint)
#define MCX_IS_DUAL_ADJOINT_TYPE(t) ((int)(t) >= (int)otAdjointMuaD)
enum TBoundary {bcUnknown, bcReflect, bcAbsorb, bcMirror, bcCyclic};
enum TMCXParent {mpStandalone, mpMATLAB, mpPython};

/* savedetflag bits: D S P M X V W (src/mcx_const.h:93-100) */
#define SAVE_DETID(a)  ((a) & 0x1)
#define SAVE_NSCAT(a)  ((a) >> 1 & 0x1)
#define SAVE_PPATH(a)  ((a) >> 2 & 0x1)
#define SAVE_MOM(a)    ((a) >> 3 & 0x1)
#define SAVE_PEXIT(a)  ((a) >> 4 & 0x1)
#define SAVE_VEXIT(a)  ((a) >> 5 & 0x1)
#define SAVE_W0(a)     ((a) >> 6 & 0x1)
#define SAVE_IQUV(a)   ((a) >> 7 & 0x1)
#define MCX_NANGLES    181              /* polar angles of the Mueller tables (src/mcx_const.h:67) */

typedef struct { float x, y, z, w; } mcx_float4;
typedef struct { unsigned int x, y, z, w; } mcx_uint4;

/* src/mcx_utils.h:77-82 */
typedef struct MCXMedium {
    float mua, mus, g, n;
} Medium;

/* src/mcx_utils.h:88-94: the scatterers of one medium of a polarised run */
typedef struct MCXPolarizeMedium {
    float mua;                    /* background absorption, 1/mm */
    float r;                      /* sphere radius, micron */
    float rho;                    /* sphere number density, 1/micron^3 */
    float nsph;                   /* sphere refractive index */
    float nmed;                   /* background refractive index */
} POLMedium;

/* src/mcx_utils.h:100-105: one additional source */
typedef struct MCXExtraSource {
    mcx_float4 srcpos, srcdir, srcparam1, srcparam2;
} ExtraSrc;

/* Photon replay inputs (PhotonReplay, src/mcx_utils.h:136-141).  The caller
   sets seed (16 bytes per photon, malloc'd; cfg.seed = SEED_FROM_FILE);
   mcx_validatecfg keeps the photons to replay and fills weight, tof, detid. */
typedef struct MCXReplay {
    void* seed;
    float* weight;                /* detected weight: w0 * prod exp(-mua * partial path) */
    float* tof;                   /* detected time of flight, s */
    int* detid;                   /* detector id | source id << 16 */
} Replay;

/* src/mcx_utils.h:113-130: the .mch header, filled for detected photons */
typedef struct MCXHistoryHeader {
    char magic[4];
    unsigned int version, maxmedia, detnum, colcount, totalphoton, detected, savedphoton;
    float unitinmm;
    unsigned int seedbyte;
    float normalizer;
    int respin;
    unsigned int srcnum, savedetflag, totalsource;
    int reserved[1];
} History;

/* src/mcx_utils.h:143-163 */
typedef struct MCXGPUInfo {
    char name[MAX_SESSION_LENGTH];
    int id, devcount, platformid, major, minor;
    size_t globalmem, constmem, sharedmem;
    int regcount, clock, sm, core;
    size_t autoblock, autothread;
    unsigned int maxgate;
    int maxmpthread, iscpu;
    int vendor;
} GPUInfo;

/* The simulation configuration.  Names and meanings as src/mcx_utils.h:165-281. */
typedef struct MCXConfig {
    size_t nphoton;
    unsigned int nblocksize;
    unsigned int nthread;
    int seed;
    mcx_float4 srcpos, srcdir;
    float tstart, tstep, tend;
    mcx_float4 steps;
    mcx_uint4 dim;
    unsigned int medianum;
    unsigned int detnum;
    unsigned int maxdetphoton;
    Medium* prop;
    mcx_float4* detpos;
    unsigned int maxgate;
    int respin;
    int gpuid;
    unsigned int* vol;            /* one word per voxel, x fastest; labels, or float mua bits (MEDIA_MUA_FLOAT) */
    char session[MAX_SESSION_LENGTH];
    char isrowmajor, isreflect, isrefint, isnormalized, issavedet, issave2pt, isgpuinfo, isspecular;
    char issrcfrom0, ismomentum, internalsrc, issaveseed, issaveexit, isatomic, issaveref;
    char srctype, autopilot, outputtype;
    float minenergy;
    float unitinmm;
    FILE* flog;
    History his;
    double energytot, energyabs, energyesc;
    int maxvoidstep, voidtime;
    mcx_float4 srcparam1, srcparam2;
    unsigned int srcnum;
    float* srcpattern;
    char deviceid[MAX_DEVICE];
    float workload[MAX_DEVICE];
    float* exportfield;           /* [Nx,Ny,Nz,gates(,sources)] x fastest */
    float* exportdetected;        /* [reclen x detected] */
    unsigned int debuglevel;
    float normalizer;
    void* seeddata;               /* detected-photon RNG seeds, 16 bytes each */
    unsigned int gscatter;
    unsigned int savedetflag;
    unsigned int detectedcount;
    unsigned int runtime;         /* kernel time, ms */
    int parentid;
    unsigned int mediabyte;
    char bc[13];
    unsigned int nphase;
    float* invcdf;
    unsigned int nangle;
    float* angleinvcdf;
    int srcid;
    unsigned int extrasrclen;
    ExtraSrc* srcdata;
    Replay replay;
    int replaydet;
    mcx_float4* detdir;           /* adjoint outputs: per detector {direction, focal length}; detectors become sources */
    float* exportjacob;           /* adjoint Jacobians: [Nx,Ny,Nz, sources x detectors] (x2 for the dual types) */                /* replay: 0 all detectors, -1 one output per detector, k detector k only */
    /* GB300 additions */
    int exactmath;                /* 1: run the IEEE-only kernel (bit-identical to the CPU oracle) */
    float kernelms;               /* kernel time from CUDA events, ms */
    uint64_t eventcount[5];       /* exact kernel only: steps, scatterings, launches, Fresnel tests, failed launches */
    unsigned int failedlaunch;    /* reference threads whose first launch found no entry point */
    unsigned int threadused;      /* reference threads (RNG streams) of the last run */
    float* exportenergy;          /* when savethreadenergy: 2 x threadused {escaped, launched} floats */
    int savethreadenergy;
    int autotune;                 /* 1: time the launch shapes on a photon sample, once per problem shape, keep the fastest */
    int savedetweight;            /* 1: fill exportdetweight */
    float* exportdetweight;       /* 2 x detectedcount: weight and time of flight (s) of each saved photon when detected */
    int replaysiteown;            /* replay: 1 = scattering-site outputs use the replayed photon's own weight and time
                                     (the reference reads the next photon's, mcx_core.cl:2571) */
    float omega;                  /* modulation angular frequency 2 pi f (rad/s), mcx_utils.h:231: > 0 runs the
                                     frequency-domain (RF) transport, or phases the rf/rfmus replay outputs */
    /* polarised transport (mcx_utils.h:174-194, 232): one POLMedium per label 1..polmedianum (malloc'd,
       freed by mcx_clearcfg), the wavelength in nm, the launch Stokes vector; mcx_validatecfg fills
       smatrix (polmedianum x MCX_NANGLES {S11, S12, S33, S34}) and the labels' mus and g from Mie theory */
    POLMedium* polprop;
    unsigned int polmedianum;
    float lambda;
    mcx_float4 srciquv;
    mcx_float4* smatrix;
    /* trajectory capture (debuglevel M): records of 6 floats {photon id (uint
       bits), x, y, z, w, source id}, at most maxjumpdebug per repetition */
    unsigned int maxjumpdebug;
    unsigned int debugdatalen;
    float* exportdebugdata;
    int errorcode;                /* last error in library mode */
    char errormsg[256];
} Config;

/* ---- drop-in host interface ------------------------------------------------ */

/* Defaults of mcx_initcfg (src/mcx_utils.c:203-366). */
void mcx_initcfg(Config* cfg);
/* Frees every buffer the Config owns (src/mcx_utils.c:368-476). */
void mcx_clearcfg(Config* cfg);
/* Checks inputs, converts to 0-based positions, scales by unitinmm, builds the
   detector mask and launch voxel (src/mcx_utils.c:1822-1964, 1521-1809).
   Replay (cfg.seed == SEED_FROM_FILE, cfg.replay.seed set): detps holds the
   baseline run's records, dimdetps {reclen, count}, seedbyte 16; the photons
   of detector replaydet (all when <= 0) whose time of flight lies in the time
   window are kept, with their detected weights (mcx_replayinit,
   src/mcx_utils.c:1355-1421). */
void mcx_validatecfg(Config* cfg, float* detps, int dimdetps[2], int seedbyte);
/* Reads a JSON input file (src/mcx_utils.c:2011-2071 with mcx_loadjson
   2401-3287): fname is a .json file, or the JSON text itself when it starts
   with '{'.  Reads the sections the transport path uses -- Session (ID,
   Photons, RNGSeed, MaxDetPhoton, BCFlags, Do* switches, DebugFlag,
   SaveDataMask, OutputType, MinEnergy), Forward (T0, T1, Dt), Optode
   (Source: Type, Pos, Dir, Param1, Param2, Weight, Frequency, WaveLength,
   SrcNum, ID, Pattern, AngleInverseCDF, extra sources as arrays of vectors;
   Detector: Pos, R, Dir), Domain (Media, MieScatter, Dim, Step, LengthUnit,
   MediaFormat, OriginType, InverseCDF, VolumeFile of byte/short/integer
   labels) and Shapes (Name, Origin, Grid, Sphere, Box, Subgrid, Cylinder,
   UpperSpace, X/Y/ZSlabs, X/Y/ZLayers) -- then validates cfg as
   mcx_validatecfg does: cfg is ready for mcx_run_simulation.  The legacy
   .inp text format is not read.  Errors go through mcx_error. */
void mcx_readconfig(char* fname, Config* cfg);
/* The same from JSON text in memory (src/mcx_utils.c, mcx_parsejson). */
void mcx_parsejson(char* jbuf, Config* cfg);
/* Lists CUDA devices into *info (caller frees with mcx_cleargpuinfo); replaces
   mcx_list_gpu(Config*, unsigned*, cl_device_id*, GPUInfo**)
   (src/mcx_host.cpp:252).  Returns the number of active devices. */
int  mcx_list_gpu(Config* cfg, unsigned int* activedev, GPUInfo** info);
void mcx_cleargpuinfo(GPUInfo** info);
/* Runs the simulation (src/mcx_host.h:168); fluence and totalenergy are unused,
   as in the reference.  Outputs go to cfg: exportfield, exportdetected,
   seeddata, detectedcount, energytot/energyesc/energyabs, normalizer, runtime.
   The calling thread's current CUDA device is the same on return as before
   (the run itself uses the device cfg selects). */
void mcx_run_simulation(Config* cfg, float* fluence, float* totalenergy);
/* Frees one output buffer that a caller took over from cfg (exportfield,
   exportdetected, seeddata, ...: set the Config's pointer to NULL first so
   mcx_clearcfg leaves it alone).  While sessions are kept (mcx_keep_sessions,
   on by default), buffers of 1 MB and more are kept too (up to 8 and 1 GB)
   for the next run's field and detected records, whose readbacks then land
   in resident pages; mcx_release_sessions frees them.  A GB300
   addition: the Python module hands the buffers to numpy arrays without
   copying them. */
void mcx_free_buffer(void* p);
/* Writes detected photons as <session>.mch: the History header, count records
   of his.colcount floats, then the seeds (src/mcx_utils.c:963-998). */
void mcx_savedetphoton(float* ppath, void* seeds, int count, int doappend, Config* cfg);
/* Scales field[i*srcnum+pidx] by scale (src/mcx_utils.c:1208-1218). */
void mcx_normalize(float field[], float scale, int fieldlen, int option, int pidx, int srcnum);
/* Error reporting.  Standalone: print and exit(id).  Library mode
   (cfg->parentid != mpStandalone): the failing public call returns with
   cfg->errorcode/errormsg set; read them with mcx_last_error(). */
void mcx_error(const int id, const char* msg, const char* file, const int linenum);
int  mcx_last_error(const Config* cfg, const char** msg);
/* Number of floats in one detected-photon record for this Config. */
unsigned int mcx_detreclen(const Config* cfg);
const char* mcx_version(void);
/* Mie scattering of a sphere of size parameter x = 2 pi r n_med / lambda and
   real relative index mrel = n_sph / n_med: the Mueller elements {S11, S12,
   S33, S34} at the 181 polar angles pi i / 180 (181 x 4 floats), the
   scattering efficiency and the anisotropy (the reference's Mie,
   src/mcx_mie.cpp:91).  0 on success. */
int mcx_mie(double x, double mrel, float* smatrix, double* qsca, double* g);
/* The n words rand() returns after srand(seed) in glibc (the reference's
   per-thread seed words), without the C library's per-call lock. */
void mcx_rand_words(unsigned int seed, uint32_t* out, size_t n);
/* Jump-ahead into the same stream: the generator's 31-word windows (the
   unshifted values of words k - 31 .. k - 1) at k = skip + j x blocklen for
   j < nblock, into starts (31 x nblock words): each block of words can then
   be generated on its own.  0 on success. */
int mcx_rand_blocks(unsigned int seed, uint64_t skip, uint32_t nblock, uint32_t blocklen, uint32_t* starts);
/* A label volume of nx x ny x nz bytes to the Config's uint32 words, x
   fastest (out: nx ny nz words).  c_order = 1 when vol is laid out [x][y][z]
   with z fastest (numpy's default order), 0 when x is already fastest.  A GB300
   addition: the Python module's volume conversion for uint8 labels. */
void mcx_labels_u8(const uint8_t* vol, uint32_t nx, uint32_t ny, uint32_t nz, int c_order, uint32_t* out);
/* Everything mcx_run_simulation does before its first launch -- device
   selection, parameter block, volume packing, upload, seeds of the first
   repetition -- and nothing after: returns the ready device session so a
   caller can launch the resident problem repeatedly with mcxg_simulate
   (benchmarks, repeated solves).  NULL on error (cfg->errorcode). */
struct mcxg_session* mcx_prepare_simulation(Config* cfg);
/* Runs n validated configurations in one persistent launch: a GB300
   addition, no counterpart in the reference (one simulation per
   mcx_run_simulation call).  Each simulation gets ceil(nphoton /
   photons_per_thread) reference threads (0: 1 photon a thread up to 2^18
   photons, 2 above) with seeds derived from its cfg.seed; flags: MCXG_GRAPH, MCXG_AGG.  Outputs go to each Config as
   mcx_run_simulation's do; an error is reported on cfgs[0].  Label volumes
   of at most 128 labels, one respin, no detectors, replay, extra sources,
   patterns or phase tables. */
void mcx_run_batch(Config** cfgs, int n, unsigned int photons_per_thread, unsigned int flags);
/* mcx_run_batch with every deposit also accumulated in FP64 (no
   counterpart in the reference): the same outputs, and in relerr (3 x n
   doubles) each simulation's max and median relative error of the
   compensated field over its non-zero elements, and the relative error of
   its total, against that FP64 accumulation of the same photons. */
void mcx_run_batch_verify(Config** cfgs, int n, unsigned int photons_per_thread, double* relerr);
/* sizeof(Config) and the byte offset of a named field ((size_t)-1 if
   unknown), for checking foreign-function mirrors of the struct. */
size_t mcx_config_sizeof(void);
size_t mcx_config_offsetof(const char* name);
/* Releases the device sessions cached per GPU by mcx_run_simulation. */
void mcx_release_sessions(void);
/* keep = 1 (the default): mcx_run_simulation and mcx_run_batch keep one
   device session per GPU between calls (device buffers, the uploaded volume
   and the tuned launch shape are reused).  keep = 0: the cached sessions
   are released now and at the end of every later call, so no device memory
   outlives a call, as with the reference's mcx_run_simulation
   (src/mcx_host.cpp, which frees every buffer before it returns).
   A session returned by mcx_prepare_simulation stays usable until the next
   mcx_run_simulation, mcx_run_batch or mcx_release_sessions.  These calls
   share the cached sessions across host threads and hold one process-wide
   lock while they run, so calls from several threads run one at a time; the
   device-layer mcxg_* calls on a session take no lock (one thread a
   session). */
void mcx_keep_sessions(int keep);

/* ---- thin device layer ------------------------------------------------------ */

/* mcxg_set_problem: 32-bit label words in, packed to bytes on the device */
#define MCXG_MEDIA_PACK 0x101u

#define MCXG_OK              0
#define MCXG_ERR_CUDA        1
#define MCXG_ERR_ARG         2
#define MCXG_ERR_NOMEM       3
#define MCXG_ERR_LIMIT       4
#define MCXG_ERR_STATE       5
#define MCXG_ERR_NODEVICE    6

/* mcxg_simulate flags */
#define MCXG_EXACT    1u   /* IEEE-only kernel with event counters */
#define MCXG_NOAGG    2u   /* no warp aggregation of deposits (the default unless autotuned) */
#define MCXG_RNGDUMP  4u   /* write each thread's RNG stream into the field (-D R) */
#define MCXG_KEEP     8u   /* keep accumulating into the field (respin); energies, records and counters restart */
#define MCXG_AGG     16u   /* aggregate same-voxel deposits of a warp before the atomics */
#define MCXG_GRAPH   32u   /* batch: capture the run as a CUDA graph once, replay it afterwards */
#define MCXG_GENERAL 64u   /* fast kernel: the general instantiation even where the one specialised for the
                              common configuration (label volume, 3-D, Henyey-Greenstein) applies */
#define MCXG_ADJ1   256u   /* fluence gradient, pass 1: each photon's loss total (mcxg_set_adjoint first) */
#define MCXG_ADJ2   512u   /* fluence gradient, pass 2: the gradients, same photons (read with
                              mcxg_get_adjoint_grad) */
#define MCXG_NOL2WINDOW 1024u /* no persisting L2 window over the field's count plane (for measurement: the
                                window keeps the counts in L2 and cuts the launch's DRAM write-backs) */
#define MCXG_VERIFY 128u   /* precision check (fast kernel, common configuration, no replay, no KEEP): every
                              deposit also goes to an FP64 field, a plain float field and a float field with
                              the reference's +-1000 spill plane; read them with mcxg_get_verify */

typedef struct mcxg_devinfo {
    char name[64];
    int major, minor, sm, clock_khz;
    size_t globalmem, sharedmem_per_block, constmem;
    int regs_per_block, max_threads_per_sm;
} mcxg_devinfo;

typedef struct mcxg_session mcxg_session;

int  mcxg_device_count(int* n);
int  mcxg_device_info(int device, mcxg_devinfo* info);
const char* mcxg_error_string(int code);

int  mcxg_create(int device, mcxg_session** s);
int  mcxg_destroy(mcxg_session* s);

/*
 * Upload one problem.  kparams points to an mcxg_kparams (csrc/mcx_kparams.h),
 * passed opaquely with its size for ABI checking.  media holds nvox voxels of
 * mediaword bytes each (1: label | detector bit << 7; 4: the reference's
 * 32-bit word), or with mediaword MCXG_MEDIA_PACK the reference's 32-bit
 * words (label | detector bit 31, labels below 128, medianum <= 128), which
 * the device packs to the one-byte form.  prop: medianum x 4 floats; detpos: detnum x 4; srcextra:
 * extrasrclen x 16; tables may be NULL when their length is 0.
 */
int  mcxg_set_problem(mcxg_session* s, const void* kparams, size_t kparams_size, const void* media,
                      uint32_t mediaword, const float* prop, const float* detpos, const float* srcextra,
                      const float* invcdf, const float* angleinvcdf, const float* srcpattern, size_t npattern);
/* Replace the parameter block of the current problem (same buffer shapes:
   photon split, time window, flags); the next launch re-uploads it. */
int  mcxg_set_params(mcxg_session* s, const void* kparams, size_t kparams_size);
/* 4 seed words per reference thread, as the reference draws them with rand(). */
int  mcxg_set_seeds(mcxg_session* s, const uint32_t* seeds, uint32_t nthread);
/* The same words generated on the device: 4 x nthread words of the additive
   generator, in nblock blocks of blocklen words ((nblock - 1) x blocklen <
   4 x nthread <= nblock x blocklen), block j starting from the 31 words
   starts[31 j ..] that mcx_rand_blocks returns. */
int  mcxg_set_seeds_lfib(mcxg_session* s, const uint32_t* starts, uint32_t nblock, uint32_t blocklen,
                         uint32_t nthread);
/* The same words with the jump-ahead also on the device: window holds the
   generator's 31 unshifted outputs before the first word (what
   mcx_rand_blocks returns for block 0); the device raises the one-step matrix
   to the block length and its powers of two and starts each block of words
   from its own window.  mcx_run_simulation seeds this way. */
int  mcxg_set_seeds_window(mcxg_session* s, const uint32_t* window, uint32_t nthread);
/* The session's 4 x nthread seed words, back to the host (out: 4 x nthread words). */
int  mcxg_get_seeds(mcxg_session* s, uint32_t* out, uint32_t nthread);
/* Trajectory capture (-D M): buffers for maxrec records (0: off); each
   launch restarts the count.  get copies min(count, maxrec, capacity)
   records and returns every record the launch made in *count. */
int  mcxg_set_trajectory(mcxg_session* s, uint32_t maxrec);
int  mcxg_get_trajectory(mcxg_session* s, float* out, uint32_t maxrec, uint32_t* count);
/* Launch shape of the persistent grid: block threads (32..256, a multiple of
   32) and resident blocks per SM (0 = automatic: 256 threads x 4).  Shapes of
   more than 512 threads per SM run the instantiation whose registers are
   capped for 1,024 resident threads (64 a thread; the specialised RF,
   polarised, split-voxel, other-encoding, precision-check and gradient
   kernels: 768 and 80), the others the uncapped one; blocks per SM are
   lowered to what fits at once. */
int  mcxg_set_launch(mcxg_session* s, int block, int blocks_per_sm);
/* Hot-voxel tile (no counterpart in the reference, which adds every deposit
   to global memory, src/mcx_core.cl:2880-2886): with elements > 0, launches
   of the fast kernel on a single simulation of the common configuration (no
   replay, extra sources or precision check) accumulate the deposits of a box
   of voxels next to the source, in the first gates, in each block's shared
   memory -- at most `elements` field elements, fewer if shared memory is
   short -- and add them to the field when the block ends.  Same fixed-point
   split, same answer.  0 (the default) turns it off.  mcxg_get_tile gives
   the last launch's box: x0 y0 z0 nx ny nz gates elements (all 0: none). */
int  mcxg_set_tile(mcxg_session* s, uint32_t elements);
int  mcxg_get_tile(mcxg_session* s, uint32_t* box);
/* ---- batches: many simulations in one persistent launch (no counterpart in
   the reference, which launches once per simulation).  sims points to nsim
   mcxg_simdesc (csrc/mcx_kparams.h, desc_size bytes each): the parameter
   block of simulation i (nthread = its reference threads, fieldlen = its
   field), its property rows (at most MCXG_BATCH_MAXMEDIA) and its offsets
   into the concatenated volume (one byte per voxel, label | detector
   bit << 7) and field.  Reference threads are numbered contiguously across
   the batch (vt_off); seeds come from splitmix64 of the simulation's seed.
   The simulations run in waves of 136, whose descriptors the kernel reads
   from constant memory.  Not supported in a batch: detectors, replay, extra
   sources, patterns, phase tables, encodings other than labels. */
int  mcxg_batch_set(mcxg_session* s, const void* sims, size_t desc_size, uint32_t nsim, const uint8_t* media,
                    uint64_t nmedia);
/* The same with each simulation's volume as the Config's 32-bit label words
   (words[i]: sims[i].kp.nvox of them, labels below 128): they are uploaded
   to media_off of an nmedia-word staging buffer and packed to the label bytes
   on the device (detector bits dropped: a batch saves no detected photons). */
int  mcxg_batch_set_words(mcxg_session* s, const void* sims, size_t desc_size, uint32_t nsim,
                          const uint32_t* const* words, uint64_t nmedia);
/* Runs every simulation of the batch; MCXG_GRAPH replays a captured graph,
   MCXG_AGG aggregates deposits, MCXG_VERIFY also accumulates every deposit
   in FP64 (read with mcxg_batch_get_verify).  *kernel_ms covers the clear,
   transport and per-simulation sums. */
int  mcxg_batch_simulate(mcxg_session* s, unsigned int flags, float* kernel_ms);
/* The precision check of the last MCXG_VERIFY batch run (no counterpart in
   the reference): the FP64 accumulation of the same deposits and the
   compensated field merged in FP64, both unscaled, for every simulation at
   its field offset (NULL skips one). */
int  mcxg_batch_get_verify(mcxg_session* s, double* f64, double* comp);
/* Per simulation: FP64 {escaped, launched} weight, 2 x nsim. */
int  mcxg_batch_get_energy(mcxg_session* s, double* out);
/* Every simulation's field, the compensated accumulator in FP64 x scales[i], at its field offset. */
int  mcxg_batch_get_field(mcxg_session* s, float* out, const double* scales);
/* Replay inputs, one entry per replayed photon: the saved xorshift128+ state
   (16 bytes), detected weight, time of flight and detector id.  Used when
   the parameter block has replay = 1; n = 0 releases nothing and clears. */
int  mcxg_set_replay(mcxg_session* s, const void* seeds16, const float* weight, const float* tof, const int* detid,
                     uint32_t n);
/* Pick the launch shape of the fast kernel for the current problem: time
   each candidate (blocks of 256, 128 and 64 threads at 1,024 resident
   threads per SM with capped registers, 256 and 128 at 512 with uncapped
   ones; then
   the fastest with warp-aggregated deposits) on the first sample_photons
   photons and keep the fastest for later mcxg_simulate calls (unless a
   shape was set with mcxg_set_launch).  Outputs may be NULL.  The trial
   runs overwrite the field and energies. */
int  mcxg_autotune(mcxg_session* s, uint32_t sample_photons, int* block, int* blocks_per_sm, int* noagg);
/* Run all photons once; kernel time (CUDA events) into *kernel_ms. */
int  mcxg_simulate(mcxg_session* s, unsigned int flags, float* kernel_ms);
/* FP64 sums over threads of escaped and launched weight. */
int  mcxg_get_energy(mcxg_session* s, double* escaped, double* launched);
/* Per-thread {escaped, launched} floats, 2 x nthread. */
int  mcxg_get_thread_energy(mcxg_session* s, float* out);
/* Field: the compensated accumulator (fixed-point count x unit + remainder) in FP64, times
   scale, rounded to float; fieldlen values. */
int  mcxg_get_field(mcxg_session* s, float* out, double scale);
/* Field split into nblocks equal blocks, block b scaled by scales[b]
   (a replay with one output per detector). */
int  mcxg_get_field_blocks(mcxg_session* s, float* out, const double* scales, uint32_t nblocks);
/* As mcxg_get_field with element i scaled by scales[i % nsrc]: the per-pattern
   normalisation of photon sharing, whose field interleaves the patterns. */
int  mcxg_get_field_interleaved(mcxg_session* s, float* out, const double* scales, uint32_t nsrc);
/* Polarised transport: nmedia x MCX_NANGLES Mueller rows {S11, S12, S33, S34}
   for labels 1..nmedia and the launch Stokes vector s0[4]; nmedia 0 turns it
   off.  Kept until the next call or mcxg_set_problem. */
int  mcxg_set_polarization(mcxg_session* s, const float* smatrix, uint32_t nmedia, const float* s0);
/* Adjoint Jacobians from the normalised float field of the last
   mcxg_get_field: fieldlen = nx ny nz maxgate (ns + nd), the first ns gate
   blocks the sources, the next nd the detectors run as sources.  kind 0:
   time-integrated phi_src x phi_det per voxel; kind 1: the dot product of
   their finite-difference gradients.  out: nx ny nz x ns x nd floats,
   source-major over detector (src/mcx_core.cl:3320-3512). */
int  mcxg_adjoint(mcxg_session* s, int kind, uint32_t ns, uint32_t nd, uint32_t nx, uint32_t ny, uint32_t nz,
                  uint32_t maxgate, float* out);
/* The same post-kernels on a caller's host field (nx ny nz maxgate (ns + nd)
   floats, the layout above); the session needs no problem.  The reference's
   mcx_adjoint_kernel / mcx_adjoint_dcoeff_kernel (src/mcx_core.cl:3393-3512)
   with a real field. */
int  mcxg_adjoint_field(mcxg_session* s, int kind, const float* field, uint32_t ns, uint32_t nd, uint32_t nx,
                        uint32_t ny, uint32_t nz, uint32_t maxgate, float* out);
/* Field: the compensated accumulator in FP64, unscaled. */
int  mcxg_get_field_f64(mcxg_session* s, double* out);
/* Fluence gradient (no counterpart in the reference, which differentiates
   detector readings only, by replay): for a loss L of the raw flux or
   fluence field, dloss = dL/dfield (fieldlen floats).  Then mcxg_simulate
   with MCXG_ADJ1 and with MCXG_ADJ2 rerun the problem's photons (same seeds)
   and mcxg_get_adjoint_grad returns dL/dmua and dL/dmus per voxel (nvox
   floats each, per voxel-unit coefficient: multiply by unitinmm for per mm).
   The paths must not depend on mua: no Russian roulette. */
int  mcxg_set_adjoint(mcxg_session* s, const float* dloss, uint32_t n);
int  mcxg_get_adjoint_grad(mcxg_session* s, float* gmua, float* gmus);
/* The compensated field's raw planes (fieldlen x components each, NULL
   skips one): the int64 fixed-point counts and the float remainders; an
   element's value is count x 2^-S + remainder, with 2^-S the unit the host
   chose for the problem (field_scale in the host driver). */
int  mcxg_get_field_planes(mcxg_session* s, int64_t* counts, float* rem);
/* The precision check's fields of the last MCXG_VERIFY launch, unscaled,
   fieldlen values each (NULL skips one): the FP64 accumulation of the same
   deposits, the plain float accumulation, and the spill accumulation with
   its two planes added in float as the reference's host does
   (src/mcx_core.cl:2880-2886, src/mcx_host.cpp:1252-1257).  No counterpart
   in the reference: it exists to state the compensated field's error. */
int  mcxg_get_verify(mcxg_session* s, double* f64, float* plain, float* spill);
/* Weight and time of flight (s) of each saved detected photon when it was
   detected, 2 floats per record, in record order. */
int  mcxg_get_detweight(mcxg_session* s, float* out);
/* Detected photons: up to maxdetphoton records (reclen floats) and seeds
   (2 x uint64 each, when enabled); *detected = all detections, including
   those beyond the buffer. */
int  mcxg_get_detected(mcxg_session* s, float* detp, uint64_t* seeds, uint32_t* detected);
/* Event counters (exact kernel) and status words. */
int  mcxg_get_counters(mcxg_session* s, uint64_t counters[5], uint32_t status[2]);
/* Measured FP32 issue peak of the session's GPU in G FMA/s (one FMA = one
   FP32 operation): the denominator of the kernel's FP32 roofline. */
int  mcxg_fp32_peak(mcxg_session* s, double* gops);
/*
 * FP64 sums of per-thread {escaped, launched} weights, allocating nothing.
 * No counterpart in the reference (its host sums the weights in double after
 * reading them back, src/mcx_host.cpp:1303-1306).  For callers that cannot let
 * the library allocate device memory -- a service that reserves its device
 * budget at start-up, or a framework that owns every device buffer -- since
 * mcxg_get_energy needs a session and a session allocates with cudaMalloc.
 * d_energy: device array of 2 x nthread floats {escaped, launched} per thread;
 * d_sums: device array receiving 2 doubles {escaped, launched}.  Runs on the
 * legacy default stream of `device` and returns after the sums are written;
 * the calling thread's current device is the same on return as on entry.
 * Scratch: a static 64 KB device array, so nthread may not exceed 8,388,608
 * (MCXG_ERR_LIMIT beyond).  The first call on a device looks up that array's
 * device address (cudaGetSymbolAddress); make the first call before any
 * stream capture.  Every call shares the array: calls that overlap on the GPU
 * (other host threads, other streams) race.
 */
int  mcxg_energy_sum_noalloc(int device, const float* d_energy, uint32_t nthread, double* d_sums);
/* The persistent grid actually used by the last launch. */
int  mcxg_get_launch(mcxg_session* s, int* grid, int* block, int* regs);

#ifdef __cplusplus
}
#endif

#endif
