/*
 * mcx_host.c -- the C host driver of the GB300 transport path.
 *
 * Drop-in for the reference's simulation driver mcx_run_simulation
 * (src/mcx_host.cpp:438-1849) and the parts of its configuration layer the
 * path needs (src/mcx_utils.c: mcx_initcfg 203-366, mcx_clearcfg 368-476,
 * mcx_validatecfg 1822-1964, mcx_preprocess 1521-1809, mcx_maskdet
 * 4085-4198, mcx_normalize 1208-1218).  It keeps the reference's
 * observable semantics -- glibc rand() seeding per reference thread, the
 * float arithmetic of the photon split, the energy bookkeeping and the
 * normalisation factors -- and calls CUDA only through the mcxg_* layer.
 *
 * What is new: a persistent device session cached per GPU (buffers are reused
 * across calls), the label volume packed on the device to one byte per voxel
 * when every label fits in seven bits, and the FP64 energy sums and field
 * normalisation done on the GPU.
 */
#define _GNU_SOURCE
#include <malloc.h>
#include <math.h>
#include <pthread.h>
#include <setjmp.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../../include/mcx_gb300.h"
#include "mcx_json.h"
#include "mcx_kparams.h"

#define H_EPS        1e-10f        /* mcx_const.h:30 */
#define H_VERY_BIG   1e10f         /* mcx_const.h:35 */
#define R_C0         3.335640951981520e-12f
#define DET_MASK     0x80000000u
#define MED_MASK     0x7FFFFFFFu

/* ------------------------------------------------------------------ errors */

static __thread jmp_buf* g_jump = NULL;
static __thread Config* g_errcfg = NULL;

void mcx_error(const int id, const char* msg, const char* file, const int linenum) {
    if (g_jump && g_errcfg) {
        g_errcfg->errorcode = id ? id : -1;
        snprintf(g_errcfg->errormsg, sizeof(g_errcfg->errormsg), "%s", msg);
        longjmp(*g_jump, 1);
    }
    fprintf(stderr, "\nMCX ERROR(%d):%s in unit %s:%d\n", id, msg, file, linenum);
    exit(id);
}

#define MCX_ERROR(id, msg) mcx_error((id), (msg), __FILE__, __LINE__)

int mcx_last_error(const Config* cfg, const char** msg) {
    if (msg) {
        *msg = cfg->errormsg;
    }
    return cfg->errorcode;
}

const char* mcx_version(void) {
    return MCX_GB300_VERSION;
}

/* library mode: a failing public call returns instead of exiting */
#define MCX_ENTER(cfg)                                   \
    jmp_buf _jb;                                         \
    jmp_buf* _prev_jump = g_jump;                        \
    Config* _prev_cfg = g_errcfg;                        \
    (cfg)->errorcode = 0;                                \
    (cfg)->errormsg[0] = '\0';                           \
    if ((cfg)->parentid != mpStandalone) {               \
        g_jump = &_jb;                                   \
        g_errcfg = (cfg);                                \
        if (setjmp(_jb)) {                               \
            g_jump = _prev_jump;                         \
            g_errcfg = _prev_cfg;                        \
            return;                                      \
        }                                                \
    }

#define MCX_LEAVE()          \
    do {                     \
        g_jump = _prev_jump; \
        g_errcfg = _prev_cfg; \
    } while (0)

/* ------------------------------------------------------------------ config */

void mcx_initcfg(Config* cfg) {
    memset(cfg, 0, sizeof(*cfg));
    cfg->tstart = 0.f;
    cfg->tend = 5e-9f;
    cfg->tstep = 5e-9f;
    cfg->mediabyte = 1;
    cfg->steps.x = cfg->steps.y = cfg->steps.z = 1.f;
    cfg->nblocksize = 64;
    cfg->nthread = (1 << 14);
    cfg->seed = 0x623F9A9E;
    cfg->isreflect = 1;
    cfg->isnormalized = 1;
    cfg->issavedet = 1;
    cfg->respin = 1;
    cfg->maxjumpdebug = 10000000;
    cfg->issave2pt = 1;
    cfg->unitinmm = 1.f;
    cfg->flog = stdout;
    cfg->savedetflag = 0x5;
    cfg->his.savedetflag = cfg->savedetflag;
    cfg->gscatter = 1000000000u;
    cfg->maxvoidstep = 1000;
    cfg->voidtime = 1;
    cfg->maxdetphoton = 1000000;
    cfg->autopilot = 1;
    cfg->srcnum = 1;
    cfg->deviceid[0] = '1';
    cfg->isatomic = 1;
    cfg->srcpos.w = 1.f;
    memcpy(cfg->his.magic, "MCXH", 4);
    cfg->his.version = 1;
    cfg->his.unitinmm = 1.f;
    cfg->his.normalizer = 1.f;
    cfg->his.srcnum = 1;
    cfg->his.respin = 1;
    cfg->parentid = mpStandalone;
    cfg->outputtype = otFlux;
    cfg->srciquv.x = 1.f;          /* unpolarised launch (mcx_utils.c:338-339) */
}

void mcx_clearcfg(Config* cfg) {
    free(cfg->prop);
    free(cfg->detpos);
    free(cfg->vol);
    free(cfg->srcpattern);
    free(cfg->exportfield);
    free(cfg->exportdetected);
    free(cfg->seeddata);
    free(cfg->invcdf);
    free(cfg->angleinvcdf);
    free(cfg->srcdata);
    free(cfg->exportenergy);
    free(cfg->exportdetweight);
    cfg->exportdetweight = NULL;
    free(cfg->detdir);
    free(cfg->exportjacob);
    cfg->detdir = NULL;
    cfg->exportjacob = NULL;
    free(cfg->replay.seed);
    free(cfg->replay.weight);
    free(cfg->replay.tof);
    free(cfg->replay.detid);
    memset(&cfg->replay, 0, sizeof(cfg->replay));
    free(cfg->polprop);
    free(cfg->smatrix);
    free(cfg->exportdebugdata);
    cfg->polprop = NULL;
    cfg->smatrix = NULL;
    cfg->exportdebugdata = NULL;
    cfg->debugdatalen = 0;
    cfg->polmedianum = 0;
    cfg->exportenergy = NULL;
    cfg->prop = NULL;
    cfg->detpos = NULL;
    cfg->vol = NULL;
    cfg->srcpattern = NULL;
    cfg->exportfield = NULL;
    cfg->exportdetected = NULL;
    cfg->seeddata = NULL;
    cfg->invcdf = NULL;
    cfg->angleinvcdf = NULL;
    cfg->srcdata = NULL;
    cfg->medianum = 0;
    cfg->detnum = 0;
    cfg->extrasrclen = 0;
}

void mcx_normalize(float field[], float scale, int fieldlen, int option, int pidx, int srcnum) {
    for (int i = 0; i < fieldlen; i++) {
        if (option == 2 && field[i * srcnum + pidx] < 0.f) {
            continue;
        }
        field[i * srcnum + pidx] *= scale;
    }
}

unsigned int mcx_detreclen(const Config* cfg) {
    unsigned int f = cfg->savedetflag;
    unsigned int partial = (cfg->medianum - 1) * (SAVE_NSCAT(f) + SAVE_PPATH(f) + SAVE_MOM(f));
    return partial + SAVE_DETID(f) + 3 * (SAVE_PEXIT(f) + SAVE_VEXIT(f)) + SAVE_W0(f) + 4 * SAVE_IQUV(f);
}

/* mcx_lookupindex (mcx_utils.c:5292-5305): face conditions "_ramc", detector flags "01" */
static int lookup_index(char* key, const char* table) {
    for (int i = 0; table[i]; i++) {
        char c = *key;
        if (c >= 'A' && c <= 'Z') {
            c = (char)(c - 'A' + 'a');
        }
        if (c == table[i]) {
            *key = (char)i;
            return 0;
        }
    }
    return 1;
}

/* mcx_maskdet (mcx_utils.c:4085-4198): mark the boundary voxels within a
   detector's reach with the detector bit */
/* mcx_prep_polarized (mcx_utils.c:1483-1519): the Mueller tables of each
   label's scatterers from Mie theory, and the label's mua, n, mus and g from
   them; a given mus (and g) sets the sphere density so that the label keeps
   its mus (or its reduced mus), in the reference's float / double mix */
static void prep_polarized(Config* cfg) {
    free(cfg->smatrix);
    cfg->smatrix = (mcx_float4*)malloc(sizeof(mcx_float4) * MCX_NANGLES * cfg->polmedianum);
    if (!cfg->smatrix) {
        MCX_ERROR(-2, "out of host memory");
    }
    for (unsigned int i = 0; i < cfg->polmedianum; i++) {
        Medium* m = &cfg->prop[i + 1];
        POLMedium* q = &cfg->polprop[i];
        m->mua = q->mua;
        m->n = q->nmed;
        double qsca, g;
        const double x = (double)(6.28318530717959f * q->r * q->nmed) / ((double)cfg->lambda * 1e-3);
        const double A = (double)(3.1415926535897932f * q->r * q->r);
        if (mcx_mie(x, (double)(q->nsph / q->nmed), (float*)(cfg->smatrix + i * MCX_NANGLES), &qsca, &g)) {
            MCX_ERROR(-6, "invalid Mie scatterer (radius, indices and wavelength must be positive)");
        }
        if (m->mus > H_EPS) {
            float target_mus = m->mus;
            if (m->g < 1.f - H_EPS) {
                const float target_musp = m->mus * (1.0f - m->g);
                target_mus = (float)(target_musp / (1.0 - g));
            }
            q->rho = (float)(target_mus / qsca / A * 1e-3);
        }
        m->mus = (float)(qsca * A * q->rho * 1e3);
        m->g = (float)g;
    }
}

/* The reference masks detectors on a copy of the volume padded by one void
   voxel on every side (mcx_utils.c:4085-4198); the same lookups are made here
   on the volume itself, at padded coordinates (1..n inside, 0 and n + 1 the
   void padding), so no padded copy is built (the head volume: 29 MB). */
static inline uint32_t pad_at(const uint32_t* vol, unsigned int nx, unsigned int ny, unsigned int nz, int x, int y, int z) {
    if (x < 1 || y < 1 || z < 1 || x > (int)nx || y > (int)ny || z > (int)nz) {
        return 0u;
    }
    return vol[((size_t)(z - 1) * ny + (size_t)(y - 1)) * nx + (size_t)(x - 1)];
}

/* a voxel lies on an interface when any of its 26 neighbours is void (label 0) */
static int touches_void(const uint32_t* vol, unsigned int nx, unsigned int ny, unsigned int nz, int x, int y, int z) {
    for (int k = -1; k <= 1; k++) {
        for (int j = -1; j <= 1; j++) {
            for (int l = -1; l <= 1; l++) {
                if ((k || j || l) && !pad_at(vol, nx, ny, nz, x + l, y + j, z + k)) {
                    return 1;
                }
            }
        }
    }
    return 0;
}

/* Two passes, so every test reads the volume as it was before masking (as
   the reference's padded copy does): the voxels to mark first, then the
   marks. */
static void maskdet(Config* cfg) {
    unsigned int nx = cfg->dim.x, ny = cfg->dim.y, nz = cfg->dim.z;
    int isonecube = (nx == 1) && (ny == 1) && (nz == 1);
    static const float corners[8][3] = {{0.f, 0.f, 0.f}, {1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f},
        {1.f, 1.f, 0.f}, {1.f, 0.f, 1.f}, {0.f, 1.f, 1.f}, {1.f, 1.f, 1.f}
    };
    size_t nmark = 0, capmark = 0;
    size_t* mark = NULL;
    for (unsigned int d = 0; d < cfg->detnum; d++) {
        const mcx_float4 dp = cfg->detpos[d];
        float d2max = (dp.w + 1.7321f) * (dp.w + 1.7321f);
        unsigned int count = 0;
        for (float z = -dp.w - 1.f; z <= dp.w + 1.f; z += 0.5f) {
            float iz = z + dp.z;
            for (float y = -dp.w - 1.f; y <= dp.w + 1.f; y += 0.5f) {
                float iy = y + dp.y;
                for (float x = -dp.w - 1.f; x <= dp.w + 1.f; x += 0.5f) {
                    float ix = x + dp.x;
                    if (iz < 0 || ix < 0 || iy < 0 || ix >= nx || iy >= ny || iz >= nz ||
                            x * x + y * y + z * z > (dp.w + 1.f) * (dp.w + 1.f)) {
                        continue;
                    }
                    float mind2 = H_VERY_BIG;
                    for (int c = 0; c < 8; c++) {
                        float rx = (int)ix - dp.x + corners[c][0];
                        float ry = (int)iy - dp.y + corners[c][1];
                        float rz = (int)iz - dp.z + corners[c][2];
                        float d2 = rx * rx + ry * ry + rz * rz;
                        if (d2 > d2max) {
                            mind2 = H_VERY_BIG;
                            break;
                        }
                        if (d2 < mind2) {
                            mind2 = d2;
                        }
                    }
                    if (mind2 == H_VERY_BIG ||
                            mind2 >= (dp.w + 0.5f * (1.f + isonecube)) * (dp.w + 0.5f * (1.f + isonecube))) {
                        continue;
                    }
                    const int px = (int)(ix + 1.f), py = (int)(iy + 1.f), pz = (int)(iz + 1.f);
                    const uint32_t v = pad_at(cfg->vol, nx, ny, nz, px, py, pz);
                    int hit;
                    if (cfg->mediabyte == 97) {
                        /* split voxels: those with a background lower half (mcx_utils.c:4155-4165) */
                        hit = !(v & 0xFF000000u) && (v & 0x00FF0000u);
                    } else {
                        hit = v && touches_void(cfg->vol, nx, ny, nz, px, py, pz);
                    }
                    if (hit) {
                        if (nmark == capmark) {
                            capmark = capmark ? 2 * capmark : 4096;
                            size_t* grown = (size_t*)realloc(mark, capmark * sizeof(size_t));
                            if (!grown) {
                                free(mark);
                                MCX_ERROR(-2, "out of host memory while masking detectors");
                            }
                            mark = grown;
                        }
                        mark[nmark++] = (size_t)(int)iz * ny * nx + (size_t)(int)iy * nx + (size_t)(int)ix;
                        count++;
                    }
                }
            }
        }
        if (count == 0 && cfg->flog) {
            fprintf(cfg->flog, "MCX WARNING: detector %u is not located on an interface, please check coordinates.\n",
                    d + 1);
        }
    }
    for (size_t i = 0; i < nmark; i++) {
        cfg->vol[mark[i]] |= DET_MASK;
    }
    free(mark);
}

/* row-major (C) to column-major volume, mcx_convertrow2col */
static void row2col(Config* cfg) {
    size_t nx = cfg->dim.x, ny = cfg->dim.y, nz = cfg->dim.z;
    uint32_t* out = (uint32_t*)malloc(nx * ny * nz * sizeof(uint32_t));
    if (!out) {
        MCX_ERROR(-2, "out of host memory");
    }
    for (size_t x = 0; x < nx; x++) {
        for (size_t y = 0; y < ny; y++) {
            for (size_t z = 0; z < nz; z++) {
                out[z * ny * nx + y * nx + x] = cfg->vol[x * ny * nz + y * nz + z];
            }
        }
    }
    free(cfg->vol);
    cfg->vol = out;
}

static void point_src_voxel(const Config* cfg, mcx_float4 pos, mcx_float4* p2) {
    union {
        float f;
        uint32_t u;
    } f2i;
    if (pos.x < 0.f || pos.y < 0.f || pos.z < 0.f || pos.x >= cfg->dim.x || pos.y >= cfg->dim.y || pos.z >= cfg->dim.z) {
        f2i.u = 0;
        p2->z = f2i.f;
        p2->w = f2i.f;
    } else {
        uint32_t idx = (uint32_t)((int)(floorf(pos.z)) * (cfg->dim.y * cfg->dim.x) + (int)(floorf(pos.y)) * cfg->dim.x +
                                  (int)(floorf(pos.x)));
        f2i.u = idx;
        p2->z = f2i.f;
        f2i.u = cfg->vol[idx] & MED_MASK;
        p2->w = f2i.f;
    }
}

/* mcx_preprocess, mcx_utils.c:1521-1809 (the parts the transport path reads) */
static void preprocess(Config* cfg) {
    int isbcdet = 0;
    double tmp = sqrt((double)cfg->srcdir.x * cfg->srcdir.x + (double)cfg->srcdir.y * cfg->srcdir.y +
                      (double)cfg->srcdir.z * cfg->srcdir.z);
    if (tmp < H_EPS) {
        MCX_ERROR(-4, "source initial direction vector can not have a length of 0");
    }
    tmp = 1.f / tmp;
    cfg->srcdir.x *= tmp;
    cfg->srcdir.y *= tmp;
    cfg->srcdir.z *= tmp;

    for (int i = 0; i < 6; i++) {
        if (cfg->bc[i] && lookup_index(cfg->bc + i, "_ramc")) {
            MCX_ERROR(-4, "unknown boundary condition specifier");
        }
    }
    for (int i = 6; i < 12; i++) {
        if (cfg->bc[i] && lookup_index(cfg->bc + i, "01")) {
            MCX_ERROR(-4, "unknown boundary detection flags");
        }
        if (cfg->bc[i]) {
            isbcdet = 1;
        }
    }
    if (cfg->medianum == 0) {
        MCX_ERROR(-4, "you must define the 'prop' field in the input structure");
    }
    if (cfg->dim.x == 0 || cfg->dim.y == 0 || cfg->dim.z == 0 || !cfg->vol) {
        MCX_ERROR(-4, "the 'vol' field in the input structure can not be empty");
    }
    if ((cfg->srctype == MCX_SRC_PATTERN || cfg->srctype == MCX_SRC_PATTERN3D) && cfg->srcpattern == NULL) {
        MCX_ERROR(-4, "the 'srcpattern' field can not be empty when your 'srctype' is 'pattern'");
    }
    if (cfg->polprop && cfg->polmedianum) {
        /* mcx_preprocess (mcx_utils.c:1536-1549), before the unit scaling of the properties */
        if (!(cfg->mediabyte <= 4)) {
            MCX_ERROR(-1, "Unsupported media format for polarized simulation");
        }
        if (cfg->medianum != cfg->polmedianum + 1) {
            MCX_ERROR(-6, "number of particle types does not match number of media");
        }
        if (cfg->lambda == 0.f) {
            MCX_ERROR(-1, "you must specify light wavelength lambda to run polarized photon simulation");
        }
        if (cfg->omega > 0.f) {
            MCX_ERROR(-6, "the polarised transport can not be combined with the frequency-domain transport");
        }
        if (cfg->dim.x == 1 || cfg->dim.y == 1 || cfg->dim.z == 1) {
            MCX_ERROR(-6, "the polarised transport takes a 3-D domain in this build");
        }
        prep_polarized(cfg);
    }
    if (cfg->steps.x != 1.f && cfg->unitinmm == 1.f) {
        cfg->unitinmm = cfg->steps.x;
    }
    if (cfg->unitinmm != 1.f) {
        cfg->steps.x = cfg->steps.y = cfg->steps.z = cfg->unitinmm;
        for (unsigned int i = 1; i < cfg->medianum; i++) {
            cfg->prop[i].mus *= cfg->unitinmm;
            cfg->prop[i].mua *= cfg->unitinmm;
        }
    }
    if (cfg->isrowmajor) {
        row2col(cfg);
        cfg->isrowmajor = 0;
    }
    if (cfg->debuglevel & 8) {
        /* MCX_DEBUG_MOVE_ONLY: trajectories only, no field and no detected
           photons (mcx_utils.c:1552-1555) */
        cfg->issave2pt = 0;
        cfg->issavedet = 0;
    }
    if (cfg->issavedet && cfg->detnum == 0 && isbcdet == 0) {
        cfg->issavedet = 0;
    }
    if (cfg->issavedet == 0) {
        cfg->issaveexit = 0;
        cfg->ismomentum = 0;
        if (cfg->seed != SEED_FROM_FILE) {
            cfg->savedetflag = 0;  /* a replay keeps the flags describing its input records */
        }
    }
    if (cfg->respin == 0) {
        MCX_ERROR(-1, "respin number can not be 0, check your -r/--repeat input or cfg.respin value");
    }
    if (cfg->respin < 0) {
        MCX_ERROR(-1, "negative respin (photon divisions) is not supported by this build");
    }
    for (unsigned int i = 0; i < cfg->medianum; i++) {
        if (cfg->prop[i].mus == 0.f && !cfg->polmedianum) {
            cfg->prop[i].mus = H_EPS;
        }
    }
    if (cfg->srcpos.w == 0.f) {
        cfg->srcpos.w = 1.f;
    }
    if (cfg->extrasrclen) {
        if (cfg->srcnum > 1) {
            MCX_ERROR(-4, "simulating multiple sources currently can not be used with photon-sharing");
        }
        if (cfg->srcid > (int)cfg->extrasrclen + 1) {
            MCX_ERROR(-4, "srcid exceeds total defined source count");
        }
        for (unsigned int i = 0; i < cfg->extrasrclen; i++) {
            if (cfg->srcdata[i].srcpos.w == 0.f) {
                cfg->srcdata[i].srcpos.w = 1.f;
            }
        }
    }
    if (cfg->srcnum > 1 && (cfg->srctype == MCX_SRC_PATTERN || cfg->srctype == MCX_SRC_PATTERN3D)) {
        if (cfg->seed == SEED_FROM_FILE) {
            MCX_ERROR(-4, "photon sharing (srcnum > 1) can not be replayed by this build");
        }
        if (cfg->srcnum > 256) {
            MCX_ERROR(-4, "photon sharing takes at most 256 patterns");
        }
    }
    size_t nvox = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
    if (cfg->mediabyte <= 4) {
        /* eight running maxima, so the compiler can keep them in one vector */
        unsigned int m8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        size_t i = 0;
        for (; i + 8 <= nvox; i += 8) {
            for (int k = 0; k < 8; k++) {
                const unsigned int l = cfg->vol[i + k] & MED_MASK;
                m8[k] = l > m8[k] ? l : m8[k];
            }
        }
        unsigned int maxlabel = 0;
        for (; i < nvox; i++) {
            const unsigned int l = cfg->vol[i] & MED_MASK;
            maxlabel = l > maxlabel ? l : maxlabel;
        }
        for (int k = 0; k < 8; k++) {
            maxlabel = m8[k] > maxlabel ? m8[k] : maxlabel;
        }
        if (cfg->medianum <= maxlabel) {
            MCX_ERROR(-4, "input media optical properties are less than the labels in the volume");
        }
    } else if (cfg->mediabyte == 99) {
        for (size_t i = 0; i < nvox; i++) {
            if ((cfg->vol[i] & 0x3FFFu) >= cfg->medianum) {
                MCX_ERROR(-4, "input media optical properties are less than the labels in the volume");
            }
        }
    } else if (cfg->mediabyte == 97) {
        /* split voxels: lower and upper labels in the top bytes of the first plane */
        for (size_t i = 0; i < nvox; i++) {
            if (((cfg->vol[i] >> 24) & 0x7Fu) >= cfg->medianum || ((cfg->vol[i] >> 16) & 0xFFu) >= cfg->medianum) {
                MCX_ERROR(-4, "input media optical properties are less than the labels in the volume");
            }
        }
    } else if (cfg->mediabyte < 100 || cfg->mediabyte > 104) {
        MCX_ERROR(-4, "this build supports label volumes (mediabyte 1/2/4), label + half property (99), half "
                  "mua/mus (100, 102), float mua (101), byte (103) and short (104) mixtures");
    }
    if (cfg->srctype <= MCX_SRC_CONE || cfg->srctype == MCX_SRC_ARCSINE || cfg->srctype == MCX_SRC_ZGAUSSIAN) {
        point_src_voxel(cfg, cfg->srcpos, &cfg->srcparam2);
        for (unsigned int i = 0; i < cfg->extrasrclen; i++) {
            point_src_voxel(cfg, cfg->srcdata[i].srcpos, &cfg->srcdata[i].srcparam2);
        }
    }
    if (cfg->issavedet) {
        maskdet(cfg);
    }
    for (int i = 0; i < MAX_DEVICE; i++) {
        if (cfg->deviceid[i] == '0') {
            cfg->deviceid[i] = '\0';
        }
    }
    if ((cfg->mediabyte == 100 || cfg->mediabyte == MEDIA_MUA_FLOAT || cfg->mediabyte == 102) && cfg->medianum < 2) {
        MCX_ERROR(-4, "the 'prop' field must contain at least 2 rows for the requested media format");
    }
    if ((cfg->mediabyte == 103 || cfg->mediabyte == 104) && cfg->medianum < 3) {
        MCX_ERROR(-4, "the 'prop' field must contain at least 3 rows for the requested media format");
    }
    if (cfg->ismomentum) {
        cfg->savedetflag |= 0x8;
    }
    if (cfg->issaveexit) {
        cfg->savedetflag |= 0x10 | 0x20;
    }
    if (cfg->polmedianum && cfg->polprop) {
        /* a polarised run records partial paths, exit direction, initial weight
           and the Stokes vector (mcx_utils.c:1777-1784) */
        cfg->savedetflag |= 0x4 | 0x20 | 0x40 | 0x80;
    } else {
        cfg->savedetflag &= ~0x80u;
    }
    if (cfg->issavedet && cfg->savedetflag == 0) {
        cfg->savedetflag = 0x5;
    }
    if (cfg->mediabyte >= 100 && cfg->savedetflag) {
        cfg->savedetflag &= ~(0x2u | 0x4u | 0x8u);
    }
    if (cfg->issaveref > 1) {
        MCX_ERROR(-4, "issaveref > 1 (per-voxel exit partial paths) is not supported by this build");
    }
}

/* mcx_replayinit (mcx_utils.c:1355-1421): keep the records of detector
   replaydet (all when <= 0) and of source srcid, compute each one's detected
   weight and time of flight from its partial paths, drop those outside the
   time window, and compact the seeds to match. */
static void replayinit(Config* cfg, const float* detps, const int dimdetps[2], int seedbyte) {
    if (cfg->seed == SEED_FROM_FILE && detps == NULL && cfg->replay.seed && cfg->replay.weight && cfg->replay.tof &&
            cfg->replay.detid) {
        /* the caller gave each photon's weight, time of flight and detector id
           directly (replays of float-mua volumes, whose records carry no
           partial paths, and gradient replays with per-photon factors) */
        for (size_t i = 0; i < cfg->nphoton; i++) {
            int d = cfg->replay.detid[i] & 0xFFFF;
            if (cfg->replaydet == -1 && (d < 1 || d > (int)cfg->detnum)) {
                MCX_ERROR(-6, "a replayed record carries a detector id outside 1..detnum");
            }
            if (cfg->replay.tof[i] < cfg->tstart || cfg->replay.tof[i] > cfg->tend) {
                MCX_ERROR(-6, "a replayed photon's time of flight lies outside the time window");
            }
        }
        return;
    }
    if (cfg->seed == SEED_FROM_FILE && detps == NULL) {
        MCX_ERROR(-6, "you give cfg.seed for replay, but did not specify cfg.detphotons.\nPlease define it as the "
                  "detphoton output from the baseline simulation\n");
    }
    if (detps == NULL || cfg->seed != SEED_FROM_FILE) {
        return;
    }
    if (!cfg->replay.seed) {
        MCX_ERROR(-6, "the seed input is empty");
    }
    if (cfg->nphoton != (size_t)dimdetps[1]) {
        MCX_ERROR(-6, "the column numbers of detphotons and seed do not match\n");
    }
    if (seedbyte == 0) {
        MCX_ERROR(-6, "the seed input is empty");
    }
    if (seedbyte != 16) {
        MCX_ERROR(-6, "the row number of cfg.seed does not match RNG seed byte-length");
    }
    int hasdetid = SAVE_DETID(cfg->savedetflag);
    unsigned int offset = SAVE_NSCAT(cfg->savedetflag) * (cfg->medianum - 1);
    if (((!hasdetid) && cfg->detnum > 1) || !SAVE_PPATH(cfg->savedetflag)) {
        MCX_ERROR(-6, "please rerun the baseline simulation and save detector ID (D) and partial-path (P) using "
                  "cfg.savedetflag='dp' ");
    }
    if ((unsigned int)dimdetps[0] < (unsigned int)hasdetid + offset + cfg->medianum - 1) {
        MCX_ERROR(-6, "the row number of detphotons is less than the record length implied by savedetflag");
    }
    size_t n = (size_t)dimdetps[1];
    free(cfg->replay.weight);
    free(cfg->replay.tof);
    free(cfg->replay.detid);
    cfg->replay.weight = (float*)malloc(sizeof(float) * (n ? n : 1));
    cfg->replay.tof = (float*)calloc(n ? n : 1, sizeof(float));
    cfg->replay.detid = (int*)calloc(n ? n : 1, sizeof(int));
    if (!cfg->replay.weight || !cfg->replay.tof || !cfg->replay.detid) {
        MCX_ERROR(-2, "out of host memory");
    }
    size_t kept = 0;
    for (size_t i = 0; i < n; i++) {
        const float* rec = detps + i * (size_t)dimdetps[0];
        int did = (int)rec[0];
        if (!(cfg->replaydet <= 0 || cfg->replaydet == (did & 0xFFFF))) {
            continue;
        }
        if (!(cfg->srcid <= 0 || ((did & 0xFFFF0000) && cfg->srcid == (int)(((unsigned int)did & 0xFFFF0000u) >> 16)))) {
            continue;
        }
        if (i != kept) {
            memmove((char*)cfg->replay.seed + kept * 16, (char*)cfg->replay.seed + i * 16, 16);
        }
        cfg->replay.weight[kept] = 1.f;
        cfg->replay.tof[kept] = 0.f;
        cfg->replay.detid[kept] = hasdetid ? did : 1;
        for (unsigned int j = (unsigned int)hasdetid; j < cfg->medianum - 1 + (unsigned int)hasdetid; j++) {
            float plen = rec[offset + j];
            cfg->replay.weight[kept] *= expf(-cfg->prop[j - hasdetid + 1].mua * plen);
            plen *= cfg->unitinmm;
            cfg->replay.tof[kept] += plen * R_C0 * cfg->prop[j - hasdetid + 1].n;
        }
        if (cfg->replay.tof[kept] < cfg->tstart || cfg->replay.tof[kept] > cfg->tend) {
            continue;
        }
        if (cfg->replaydet == -1 && ((cfg->replay.detid[kept] & 0xFFFF) < 1 ||
                                     (cfg->replay.detid[kept] & 0xFFFF) > (int)cfg->detnum)) {
            MCX_ERROR(-6, "a replayed record carries a detector id outside 1..detnum");
        }
        kept++;
    }
    cfg->nphoton = kept;
}

void mcx_validatecfg(Config* cfg, float* detps, int dimdetps[2], int seedbyte) {
    MCX_ENTER(cfg);
    if (cfg->seed == SEED_FROM_FILE && cfg->replaydet > (int)cfg->detnum) {
        MCX_ERROR(-4, "replay detector ID exceeds the maximum detector number");
    }
    if (cfg->replaydet == -1 && cfg->detnum == 1) {
        cfg->replaydet = 1;
    }
    if (!cfg->issrcfrom0) {
        cfg->srcpos.x--;
        cfg->srcpos.y--;
        cfg->srcpos.z--;
        for (unsigned int i = 0; i < cfg->extrasrclen; i++) {
            cfg->srcdata[i].srcpos.x--;
            cfg->srcdata[i].srcpos.y--;
            cfg->srcdata[i].srcpos.z--;
        }
    }
    if (cfg->tstart > cfg->tend || cfg->tstep == 0.f) {
        MCX_ERROR(-6, "incorrect time gate settings");
    }
    if (fabs(cfg->srcdir.x * cfg->srcdir.x + cfg->srcdir.y * cfg->srcdir.y + cfg->srcdir.z * cfg->srcdir.z - 1.f) > 1e-5) {
        MCX_ERROR(-6, "field 'srcdir' must be a unitary vector");
    }
    if (cfg->steps.x == 0.f || cfg->steps.y == 0.f || cfg->steps.z == 0.f) {
        MCX_ERROR(-6, "field 'steps' can not have zero elements");
    }
    if (cfg->tend <= cfg->tstart) {
        MCX_ERROR(-6, "field 'tend' must be greater than field 'tstart'");
    }
    int gates = (int)((cfg->tend - cfg->tstart) / cfg->tstep + 0.5);
    if (cfg->maxgate > (unsigned int)gates) {
        cfg->maxgate = gates;
    }
    int replayout = cfg->outputtype == otJacobian || cfg->outputtype == otWP || cfg->outputtype == otDCS ||
                    cfg->outputtype == otRF || cfg->outputtype == otRFmus || cfg->outputtype == otWLTOF ||
                    cfg->outputtype == otWPTOF;
    if (replayout && cfg->seed != SEED_FROM_FILE) {
        MCX_ERROR(-6, "Jacobian output is only valid in the reply mode. Please define cfg.seed");
    }
    if (cfg->omega < 0.f) {
        MCX_ERROR(-6, "the modulation frequency omega must not be negative");
    }
    if (cfg->omega > 0.f && MCX_IS_ADJOINT_TYPE(cfg->outputtype)) {
        MCX_ERROR(-6, "frequency-domain adjoint outputs are not supported by this build");
    }
    if (cfg->omega > 0.f && cfg->srcnum > 1 && (cfg->srctype == MCX_SRC_PATTERN || cfg->srctype == MCX_SRC_PATTERN3D)) {
        MCX_ERROR(-6, "the frequency-domain transport can not be combined with photon sharing");
    }
    if (!replayout && cfg->outputtype != otFlux && cfg->outputtype != otFluence && cfg->outputtype != otEnergy &&
            cfg->outputtype != otL && !MCX_IS_ADJOINT_TYPE(cfg->outputtype)) {
        MCX_ERROR(-6, "unsupported output type");
    }
    if (MCX_IS_ADJOINT_TYPE(cfg->outputtype) && (cfg->detnum == 0 || cfg->detdir == NULL)) {
        MCX_ERROR(-6, "adjoint outputs need detectors with directions (cfg.detdir)");
    }
    /* adjoint outputs: each detector becomes an extra source at its position,
       along its direction, radius in srcparam1.x, sharing photons with the
       sources (mcx_utils.c:1902-1926; the positions are taken before the
       detectors' own conversion to 0-based, as there) */
    if ((MCX_IS_ADJOINT_TYPE(cfg->outputtype) || cfg->srcid == -2) && cfg->seed != SEED_FROM_FILE && cfg->detnum > 0 &&
            cfg->detdir != NULL) {
        unsigned int orig = cfg->extrasrclen;
        ExtraSrc* ns = (ExtraSrc*)realloc(cfg->srcdata, (orig + cfg->detnum) * sizeof(ExtraSrc));
        if (!ns) {
            MCX_ERROR(-2, "out of host memory");
        }
        cfg->srcdata = ns;
        memset(cfg->srcdata + orig, 0, cfg->detnum * sizeof(ExtraSrc));
        for (unsigned int i = 0; i < cfg->detnum; i++) {
            cfg->srcdata[orig + i].srcpos.x = cfg->detpos[i].x;
            cfg->srcdata[orig + i].srcpos.y = cfg->detpos[i].y;
            cfg->srcdata[orig + i].srcpos.z = cfg->detpos[i].z;
            cfg->srcdata[orig + i].srcpos.w = 1.f;
            cfg->srcdata[orig + i].srcdir = cfg->detdir[i];
            cfg->srcdata[orig + i].srcparam1.x = cfg->detpos[i].w;
        }
        cfg->extrasrclen += cfg->detnum;
        if (MCX_IS_ADJOINT_TYPE(cfg->outputtype)) {
            cfg->srcid = -1;
        }
    }
    if (!cfg->issrcfrom0) {
        for (unsigned int i = 0; i < cfg->detnum; i++) {
            cfg->detpos[i].x--;
            cfg->detpos[i].y--;
            cfg->detpos[i].z--;
        }
    }
    preprocess(cfg);
    cfg->his.maxmedia = cfg->medianum - 1;
    cfg->his.detnum = cfg->detnum;
    cfg->his.srcnum = cfg->srcnum;
    cfg->his.colcount = mcx_detreclen(cfg);
    cfg->his.savedetflag = cfg->savedetflag;
    cfg->his.totalsource = ((cfg->srcid <= 0) ? cfg->extrasrclen + 1 : 1);
    replayinit(cfg, detps, dimdetps, seedbyte);
    MCX_LEAVE();
}

/* ------------------------------------------------------------- JSON input */

/* mcx_parsejson (src/mcx_utils.c, called from mcx_readconfig 2041): the JSON
   text into cfg, then what the reference's mcx_prepdomain does after
   loading (0-based positions, volume preprocessing, detector mask) through
   mcx_validatecfg: cfg is ready for mcx_run_simulation. */
void mcx_parsejson(char* jbuf, Config* cfg) {
    MCX_ENTER(cfg);
    char err[256];
    if (!jbuf) {
        MCX_ERROR(-1, "no JSON input");
    }
    const int rc = mcxj_load(jbuf, cfg, err, sizeof(err));
    if (rc) {
        MCX_ERROR(rc, err);
    }
    MCX_LEAVE();
    mcx_validatecfg(cfg, NULL, NULL, 0);
}

/* mcx_readconfig (src/mcx_utils.c:2011-2071): a .json input file, or the
   JSON text itself when the name starts with '{'.  The reference's legacy
   .inp text format is not read by this build. */
void mcx_readconfig(char* fname, Config* cfg) {
    MCX_ENTER(cfg);
    char err[256];
    if (!fname || !fname[0]) {
        MCX_ERROR(-2, "reading the configuration from standard input is not supported by this build");
    }
    char* text = fname;
    if (fname[0] != '{') {
        if (!strstr(fname, ".json")) {
            MCX_ERROR(-2, "this build reads JSON input files (.json) only");
        }
        FILE* fp = fopen(fname, "rb");
        if (!fp) {
            MCX_ERROR(-2, "can not load the specified config file");
        }
        long len = -1;
        if (fseek(fp, 0, SEEK_END) == 0) {
            len = ftell(fp);
        }
        text = (len >= 0) ? (char*)malloc((size_t)len + 1) : NULL;
        if (!text || fseek(fp, 0, SEEK_SET) != 0 || fread(text, 1, (size_t)len, fp) != (size_t)len) {
            fclose(fp);
            free(text);
            MCX_ERROR(-2, "reading input file is terminated");
        }
        fclose(fp);
        text[len] = '\0';
    }
    const int rc = mcxj_load(text, cfg, err, sizeof(err));
    if (text != fname) {
        free(text);
    }
    if (rc) {
        MCX_ERROR(rc, err);
    }
    if (cfg->session[0] == '\0') {
        snprintf(cfg->session, sizeof(cfg->session), "%s", fname);
    }
    MCX_LEAVE();
    mcx_validatecfg(cfg, NULL, NULL, 0);
}

/* ----------------------------------------------------------------- devices */

/* mcx_nv_corecount (mcx_host.cpp:224-240) */
static int nv_corecount(int v1, int v2) {
    int v = v1 * 10 + v2;
    if (v < 20) {
        return 8;
    } else if (v < 21) {
        return 32;
    } else if (v < 30) {
        return 48;
    } else if (v < 50) {
        return 192;
    } else if (v < 60 || v == 61 || v >= 89) {
        return 128;
    }
    return 64;
}

int mcx_list_gpu(Config* cfg, unsigned int* activedev, GPUInfo** info) {
    int n = 0;
    unsigned int act = 0;
    *info = NULL;
    if (activedev) {
        *activedev = 0;
    }
    if (mcxg_device_count(&n) != MCXG_OK || n <= 0) {
        return 0;
    }
    *info = (GPUInfo*)calloc((size_t)n, sizeof(GPUInfo));
    for (int i = 0; i < n; i++) {
        mcxg_devinfo d;
        if (mcxg_device_info(i, &d) != MCXG_OK) {
            continue;
        }
        int selected = (i < MAX_DEVICE && cfg->deviceid[i] == '1');
        if (!selected && activedev) {
            continue;
        }
        GPUInfo* g = (*info) + act;
        memset(g, 0, sizeof(*g));
        snprintf(g->name, sizeof(g->name), "%s", d.name);
        g->id = i + 1;
        g->devcount = n;
        g->major = d.major;
        g->minor = d.minor;
        g->globalmem = d.globalmem;
        g->constmem = d.constmem;
        g->sharedmem = d.sharedmem_per_block;
        g->regcount = d.regs_per_block;
        g->clock = d.clock_khz / 1000;
        g->sm = d.sm;
        g->core = d.sm * nv_corecount(d.major, d.minor);
        g->autoblock = 64;
        g->autothread = g->autoblock * (size_t)g->core;
        g->maxgate = cfg->maxgate;
        g->maxmpthread = d.max_threads_per_sm;
        g->vendor = 1;
        if (cfg->isgpuinfo && cfg->flog) {
            fprintf(cfg->flog, "============ GPU device ID %d [%d of %d]: %s  ============\n", i, i + 1, n, g->name);
            fprintf(cfg->flog, " Compute units   :\t%d core(s)\n", g->sm);
            fprintf(cfg->flog, " Global memory   :\t%.0f B\n", (double)g->globalmem);
            fprintf(cfg->flog, " Local memory    :\t%.0f B\n", (double)g->sharedmem);
            fprintf(cfg->flog, " Constant memory :\t%.0f B\n", (double)g->constmem);
            fprintf(cfg->flog, " Clock speed     :\t%d MHz\n", g->clock);
            fprintf(cfg->flog, " Compute Capacity:\t%d.%d\n", g->major, g->minor);
            fprintf(cfg->flog, " Stream Processor:\t%d\n", g->core);
        }
        act++;
    }
    if (activedev) {
        *activedev = act;
    }
    return (int)act;
}

/* Output buffers handed back with mcx_free_buffer, kept for the next run's
   field and detected records: their pages are resident, so the copies from
   the device skip the first-touch page faults (a 43 MB field: 1.7 ms into
   new pages, 0.3 ms into resident ones).  Buffers of 1 MB and more, at most
   8 of them and 1 GB; released with the device sessions. */
#define OUTCACHE_N 8
/* 1: device sessions stay cached per GPU between calls (buffers, uploaded
   volume and tuned launch shape are reused), and so do given-back output
   buffers; 0: every call releases them */
static int g_keep_sessions = 1;
static pthread_mutex_t g_outcache_lock = PTHREAD_MUTEX_INITIALIZER;
static void* g_outcache[OUTCACHE_N];
static size_t g_outcache_size[OUTCACHE_N];

/* n bytes for an output the run writes in full: the smallest cached buffer
   that holds n and wastes at most n + 1 MB, else a new one */
static void* outbuf_alloc(size_t n) {
    void* p = NULL;
    int pick = -1;
    pthread_mutex_lock(&g_outcache_lock);
    for (int i = 0; i < OUTCACHE_N; i++) {
        if (g_outcache[i] && g_outcache_size[i] >= n && g_outcache_size[i] <= 2 * n + ((size_t)1 << 20) &&
                (pick < 0 || g_outcache_size[i] < g_outcache_size[pick])) {
            pick = i;
        }
    }
    if (pick >= 0) {
        p = g_outcache[pick];
        g_outcache[pick] = NULL;
        g_outcache_size[pick] = 0;
    }
    pthread_mutex_unlock(&g_outcache_lock);
    return p ? p : malloc(n ? n : 1);
}

static void outcache_release(void) {
    pthread_mutex_lock(&g_outcache_lock);
    for (int i = 0; i < OUTCACHE_N; i++) {
        free(g_outcache[i]);
        g_outcache[i] = NULL;
        g_outcache_size[i] = 0;
    }
    pthread_mutex_unlock(&g_outcache_lock);
}

void mcx_free_buffer(void* p) {
    if (!p) {
        return;
    }
    const size_t n = malloc_usable_size(p);
    if (g_keep_sessions && n >= ((size_t)1 << 20)) {
        pthread_mutex_lock(&g_outcache_lock);
        size_t held = 0;
        int slot = -1;
        for (int i = 0; i < OUTCACHE_N; i++) {
            held += g_outcache_size[i];
            if (!g_outcache[i] && slot < 0) {
                slot = i;
            }
        }
        if (slot >= 0 && held + n <= ((size_t)1 << 30)) {
            g_outcache[slot] = p;
            g_outcache_size[slot] = n;
            p = NULL;
        }
        pthread_mutex_unlock(&g_outcache_lock);
    }
    free(p);
}

void mcx_cleargpuinfo(GPUInfo** info) {
    if (info && *info) {
        free(*info);
        *info = NULL;
    }
}

/* one cached device session per GPU; buffers are reused across calls */
static mcxg_session* g_sessions[MAX_DEVICE];

static mcxg_session* session_for(int device) {
    if (device < 0 || device >= MAX_DEVICE) {
        return NULL;
    }
    if (!g_sessions[device]) {
        if (mcxg_create(device, &g_sessions[device]) != MCXG_OK) {
            g_sessions[device] = NULL;
        }
    }
    return g_sessions[device];
}

/* launch shape picked by the autotuner, per device, for the last problem shape tuned */
typedef struct {
    int valid;
    uint64_t sig;
    int block, bpsm, noagg;
} TuneCache;
static TuneCache g_tune[MAX_DEVICE];

static uint64_t mix64(uint64_t h, uint64_t v) {
    h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    return h;
}

/* what the launch shape depends on: the volume, the media, the source, the
   outputs compiled in and the photon budget per thread */
static uint64_t tune_signature(const Config* cfg, const mcxg_kparams* kp) {
    uint64_t h = 1469598103934665603ull;
    h = mix64(h, kp->nvox);
    h = mix64(h, kp->dimx);
    h = mix64(h, kp->fieldlen);
    h = mix64(h, (uint64_t)kp->medianum << 32 | (uint32_t)kp->srctype);
    h = mix64(h, (uint64_t)kp->savedet << 8 | (uint64_t)kp->dorefl_compiled << 4 | (uint64_t)kp->issaveref);
    h = mix64(h, kp->nthread);
    h = mix64(h, (uint64_t)(cfg->nphoton / 1000));
    h = mix64(h, (uint64_t)cfg->dim.y << 32 | cfg->dim.z);
    for (unsigned int i = 0; i < cfg->medianum && i < 16; i++) {
        uint32_t w[4];
        memcpy(w, &cfg->prop[i], sizeof(w));
        h = mix64(h, (uint64_t)w[0] << 32 | w[1]);
        h = mix64(h, (uint64_t)w[2] << 32 | w[3]);
    }
    return h;
}

/* The cached sessions are shared by every host thread of the process: the
   public entry points that use or release them hold this lock, so calls from
   several threads run one after another instead of sharing device buffers. */
static pthread_mutex_t g_run_lock = PTHREAD_MUTEX_INITIALIZER;

/* the device layer switches the thread's current CUDA device to the one it
   runs on; the public calls put the caller's back (mcx_device.cu) */
int mcxg_internal_current_device(void);
void mcxg_internal_restore_device(int d);

static void release_sessions(void) {
    for (int i = 0; i < MAX_DEVICE; i++) {
        if (g_sessions[i]) {
            mcxg_destroy(g_sessions[i]);
            g_sessions[i] = NULL;
        }
    }
    outcache_release();
}

void mcx_release_sessions(void) {
    pthread_mutex_lock(&g_run_lock);
    release_sessions();
    pthread_mutex_unlock(&g_run_lock);
}

static void device_check(int rc, const char* what) {
    if (rc != MCXG_OK) {
        char msg[256];
        snprintf(msg, sizeof(msg), "%s failed: %s", what, mcxg_error_string(rc));
        MCX_ERROR(-(100 + rc), msg);
    }
}

/* the kernel constant block of one simulation (mcx_host.cpp:507-524, 674-693) */
/* The words rand() returns after srand(seed) in the C library the reference
   runs on (glibc's default generator): an additive lagged-Fibonacci
   generator x[n] = x[n-3] + x[n-31] (mod 2^32) whose 31 words of state come
   from the Park-Miller minimal standard generator (16807 x mod 2^31 - 1, in
   Schrage's factorisation), the first 310 outputs discarded and each output
   x >> 1.  Restated here because the library's rand() takes a lock on every
   call and the reference draws four words per reference thread. */
typedef struct AddRand {
    uint32_t x[31];
    int f, b;                      /* the x[n-3] and x[n-31] taps into the ring */
} AddRand;

static inline uint32_t addrand_next(AddRand* g) {
    const uint32_t v = (g->x[g->f] += g->x[g->b]);
    g->f = (g->f == 30) ? 0 : g->f + 1;
    g->b = (g->b == 30) ? 0 : g->b + 1;
    return v >> 1;
}

static void addrand_seed(AddRand* g, unsigned int seed) {
    int32_t w = (int32_t)(seed ? seed : 1u);
    g->x[0] = (uint32_t)w;
    for (int i = 1; i < 31; i++) {
        const int64_t hi = w / 127773, lo = w % 127773;
        w = (int32_t)(16807 * lo - 2836 * hi);
        if (w < 0) {
            w += 2147483647;
        }
        g->x[i] = (uint32_t)w;
    }
    g->f = 3;
    g->b = 0;
    for (int i = 0; i < 310; i++) {
        (void)addrand_next(g);
    }
}

static void addrand_fill(AddRand* g, uint32_t* out, size_t n) {
    for (size_t i = 0; i < n; i++) {
        out[i] = addrand_next(g);
    }
}

void mcx_rand_words(unsigned int seed, uint32_t* out, size_t n) {
    AddRand g;
    addrand_seed(&g, seed);
    addrand_fill(&g, out, n);
}

/* Jump-ahead.  The generator is linear over the integers mod 2^32: with the
   window W = (o[k-31], ..., o[k-1]) of its unshifted outputs, one step is
   W' = M W with W'[t] = W[t+1] (t < 30) and W'[30] = W[0] + W[28] (o[k] =
   o[k-31] + o[k-3]; the ring slot f holds o[k-31], b = f - 3 holds o[k-3]), so n steps
   are M^n W, M^n by repeated squaring (31 x 31 matrices of words, products
   wrapping mod 2^32 as the generator's sums do). */
#define LF_N 31

static void lf_matmul(const uint32_t* A, const uint32_t* B, uint32_t* C) {
    uint32_t T[LF_N * LF_N];
    for (int i = 0; i < LF_N; i++) {
        uint32_t row[LF_N] = {0};
        for (int k = 0; k < LF_N; k++) {
            const uint32_t a = A[i * LF_N + k];
            for (int j = 0; j < LF_N; j++) {
                row[j] += a * B[k * LF_N + j];
            }
        }
        memcpy(T + i * LF_N, row, sizeof(row));
    }
    memcpy(C, T, sizeof(T));
}

static void lf_matvec(const uint32_t* A, const uint32_t* w, uint32_t* out) {
    uint32_t r[LF_N];
    for (int i = 0; i < LF_N; i++) {
        uint32_t acc = 0;
        for (int k = 0; k < LF_N; k++) {
            acc += A[i * LF_N + k] * w[k];
        }
        r[i] = acc;
    }
    memcpy(out, r, sizeof(r));
}

/* P = M^e */
static void lf_pow(uint64_t e, uint32_t* P) {
    uint32_t B[LF_N * LF_N] = {0};
    memset(P, 0, sizeof(uint32_t) * LF_N * LF_N);
    for (int i = 0; i < LF_N; i++) {
        P[i * LF_N + i] = 1u;
    }
    for (int t = 0; t < LF_N - 1; t++) {
        B[t * LF_N + t + 1] = 1u;
    }
    B[(LF_N - 1) * LF_N + 0] = 1u;
    B[(LF_N - 1) * LF_N + 28] = 1u;
    while (e) {
        if (e & 1u) {
            lf_matmul(P, B, P);
        }
        e >>= 1;
        if (e) {
            lf_matmul(B, B, B);
        }
    }
}

static void addrand_window(const AddRand* g, uint32_t* W) {
    for (int t = 0; t < LF_N; t++) {
        W[t] = g->x[(g->f + t) % LF_N];
    }
}

static void addrand_set_window(AddRand* g, const uint32_t* W) {
    memcpy(g->x, W, sizeof(uint32_t) * LF_N);
    g->f = 0;
    g->b = 28;
}

/* g moved on by nword words */
static void addrand_skip(AddRand* g, uint64_t nword) {
    uint32_t P[LF_N * LF_N], W[LF_N];
    addrand_window(g, W);
    lf_pow(nword, P);
    lf_matvec(P, W, W);
    addrand_set_window(g, W);
}

/* the windows at g's position + j x blocklen (j < nblock) into starts, and g
   moved on by nword words */
static void addrand_blocks(AddRand* g, uint64_t nword, uint32_t nblock, uint32_t blocklen, uint32_t* starts) {
    uint32_t P[LF_N * LF_N], W[LF_N];
    addrand_window(g, W);
    lf_pow(blocklen, P);
    for (uint32_t j = 0; j < nblock; j++) {
        memcpy(starts + (size_t)LF_N * j, W, sizeof(W));
        if (j + 1 < nblock) {
            lf_matvec(P, W, W);
        }
    }
    addrand_skip(g, nword);
}

/* Label bytes to the Config's uint32 words, x fastest.  A C-ordered volume
   ([x][y][z] in memory, numpy's default) is transposed per y slice in 32 x 32
   tiles of (z, x): each tile reads 32 rows of 32 bytes and writes 32 runs of
   32 words, all cache-resident (one x86 core: a cube of 128 in 3.2 ms and
   the 181 x 217 x 181 head in 15 ms, against 9 and 27 ms for numpy's strided
   pass). */
void mcx_labels_u8(const uint8_t* vol, uint32_t nx, uint32_t ny, uint32_t nz, int c_order, uint32_t* out) {
    const size_t nxy = (size_t)nx * ny, nyz = (size_t)ny * nz;
    if (!c_order) {
        const size_t n = nxy * nz;
        for (size_t i = 0; i < n; i++) {
            out[i] = vol[i];
        }
        return;
    }
    for (uint32_t y = 0; y < ny; y++) {
        for (uint32_t z0 = 0; z0 < nz; z0 += 32) {
            const uint32_t z1 = z0 + 32 < nz ? z0 + 32 : nz;
            for (uint32_t x0 = 0; x0 < nx; x0 += 32) {
                const uint32_t x1 = x0 + 32 < nx ? x0 + 32 : nx;
                for (uint32_t z = z0; z < z1; z++) {
                    uint32_t* o = out + (size_t)z * nxy + (size_t)y * nx;
                    const uint8_t* in = vol + (size_t)y * nz + z;
                    for (uint32_t x = x0; x < x1; x++) {
                        o[x] = in[(size_t)x * nyz];
                    }
                }
            }
        }
    }
}

int mcx_rand_blocks(unsigned int seed, uint64_t skip, uint32_t nblock, uint32_t blocklen, uint32_t* starts) {
    if (!starts || nblock == 0 || blocklen == 0) {
        return -1;
    }
    AddRand g;
    addrand_seed(&g, seed);
    if (skip) {
        addrand_skip(&g, skip);
    }
    addrand_blocks(&g, 0, nblock, blocklen, starts);
    return 0;
}

/* The field accumulator's fixed-point unit 2^-S (the transport kernel's
   deposits split into int64 counts of 2^-S and float remainders): the
   largest S, at most 40, for which no element can reach 2^61 counts.  An
   element gathers at most every photon's whole path -- the time window at
   the speed of light, in voxels -- times its weight (a replay: the largest
   replay weight), with a factor 4 to spare. */
static void field_scale(const Config* cfg, int replay, float* sc, float* unit) {
    const double twin1 = (double)cfg->tstart + (double)cfg->tstep * cfg->maxgate;
    double path = twin1 * 2.99792458e11 / (cfg->unitinmm > 0.f ? cfg->unitinmm : 1.f);
    path = path > 1.0 ? path : 1.0;
    double wmax = 1.0;
    if (replay && cfg->replay.weight) {
        for (size_t i = 0; i < cfg->nphoton; i++) {
            const double w = fabs((double)cfg->replay.weight[i]);
            wmax = w > wmax ? w : wmax;
        }
    }
    const double bound = 4.0 * (double)(cfg->nphoton ? cfg->nphoton : 1) * path * wmax;
    int S = (int)floor(61.0 - log2(bound));
    S = S < 0 ? 0 : (S > 40 ? 40 : S);
    *sc = ldexpf(1.f, S);
    *unit = ldexpf(1.f, -S);
}

static void make_kparams(const Config* cfg, size_t nvox, size_t fieldlen, size_t autothread, unsigned int hostdetreclen,
                         unsigned int partialdata, unsigned int is2d, int replay, mcxg_kparams* kp) {
    memset(kp, 0, sizeof(*kp));
    kp->srcpos = (mcxg_float4) {cfg->srcpos.x, cfg->srcpos.y, cfg->srcpos.z, cfg->srcpos.w};
    kp->srcdir = (mcxg_float4) {cfg->srcdir.x, cfg->srcdir.y, cfg->srcdir.z, cfg->srcdir.w};
    kp->srcparam1 = (mcxg_float4) {cfg->srcparam1.x, cfg->srcparam1.y, cfg->srcparam1.z, cfg->srcparam1.w};
    kp->srcparam2 = (mcxg_float4) {cfg->srcparam2.x, cfg->srcparam2.y, cfg->srcparam2.z, cfg->srcparam2.w};
    kp->maxidx = (mcxg_float4) {(float)cfg->dim.x, (float)cfg->dim.y, (float)cfg->dim.z, 0.f};
    kp->dimx = cfg->dim.x;
    kp->dimy = cfg->dim.y;
    kp->dimz = cfg->dim.z;
    kp->dimxy = cfg->dim.x * cfg->dim.y;
    kp->nvox = (uint32_t)nvox;
    kp->fieldlen = (uint32_t)fieldlen;
    kp->twin0 = cfg->tstart;
    kp->twin1 = cfg->tstart + cfg->tstep * cfg->maxgate;
    field_scale(cfg, replay, &kp->fxscale, &kp->fxunit);
    float minstep = fminf(fminf(cfg->steps.x, cfg->steps.y), cfg->steps.z);
    kp->oneoverc0 = R_C0 * cfg->unitinmm;
    kp->Rtstep = 1.f / cfg->tstep;
    kp->minenergy = cfg->minenergy;
    kp->minaccumtime = minstep * R_C0 * cfg->unitinmm;
    kp->doreflect = (uint32_t)cfg->isreflect;
    {
        const char allabsorb[6] = {bcAbsorb, bcAbsorb, bcAbsorb, bcAbsorb, bcAbsorb, bcAbsorb};
        const char allunknown[6] = {0, 0, 0, 0, 0, 0};
        int refl = cfg->isreflect || (memcmp(cfg->bc, allabsorb, 6) && memcmp(cfg->bc, allunknown, 6));
        for (int i = 0; i < 6; i++) {
            if (cfg->bc[i] == bcReflect || cfg->bc[i] == bcMirror) {
                refl = 1;
            }
        }
        kp->dorefl_compiled = (uint32_t)refl;
    }
    kp->save2pt = cfg->issave2pt ? 1 : 0;
    kp->savedet = (uint32_t)cfg->issavedet;
    kp->maxdetphoton = cfg->maxdetphoton;
    kp->maxmedia = cfg->medianum - 1;
    kp->medianum = cfg->medianum;
    kp->detnum = cfg->detnum;
    kp->voidtime = (uint32_t)cfg->voidtime;
    kp->srctype = (uint32_t)cfg->srctype;
    kp->maxvoidstep = (uint32_t)cfg->maxvoidstep;
    kp->issaveseed = cfg->issaveseed > 0;
    kp->issaveref = (uint32_t)cfg->issaveref;
    kp->isspecular = cfg->isspecular > 0;
    kp->maxgate = cfg->maxgate;
    kp->outputtype = (uint32_t)cfg->outputtype;
    kp->savedetflag = cfg->savedetflag;
    kp->reclen = hostdetreclen;
    kp->partialdata = partialdata;
    kp->mediaformat = cfg->mediabyte;
    kp->gscatter = cfg->gscatter;
    kp->is2d = is2d;
    kp->nphase = cfg->nphase;
    kp->nangle = cfg->nangle;
    kp->extrasrclen = cfg->extrasrclen;
    kp->srcid = cfg->srcid;
    kp->srcnum = (cfg->srcnum > 1 && (cfg->srctype == MCX_SRC_PATTERN || cfg->srctype == MCX_SRC_PATTERN3D))
                 ? cfg->srcnum : 1u;
    kp->omega = cfg->omega;
    kp->nthread = (uint32_t)autothread;
    if (replay) {
        kp->replay = 1;
        kp->nreplay = (uint32_t)cfg->nphoton;
        kp->replaydet = cfg->replaydet;
        kp->siteshift = cfg->replaysiteown ? 0u : 1u;
    }
    for (int i = 0; i < 12; i++) {
        kp->bc[i] = (uint8_t)cfg->bc[i];
    }
}

/* Adjoint Jacobians from the normalised forward fluences of the sources and
   of the detectors run as sources (mcx_host.cpp:1466-1642): phi_src phi_det
   (mua) and/or grad phi_src . grad phi_det (diffusion coefficient), scaled
   by -Vvox and -unitinmm, and for the mus / mus' types by the medium's
   1 / (3 (1-g) mus^2) or 1 / (3 (1-g)^2 mus^2). */
static void adjoint_jacobians(Config* cfg, mcxg_session* s, size_t nvox) {
    const int isdual = MCX_IS_DUAL_ADJOINT_TYPE(cfg->outputtype);
    const unsigned int Ns = cfg->extrasrclen + 1 - cfg->detnum, Nd = cfg->detnum;
    const size_t adjlen = nvox * Ns * Nd;
    const float Vvox = cfg->steps.x * cfg->steps.y * cfg->steps.z;
    free(cfg->exportjacob);
    cfg->exportjacob = (float*)malloc(sizeof(float) * adjlen * (isdual ? 2 : 1));
    if (!cfg->exportjacob) {
        MCX_ERROR(-2, "out of host memory");
    }
    float* first = cfg->exportjacob;
    float* second = isdual ? cfg->exportjacob + adjlen : cfg->exportjacob;
    if (isdual || cfg->outputtype == otAdjoint) {
        device_check(mcxg_adjoint(s, 0, Ns, Nd, cfg->dim.x, cfg->dim.y, cfg->dim.z, cfg->maxgate, first),
                     "computing the adjoint mua Jacobian");
    }
    if (isdual || cfg->outputtype != otAdjoint) {
        device_check(mcxg_adjoint(s, 1, Ns, Nd, cfg->dim.x, cfg->dim.y, cfg->dim.z, cfg->maxgate, second),
                     "computing the adjoint diffusion Jacobian");
    }
    if (isdual) {
        for (size_t k = 0; k < adjlen; k++) {
            first[k] *= -Vvox;
        }
        for (size_t k = 0; k < adjlen; k++) {
            second[k] *= -cfg->unitinmm;
        }
    } else {
        const float adj_scale = (cfg->outputtype == otAdjoint) ? -Vvox : -cfg->unitinmm;
        for (size_t k = 0; k < adjlen; k++) {
            first[k] *= adj_scale;
        }
    }
    const int musform = (cfg->outputtype == otAdjointMus) ? 1 :
                        ((cfg->outputtype == otAdjointMusp || cfg->outputtype == otAdjointMuaMusp) ? 2 : 0);
    if (musform) {
        for (size_t vox = 0; vox < nvox; vox++) {
            unsigned int medid = cfg->vol[vox] & 0xFF;
            float opscale = 0.f;
            if (medid < cfg->medianum) {
                float mus = cfg->prop[medid].mus;
                float onemg = 1.f - cfg->prop[medid].g;
                if (mus > 0.f && onemg > 0.f) {
                    opscale = (musform == 1) ? 1.f / (3.f * onemg * mus * mus) : 1.f / (3.f * onemg * onemg * mus * mus);
                }
            }
            for (unsigned int sd = 0; sd < Ns * Nd; sd++) {
                second[vox + (size_t)sd * nvox] *= opscale;
            }
        }
    }
}

/* --------------------------------------------------------------- the driver */

/* set by mcx_prepare_simulation: stop once the problem and the first seeds are resident */
static __thread int prepare_only = 0;
static __thread mcxg_session* prepared_session = NULL;

static void run_simulation(Config* cfg) {
    GPUInfo* gpu = NULL;
    /* temporaries live in thread-local slots so the library-mode error path
       (longjmp back to this frame) can free them */
    static __thread void* tmp[6];
    for (int i = 0; i < 6; i++) {
        free(tmp[i]);
        tmp[i] = NULL;
    }
#define fieldtmp (*(float**)&tmp[4])
#define blockscale (*(double**)&tmp[5])
    MCX_ENTER(cfg);

    unsigned int partialdata = (cfg->medianum - 1) *
                               (SAVE_NSCAT(cfg->savedetflag) + SAVE_PPATH(cfg->savedetflag) + SAVE_MOM(cfg->savedetflag));
    unsigned int hostdetreclen = mcx_detreclen(cfg);
    unsigned int is2d = (cfg->dim.x == 1 ? 1 : (cfg->dim.y == 1 ? 2 : (cfg->dim.z == 1 ? 3 : 0)));
    if (is2d) {
        is2d = is2d * (((cfg->dim.x > 1) + (cfg->dim.y > 1) + (cfg->dim.z > 1)) == 2);
    }
    unsigned int workdev = 0;
    mcx_list_gpu(cfg, &workdev, &gpu);
    if (workdev == 0) {
        free(gpu);
        MCX_ERROR(-99, "Specified GPU does not exist");
    }
    /* one GPU per call: the first selected device runs every photon */
    GPUInfo g = gpu[0];
    free(gpu);
    gpu = NULL;
    int device = g.id - 1;

    size_t autothread, autoblock;
    if (cfg->autopilot) {
        /* the reference's NVIDIA compute >= 6 choice (mcx_host.cpp:617-620),
           which the exact kernel keeps.  The fast kernel's persistent grid
           ends when its slowest reference thread does, so it takes up to 32
           times as many threads, down to 2 photons each: shorter threads
           shorten the end of the launch (cube + sphere at 1e8 photons: +10 %
           with 8 times the threads, +1.3 % more with 32; at 1e7 photons, 2
           photons a thread instead of 16: +17 %) */
        autoblock = 64;
        autothread = autoblock * 64 * (size_t)g.sm;
        if (!cfg->exactmath && !(cfg->debuglevel & 1)) {
            const size_t per = (size_t)(cfg->nphoton / (cfg->respin > 0 ? cfg->respin : 1)) / 2;
            const size_t cap = 32 * autothread;
            autothread = per > cap ? cap : (per > autothread ? per : autothread);
        }
    } else {
        autothread = cfg->nthread;
        autoblock = cfg->nblocksize ? cfg->nblocksize : 64;
    }
    if (autothread % autoblock) {
        autothread = (autothread / autoblock) * autoblock;
    }
    if (autothread == 0) {
        MCX_ERROR(-1, "thread number must be at least the block size");
    }
    if (is2d) {
        float* vec = &(cfg->srcdir.x);
        if (fabsf(vec[is2d - 1]) > H_EPS) {
            MCX_ERROR(-1, "input domain is 2D, the initial direction can not have non-zero value in the singular dimension");
        }
    }
    cfg->maxgate = (unsigned int)(int)((cfg->tend - cfg->tstart) / cfg->tstep + 0.5);
    size_t nvox = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
    size_t mult = (cfg->extrasrclen && cfg->srcid < 0) ? (cfg->extrasrclen + 1) : 1;
    /* photon sharing: one field per pattern, interleaved innermost
       (mcx_host.cpp:474, 679) */
    const unsigned int nshare = (cfg->srcnum > 1 && (cfg->srctype == MCX_SRC_PATTERN || cfg->srctype == MCX_SRC_PATTERN3D))
                                ? cfg->srcnum : 1u;
    mult *= nshare;
    const int replay = (cfg->seed == SEED_FROM_FILE);
    if (replay && cfg->replaydet == -1) {
        mult *= cfg->detnum;    /* one block of gates per detector (mcx_host.cpp:684-687) */
    }
    if (replay && cfg->nphoton && (!cfg->replay.seed || !cfg->replay.weight || !cfg->replay.tof || !cfg->replay.detid)) {
        MCX_ERROR(-6, "replay inputs are missing: call mcx_validatecfg with the baseline records first");
    }
    size_t fieldlen = nvox * cfg->maxgate * mult;
    /* the kernel forms index + gate x nvox in 32 bits, one gate past the end
       included (a time of flight a rounding below the window's end) */
    if (fieldlen + nvox > 0xFFFFFFFFull || nvox > 0x7FFFFFFFull) {
        MCX_ERROR(-1, "volume x gates too large for 32-bit field indices");
    }

    float fullload = 0.f;
    for (unsigned int i = 0; i < workdev && i < MAX_DEVICE; i++) {
        fullload += cfg->workload[i];
    }
    float workload0 = cfg->workload[0];
    if (fullload < H_EPS) {
        workload0 = (float)g.core;
        fullload = (float)g.core;
    }

    mcxg_kparams kp;
    make_kparams(cfg, nvox, fieldlen, autothread, hostdetreclen, partialdata, is2d, replay, &kp);

    /* the label volume: one byte per voxel (label | detector bit << 7) when
       every label fits in seven bits -- the 32-bit words go up and the device
       packs them -- else the reference's 32-bit words */
    const uint32_t mediaword = (cfg->mediabyte <= 4 && cfg->medianum <= 128) ? MCXG_MEDIA_PACK : 4u;

    mcxg_session* s = session_for(device);
    if (!s) {
        MCX_ERROR(-99, "failed to open a CUDA session on the selected GPU");
    }
    int rc = mcxg_set_problem(s, &kp, sizeof(kp), (const void*)cfg->vol, mediaword,
                              (const float*)cfg->prop, (const float*)cfg->detpos, (const float*)cfg->srcdata,
                              cfg->invcdf, cfg->angleinvcdf, cfg->srcpattern,
                              cfg->srctype == MCX_SRC_PATTERN ? (size_t)((int)(cfg->srcparam1.w * cfg->srcparam2.w) * cfg->srcnum)
                              : (cfg->srctype == MCX_SRC_PATTERN3D ?
                                 (size_t)((int)(cfg->srcparam1.x * cfg->srcparam1.y * cfg->srcparam1.z) * cfg->srcnum) : 0));
    device_check(rc, "uploading the problem");
    device_check(mcxg_set_replay(s, cfg->replay.seed, cfg->replay.weight, cfg->replay.tof, cfg->replay.detid,
                                 replay ? (uint32_t)cfg->nphoton : 0u), "uploading the replay inputs");
    device_check(mcxg_set_polarization(s, (const float*)cfg->smatrix, (cfg->polprop && cfg->smatrix) ? cfg->polmedianum : 0u,
                                       &cfg->srciquv.x), "uploading the Mueller tables");

    /* seeds: srand(seed) then 4 rand() words per reference thread
       (mcx_host.cpp:696-700, 759-768); a replay launches every photon from its
       saved state, so its per-thread words are never drawn from */
    AddRand ar;
    addrand_seed(&ar, cfg->seed > 0 ? (unsigned int)cfg->seed : (replay ? 1u : (unsigned int)time(0)));
    cfg->detectedcount = 0;
    cfg->his.detected = 0;
    free(cfg->exportdebugdata);
    cfg->exportdebugdata = NULL;
    cfg->debugdatalen = 0;
    cfg->his.respin = cfg->respin;
    cfg->his.colcount = hostdetreclen;
    cfg->energytot = 0.0;
    cfg->energyesc = 0.0;
    cfg->runtime = 0;
    cfg->kernelms = 0.f;
    cfg->failedlaunch = 0;
    memset(cfg->eventcount, 0, sizeof(cfg->eventcount));

    float kms_total = 0.f;
    for (int iter = 0; iter < cfg->respin; iter++) {
        /* the words are generated on the device from the generator's window
           at this repetition's first word: the device jumps each block of
           words ahead from it; the host moves on only for a next repetition */
        const uint64_t nword = 4ull * autothread;
        uint32_t window[LF_N];
        addrand_window(&ar, window);
        device_check(mcxg_set_seeds_window(s, window, (uint32_t)autothread), "generating seeds");
        if (iter + 1 < cfg->respin) {
            addrand_skip(&ar, nword);
        }
        /* photon split in the reference's float arithmetic (mcx_host.cpp:1101-1102) */
        float tp = (float)cfg->nphoton * workload0 / (fullload * (float)autothread * (float)cfg->respin);
        kp.threadphoton = (uint32_t)(int)tp;
        kp.oddphoton = (int)((float)cfg->nphoton * workload0 / (fullload * (float)cfg->respin) -
                             (float)((size_t)kp.threadphoton * autothread));
        device_check(mcxg_set_params(s, &kp, sizeof(kp)), "updating parameters");
        if (prepare_only) {
            /* mcx_prepare_simulation: everything is resident, nothing has run */
            prepared_session = s;
            cfg->threadused = (unsigned int)autothread;
            break;
        }
        unsigned int flags = (cfg->exactmath ? MCXG_EXACT : 0u) | (iter ? MCXG_KEEP : 0u) |
                             ((cfg->debuglevel & 1) ? MCXG_RNGDUMP : 0u);
        if (iter == 0) {
            device_check(mcxg_set_launch(s, 0, 0), "resetting the launch shape");
            /* MCX_DEBUG_MOVE (2) and MCX_DEBUG_MOVE_ONLY (8) both record (mcx_host.cpp:702, 1173);
               set before any launch so a cached session never keeps the last run's setting */
            device_check(mcxg_set_trajectory(s, (cfg->debuglevel & 10) ? cfg->maxjumpdebug : 0u),
                         "allocating the trajectory records");
        }
        /* trajectory runs take the general instantiation and record at every
           launch: they are not tuned (the tuned shape is for the common one) */
        if (cfg->autotune && !cfg->exactmath && !(cfg->debuglevel & 11)) {
            uint64_t sig = tune_signature(cfg, &kp);
            TuneCache* tc = &g_tune[device];
            if (!tc->valid || tc->sig != sig) {
                /* 1/64 of the photons per candidate, at most 2e6 and at least 2e5 */
                double want = cfg->nphoton / 64.0;
                uint32_t sample = (uint32_t)(want > 2e6 ? 2e6 : (want < 2e5 ? 2e5 : want));
                int blk = 0, bpsm = 0, noagg = 1;
                device_check(mcxg_autotune(s, sample, &blk, &bpsm, &noagg), "autotuning the launch shape");
                tc->valid = 1;
                tc->sig = sig;
                tc->block = blk;
                tc->bpsm = bpsm;
                tc->noagg = noagg;
            }
            device_check(mcxg_set_launch(s, tc->block, tc->bpsm), "setting the launch shape");
            flags |= tc->noagg ? MCXG_NOAGG : MCXG_AGG;
        }
        float kms = 0.f;
        device_check(mcxg_simulate(s, flags, &kms), "running the transport kernel");
        kms_total += kms;
        if ((cfg->debuglevel & 10) && cfg->maxjumpdebug) {
            /* append this repetition's records (mcx_host.cpp:1175-1192) */
            uint32_t made = 0;
            device_check(mcxg_get_trajectory(s, NULL, 0, &made), "reading the trajectory count");
            const uint32_t take = made < cfg->maxjumpdebug ? made : cfg->maxjumpdebug;
            if (made > cfg->maxjumpdebug) {
                fprintf(stderr, "WARNING: the saved trajectory positions (%u) are more than maxjumpdebug (%u)\n",
                            made, cfg->maxjumpdebug);
            }
            float* grown = (float*)realloc(cfg->exportdebugdata, sizeof(float) * 6 * ((size_t)cfg->debugdatalen + take + 1));
            if (!grown) {
                MCX_ERROR(-2, "out of host memory");
            }
            cfg->exportdebugdata = grown;
            if (take) {
                device_check(mcxg_get_trajectory(s, grown + (size_t)6 * cfg->debugdatalen, take, &made),
                             "reading the trajectory records");
            }
            cfg->debugdatalen += take;
        }

        double esc = 0.0, tot = 0.0;
        device_check(mcxg_get_energy(s, &esc, &tot), "reducing energies");
        if (cfg->savethreadenergy && iter == 0) {
            free(cfg->exportenergy);
            cfg->exportenergy = (float*)malloc(sizeof(float) * 2 * autothread);
            if (!cfg->exportenergy) {
                MCX_ERROR(-2, "out of host memory");
            }
            device_check(mcxg_get_thread_energy(s, cfg->exportenergy), "reading per-thread energies");
        }
        cfg->energyesc += esc;
        cfg->energytot += tot;
        uint64_t ev[5];
        uint32_t stw[2];
        device_check(mcxg_get_counters(s, ev, stw), "reading counters");
        for (int k = 0; k < 5; k++) {
            cfg->eventcount[k] += ev[k];
        }
        cfg->failedlaunch += stw[0];

        if (cfg->issavedet) {
            /* the count first, then this repetition's records straight into the
               grown export buffers */
            uint32_t detected = 0;
            device_check(mcxg_get_detected(s, NULL, NULL, &detected), "reading the detected photon count");
            if (detected > cfg->maxdetphoton && cfg->flog) {
                fprintf(cfg->flog, "WARNING: the detected photon number is more than what your have specified (%u > %u), "
                        "please use the -H option to specify a greater number\t", detected, cfg->maxdetphoton);
            }
            cfg->his.detected += detected;
            uint32_t saved = detected < cfg->maxdetphoton ? detected : cfg->maxdetphoton;
            if (saved) {
                const size_t dbytes = sizeof(float) * ((size_t)cfg->detectedcount + saved) * (hostdetreclen ? hostdetreclen : 1);
                float* nd = cfg->exportdetected ? (float*)realloc(cfg->exportdetected, dbytes) : (float*)outbuf_alloc(dbytes);
                if (!nd) {
                    MCX_ERROR(-2, "out of host memory");
                }
                cfg->exportdetected = nd;
                uint64_t* sd = NULL;
                if (cfg->issaveseed) {
                    const size_t sbytes = sizeof(uint64_t) * 2 * ((size_t)cfg->detectedcount + saved);
                    void* ns = cfg->seeddata ? realloc(cfg->seeddata, sbytes) : outbuf_alloc(sbytes);
                    if (!ns) {
                        MCX_ERROR(-2, "out of host memory");
                    }
                    cfg->seeddata = ns;
                    sd = (uint64_t*)cfg->seeddata + (size_t)cfg->detectedcount * 2;
                }
                device_check(mcxg_get_detected(s, cfg->exportdetected + (size_t)cfg->detectedcount * hostdetreclen, sd,
                                               &detected), "reading detected photons");
                if (cfg->savedetweight) {
                    float* nw = (float*)realloc(cfg->exportdetweight, sizeof(float) * 2 * ((size_t)cfg->detectedcount + saved));
                    if (!nw) {
                        MCX_ERROR(-2, "out of host memory");
                    }
                    cfg->exportdetweight = nw;
                    device_check(mcxg_get_detweight(s, cfg->exportdetweight + (size_t)cfg->detectedcount * 2),
                                 "reading detected weights");
                }
                cfg->detectedcount += saved;
            }
        }
    }
    if (prepare_only) {
        for (int i = 0; i < 6; i++) {
            free(tmp[i]);
            tmp[i] = NULL;
        }
        MCX_LEAVE();
        return;
    }
    cfg->kernelms = kms_total;
    cfg->threadused = (unsigned int)autothread;
    cfg->runtime = (unsigned int)(kms_total + 0.5f);

    /* normalisation (mcx_host.cpp:1382-1465), applied in FP64 on the GPU; a
       replay with one output per detector scales each detector's block by its
       own replayed weight (1398-1419) */
    double scale = 1.0;
    uint32_t nblocks = 1;
    if (cfg->issave2pt) {
        int replayout = cfg->outputtype == otJacobian || cfg->outputtype == otWP || cfg->outputtype == otDCS ||
                        cfg->outputtype == otRF || cfg->outputtype == otRFmus ||
                        cfg->outputtype == otWLTOF || cfg->outputtype == otWPTOF;
        if (cfg->isnormalized) {
            float Vvox = cfg->steps.x * cfg->steps.y * cfg->steps.z;
            float sc = 1.f;
            cfg->energyabs += cfg->energytot - cfg->energyesc;
            if (cfg->outputtype == otFlux || cfg->outputtype == otFluence || MCX_IS_ADJOINT_TYPE(cfg->outputtype) ||
                    (cfg->omega > 0.f && !replay)) {
                sc = (float)(cfg->unitinmm / (cfg->energytot * Vvox * cfg->tstep));
                if (cfg->outputtype == otFluence || MCX_IS_ADJOINT_TYPE(cfg->outputtype)) {
                    sc *= cfg->tstep;
                }
            } else if (cfg->outputtype == otEnergy || cfg->outputtype == otL) {
                sc = (float)(1.0 / cfg->energytot);
            } else if (replayout) {
                if (replay && cfg->replaydet == -1) {
                    nblocks = cfg->detnum * (uint32_t)mult / cfg->detnum;
                    blockscale = (double*)calloc(nblocks, sizeof(double));
                    if (!blockscale) {
                        MCX_ERROR(-2, "out of host memory");
                    }
                    for (uint32_t d = 0; d < cfg->detnum; d++) {
                        float w = 0.f;
                        for (size_t i = 0; i < cfg->nphoton; i++) {
                            if ((cfg->replay.detid[i] & 0xFFFF) == (int)d + 1) {
                                w += cfg->replay.weight[i];
                            }
                        }
                        if (w > 0.f) {
                            w = cfg->unitinmm / w;
                        }
                        for (uint32_t b = d; b < nblocks; b += cfg->detnum) {
                            blockscale[b] = (double)w;
                        }
                        sc = w;    /* the reference leaves the last detector's factor as the normaliser */
                    }
                } else {
                    sc = 0.f;
                    for (size_t i = 0; i < cfg->nphoton; i++) {
                        sc += cfg->replay.weight[i];
                    }
                    if (sc > 0.f) {
                        sc = cfg->unitinmm / sc;
                    }
                }
            }
            if (nshare > 1) {
                /* each pattern by its total weight (mcx_host.cpp:1436-1447): the
                   pattern sums in the reference's float Kahan summation */
                int psize = (cfg->srctype == MCX_SRC_PATTERN3D)
                            ? (int)cfg->srcparam1.x * (int)cfg->srcparam1.y * (int)cfg->srcparam1.z
                            : (int)cfg->srcparam1.w * (int)cfg->srcparam2.w;
                nblocks = nshare;
                blockscale = (double*)calloc(nblocks, sizeof(double));
                if (!blockscale) {
                    MCX_ERROR(-2, "out of host memory");
                }
                const float scaleref = sc;
                for (uint32_t i = 0; i < nshare; i++) {
                    float sum = 0.f, comp = 0.f;
                    for (int j = 0; j < psize; j++) {
                        const float y = cfg->srcpattern[(size_t)j * nshare + i] - comp;
                        const float t = sum + y;
                        comp = (t - sum) - y;
                        sum = t;
                    }
                    const float si = (float)psize / sum * scaleref;
                    blockscale[i] = (double)si;
                    if (i == 0) {
                        sc = si;
                    }
                }
            }
            if (cfg->extrasrclen && cfg->srcid < 0) {
                sc *= (float)(cfg->extrasrclen + 1);
                if (blockscale) {
                    for (uint32_t b = 0; b < nblocks; b++) {
                        blockscale[b] *= (double)(cfg->extrasrclen + 1);
                    }
                }
            }
            cfg->normalizer = sc;
            cfg->his.normalizer = sc;
            scale = (double)sc;
        }
        if (cfg->debuglevel & 1) {
            scale = 1.0;
            free(blockscale);
            blockscale = NULL;
        }
        /* a complex field (RF transport, rf / rfmus replay) exports its real part
           then its imaginary part (mcx_host.cpp:1050-1052, 1262-1274) */
        const size_t fcomp = ((cfg->omega > 0.f && !replay) ||
                              (replay && (cfg->outputtype == otRF || cfg->outputtype == otRFmus))) ? 2 : 1;
        float* dst = cfg->exportfield;
        if (!dst) {
            /* every element is written by the readback below */
            cfg->exportfield = (float*)outbuf_alloc(sizeof(float) * fieldlen * fcomp);
            if (!cfg->exportfield) {
                MCX_ERROR(-2, "out of host memory");
            }
            dst = cfg->exportfield;
        } else {
            /* caller-supplied buffer: add, as the reference does (mcx_host.cpp:1292-1296) */
            fieldtmp = (float*)malloc(sizeof(float) * fieldlen * fcomp);
            if (!fieldtmp) {
                MCX_ERROR(-2, "out of host memory");
            }
            dst = fieldtmp;
        }
        if (blockscale && nshare > 1) {
            device_check(mcxg_get_field_interleaved(s, dst, blockscale, nblocks), "reading the field");
        } else if (blockscale) {
            device_check(mcxg_get_field_blocks(s, dst, blockscale, nblocks), "reading the field");
        } else {
            device_check(mcxg_get_field(s, dst, scale), "reading the field");
        }
        if (dst == fieldtmp) {
            for (size_t i = 0; i < fieldlen * fcomp; i++) {
                cfg->exportfield[i] += fieldtmp[i];
            }
        }
        if (MCX_IS_ADJOINT_TYPE(cfg->outputtype) && cfg->detdir && !(cfg->debuglevel & 1)) {
            adjoint_jacobians(cfg, s, nvox);
        }
    }
    cfg->his.unitinmm = cfg->unitinmm;
    cfg->his.totalphoton = (unsigned int)cfg->nphoton;
    cfg->his.savedphoton = cfg->detectedcount;
    cfg->his.seedbyte = cfg->issaveseed ? 16u : 0u;

    if (cfg->flog && cfg->parentid == mpStandalone) {
        fprintf(cfg->flog, "simulated %zu photons (%zu) with 1 devices (repeat x%d)\nMCX simulation speed: %.2f photon/ms\n",
                cfg->nphoton, cfg->nphoton, cfg->respin,
                (double)cfg->nphoton * (cfg->respin > 1 ? cfg->respin : 1) / (kms_total > 0.f ? kms_total : 1.f));
        fprintf(cfg->flog, "total simulated energy: %.2f\tabsorbed: %5.5f%%\n(loss due to initial specular reflection is "
                "excluded in the total)\n", cfg->energytot,
                (cfg->energytot - cfg->energyesc) / cfg->energytot * 100.f);
    }
    for (int i = 0; i < 6; i++) {
        free(tmp[i]);
        tmp[i] = NULL;
    }
#undef fieldtmp
#undef blockscale
    MCX_LEAVE();
}

/* mcx_savedetphoton (mcx_utils.c:963-998): the History header, count
   records of his.colcount floats and, when seeds are saved, count seeds of
   his.seedbyte bytes, to <session>.mch (<session>.mct for trajectories). */
void mcx_savedetphoton(float* ppath, void* seeds, int count, int doappend, Config* cfg) {
    MCX_ENTER(cfg);
    char fname[MAX_SESSION_LENGTH + 8];
    char filetag = (cfg->his.detected == 0 && cfg->his.savedphoton) ? 't' : 'h';
    snprintf(fname, sizeof(fname), "%s.mc%c", cfg->session, filetag);
    FILE* fp = fopen(fname, doappend ? "ab" : "wb");
    if (fp == NULL) {
        MCX_ERROR(-2, "can not save data to disk");
    }
    size_t ok = fwrite(&(cfg->his), sizeof(History), 1, fp);
    if (count > 0 && ppath) {
        ok &= fwrite(ppath, sizeof(float), (size_t)count * cfg->his.colcount, fp) == (size_t)count * cfg->his.colcount;
    }
    if (cfg->issaveseed && seeds != NULL && count > 0) {
        ok &= fwrite(seeds, cfg->his.seedbyte, (size_t)count, fp) == (size_t)count;
    }
    fclose(fp);
    if (!ok) {
        MCX_ERROR(-2, "can not save data to disk");
    }
    MCX_LEAVE();
}

/* Reference threads of one batch simulation: ceil(nphoton / ppt), and with
   ppt 0 one photon a thread up to 2^18 photons and two above.  A simulation
   of more than 2^18 photons then has at least 2^17 threads, so the resident
   threads work on one or two simulations at a time and a warp's lanes read
   one descriptor; short threads end each wave with a short tail (2 photons
   a thread ran the 512-simulation batch in 7.32 s, up to 16 in 7.86 s). */
static size_t batch_threads(size_t nphoton, unsigned int ppt) {
    if (!ppt) {
        size_t p = (nphoton + (1u << 18) - 1) >> 18;
        ppt = (unsigned int)(p < 1 ? 1 : (p > 2 ? 2 : p));
    }
    return (nphoton + ppt - 1) / ppt;
}

/* Runs n validated configurations in one persistent launch (a GB300
   addition: the reference runs one simulation per call).  Outputs go to each
   Config as mcx_run_simulation's do; errors are reported on cfgs[0]. */
static int cmp_double(const void* x, const void* y) {
    const double a = *(const double*)x, b = *(const double*)y;
    return (a > b) - (a < b);
}

/* relerr (3 per simulation): the compensated field's max and median
   relative error over the simulation's non-zero elements and the error of
   its total, against the FP64 accumulation of the same deposits */
static void batch_run(Config** cfgs, int n, unsigned int photons_per_thread, unsigned int flags, double* relerr) {
    static __thread void* btmp[7];
    for (int i = 0; i < 7; i++) {
        free(btmp[i]);
        btmp[i] = NULL;
    }
#define bdesc  (*(mcxg_simdesc**)&btmp[0])
#define bwords (*(const uint32_t***)&btmp[1])
#define bscale (*(double**)&btmp[2])
#define bfield (*(float**)&btmp[3])
#define bsums  (*(double**)&btmp[4])
#define bf64   (*(double**)&btmp[5])
#define bcomp  (*(double**)&btmp[6])
    if (n <= 0 || !cfgs || !cfgs[0]) {
        return;
    }
    Config* cfg0 = cfgs[0];
    MCX_ENTER(cfg0);
    uint64_t nmedia = 0, nfield = 0, nvt = 0;
    for (int k = 0; k < n; k++) {
        Config* cfg = cfgs[k];
        if (!cfg || cfg->issavedet || cfg->seed == SEED_FROM_FILE || cfg->extrasrclen || cfg->nphase || cfg->nangle ||
                cfg->srctype == MCX_SRC_PATTERN || cfg->srctype == MCX_SRC_PATTERN3D || cfg->mediabyte > 4 || cfg->omega > 0.f || cfg->polmedianum ||
                cfg->medianum > MCXG_BATCH_MAXMEDIA || cfg->respin != 1 || cfg->issaveref || (cfg->debuglevel & 11)) {
            MCX_ERROR(-4, "a batch simulation takes label volumes of at most 4 property rows, one respin, and no "
                      "detectors, replay, extra sources, patterns, phase tables, saved reflectance or RF");
        }
        if (cfg->nphoton == 0) {
            MCX_ERROR(-4, "every simulation of a batch needs at least one photon");
        }
        cfg->maxgate = (unsigned int)(int)((cfg->tend - cfg->tstart) / cfg->tstep + 0.5);
        size_t nvox = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
        nmedia += nvox;
        nfield += nvox * cfg->maxgate;
        nvt += batch_threads(cfg->nphoton, photons_per_thread);
    }
    if (nfield >= 0x7FFFFFFFull || nvt >= 0xF0000000ull) {
        MCX_ERROR(-1, "batch too large for 32-bit field indices or thread numbering");
    }
    unsigned int workdev = 0;
    GPUInfo* gpu = NULL;
    mcx_list_gpu(cfg0, &workdev, &gpu);
    if (workdev == 0) {
        free(gpu);
        MCX_ERROR(-99, "Specified GPU does not exist");
    }
    int device = gpu[0].id - 1;
    free(gpu);

    bdesc = (mcxg_simdesc*)calloc((size_t)n, sizeof(mcxg_simdesc));
    bwords = (const uint32_t**)malloc(sizeof(uint32_t*) * (size_t)n);
    if (!bdesc || !bwords) {
        MCX_ERROR(-2, "out of host memory");
    }
    uint64_t moff = 0, foff = 0, voff = 0;
    for (int k = 0; k < n; k++) {
        Config* cfg = cfgs[k];
        size_t nvox = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
        size_t fieldlen = nvox * cfg->maxgate;
        size_t vts = batch_threads(cfg->nphoton, photons_per_thread);
        unsigned int is2d = (cfg->dim.x == 1 ? 1 : (cfg->dim.y == 1 ? 2 : (cfg->dim.z == 1 ? 3 : 0)));
        if (is2d) {
            is2d = is2d * (((cfg->dim.x > 1) + (cfg->dim.y > 1) + (cfg->dim.z > 1)) == 2);
        }
        mcxg_simdesc* d = &bdesc[k];
        make_kparams(cfg, nvox, fieldlen, vts, 0, 0, is2d, 0, &d->kp);
        d->kp.threadphoton = (uint32_t)(cfg->nphoton / vts);
        d->kp.oddphoton = (int32_t)(cfg->nphoton - (size_t)d->kp.threadphoton * vts);
        d->kp.mediaword = 1;
        d->kp.savedet = 0;
        d->media_off = moff;
        d->field_off = foff;
        d->vt_off = voff;
        d->seed = (uint64_t)(uint32_t)(cfg->seed > 0 ? cfg->seed : (int)time(0) + k) * 0x100000001B3ull;
        bwords[k] = cfg->vol;        /* packed to label bytes on the device */
        memcpy(d->prop, cfg->prop, sizeof(float) * 4 * cfg->medianum);
        moff += nvox;
        foff += fieldlen;
        voff += vts;
        cfg->threadused = (unsigned int)vts;
    }

    mcxg_session* s = session_for(device);
    if (!s) {
        MCX_ERROR(-99, "failed to open a CUDA session on the selected GPU");
    }
    device_check(mcxg_batch_set_words(s, bdesc, sizeof(mcxg_simdesc), (uint32_t)n, bwords, nmedia), "uploading the batch");
    float kms = 0.f;
    device_check(mcxg_batch_simulate(s, flags | (relerr ? MCXG_VERIFY : 0u), &kms), "running the batch");
    /* the volume copy is resident now (every slot is freed on both exit paths) */
    free(btmp[1]);
    btmp[1] = NULL;
    if (relerr) {
        bf64 = (double*)malloc(sizeof(double) * (nfield ? nfield : 1));
        bcomp = (double*)malloc(sizeof(double) * (nfield ? nfield : 1));
        if (!bf64 || !bcomp) {
            MCX_ERROR(-2, "out of host memory");
        }
        device_check(mcxg_batch_get_verify(s, bf64, bcomp), "reading the precision check");
        for (int k = 0; k < n; k++) {
            const Config* cfg = cfgs[k];
            const size_t off = bdesc[k].field_off, len = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z * cfg->maxgate;
            double tf = 0.0, tc = 0.0, mx = 0.0;
            size_t m = 0;
            for (size_t i = 0; i < len; i++) {
                const double f = bf64[off + i], c = bcomp[off + i];
                tf += f;
                tc += c;
                if (f > 0.0) {
                    const double r = fabs(c - f) / f;
                    mx = r > mx ? r : mx;
                    bf64[off + m++] = r;           /* reuse the slot for the sorted errors */
                }
            }
            qsort(bf64 + off, m, sizeof(double), cmp_double);
            relerr[3 * k] = mx;
            relerr[3 * k + 1] = m ? bf64[off + m / 2] : 0.0;
            relerr[3 * k + 2] = tf > 0.0 ? fabs(tc - tf) / tf : 0.0;
        }
    }
    bscale = (double*)malloc(sizeof(double) * (size_t)n);
    double* scales = bscale;
    bsums = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    if (!bsums || !scales) {
        MCX_ERROR(-2, "out of host memory");
    }
    device_check(mcxg_batch_get_energy(s, bsums), "reducing energies");
    for (int k = 0; k < n; k++) {
        Config* cfg = cfgs[k];
        cfg->energyesc = bsums[2 * k];
        cfg->energytot = bsums[2 * k + 1];
        cfg->energyabs = 0.0;
        cfg->kernelms = kms;
        cfg->runtime = (unsigned int)(kms + 0.5f);
        cfg->detectedcount = 0;
        double sc = 1.0;
        if (cfg->isnormalized) {
            float Vvox = cfg->steps.x * cfg->steps.y * cfg->steps.z;
            float f = 1.f;
            cfg->energyabs = cfg->energytot - cfg->energyesc;
            if (cfg->outputtype == otFlux || cfg->outputtype == otFluence) {
                f = (float)(cfg->unitinmm / (cfg->energytot * Vvox * cfg->tstep));
                if (cfg->outputtype == otFluence) {
                    f *= cfg->tstep;
                }
            } else if (cfg->outputtype == otEnergy || cfg->outputtype == otL) {
                f = (float)(1.0 / cfg->energytot);
            }
            cfg->normalizer = f;
            cfg->his.normalizer = f;
            sc = (double)f;
        }
        scales[k] = sc;
        cfg->his.unitinmm = cfg->unitinmm;
        cfg->his.totalphoton = (unsigned int)cfg->nphoton;
    }
    bfield = (float*)malloc(sizeof(float) * (nfield ? nfield : 1));
    if (!bfield) {
        MCX_ERROR(-2, "out of host memory");
    }
    device_check(mcxg_batch_get_field(s, bfield, scales), "reading the fields");
    for (int k = 0; k < n; k++) {
        Config* cfg = cfgs[k];
        size_t len = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z * cfg->maxgate;
        const float* src = bfield + bdesc[k].field_off;
        if (!cfg->exportfield) {
            cfg->exportfield = (float*)malloc(len * sizeof(float));
            if (!cfg->exportfield) {
                MCX_ERROR(-2, "out of host memory");
            }
            memcpy(cfg->exportfield, src, len * sizeof(float));
        } else {
            /* a caller's buffer accumulates, as a respin of mcx_run_simulation does */
            for (size_t i = 0; i < len; i++) {
                cfg->exportfield[i] += src[i];
            }
        }
    }
    for (int i = 0; i < 7; i++) {
        free(btmp[i]);
        btmp[i] = NULL;
    }
#undef bdesc
#undef bwords
#undef bscale
#undef bfield
#undef bsums
#undef bf64
#undef bcomp
    MCX_LEAVE();
}


void mcx_keep_sessions(int keep) {
    pthread_mutex_lock(&g_run_lock);
    g_keep_sessions = keep != 0;
    if (!g_keep_sessions) {
        release_sessions();
    }
    pthread_mutex_unlock(&g_run_lock);
}

void mcx_run_simulation(Config* cfg, float* fluence, float* totalenergy) {
    (void)fluence;
    (void)totalenergy;
    pthread_mutex_lock(&g_run_lock);
    const int dev = mcxg_internal_current_device();
    run_simulation(cfg);         /* library-mode errors return here through its own setjmp */
    if (!g_keep_sessions) {
        release_sessions();
    }
    mcxg_internal_restore_device(dev);
    pthread_mutex_unlock(&g_run_lock);
}

void mcx_run_batch(Config** cfgs, int n, unsigned int photons_per_thread, unsigned int flags) {
    pthread_mutex_lock(&g_run_lock);
    const int dev = mcxg_internal_current_device();
    batch_run(cfgs, n, photons_per_thread, flags, NULL);
    if (!g_keep_sessions) {
        release_sessions();
    }
    mcxg_internal_restore_device(dev);
    pthread_mutex_unlock(&g_run_lock);
}

void mcx_run_batch_verify(Config** cfgs, int n, unsigned int photons_per_thread, double* relerr) {
    pthread_mutex_lock(&g_run_lock);
    const int dev = mcxg_internal_current_device();
    batch_run(cfgs, n, photons_per_thread, 0u, relerr);
    if (!g_keep_sessions) {
        release_sessions();
    }
    mcxg_internal_restore_device(dev);
    pthread_mutex_unlock(&g_run_lock);
}

mcxg_session* mcx_prepare_simulation(Config* cfg) {
    pthread_mutex_lock(&g_run_lock);
    prepare_only = 1;
    prepared_session = NULL;
    run_simulation(cfg);
    prepare_only = 0;
    mcxg_session* s = cfg->errorcode ? NULL : prepared_session;
    pthread_mutex_unlock(&g_run_lock);
    return s;
}

/* ---- layout introspection, so foreign-function mirrors of Config can be checked */

#include <stddef.h>
#define MCX_FIELD(f) {#f, offsetof(Config, f)}
static const struct {
    const char* name;
    size_t off;
} g_cfg_fields[] = {
    MCX_FIELD(nphoton), MCX_FIELD(nblocksize), MCX_FIELD(nthread), MCX_FIELD(seed), MCX_FIELD(srcpos),
    MCX_FIELD(srcdir), MCX_FIELD(tstart), MCX_FIELD(tstep), MCX_FIELD(tend), MCX_FIELD(steps), MCX_FIELD(dim),
    MCX_FIELD(medianum), MCX_FIELD(detnum), MCX_FIELD(maxdetphoton), MCX_FIELD(prop), MCX_FIELD(detpos),
    MCX_FIELD(maxgate), MCX_FIELD(respin), MCX_FIELD(gpuid), MCX_FIELD(vol), MCX_FIELD(session),
    MCX_FIELD(isrowmajor), MCX_FIELD(isreflect), MCX_FIELD(isrefint), MCX_FIELD(isnormalized), MCX_FIELD(issavedet),
    MCX_FIELD(issave2pt), MCX_FIELD(isgpuinfo), MCX_FIELD(isspecular), MCX_FIELD(issrcfrom0), MCX_FIELD(ismomentum),
    MCX_FIELD(internalsrc), MCX_FIELD(issaveseed), MCX_FIELD(issaveexit), MCX_FIELD(isatomic), MCX_FIELD(issaveref),
    MCX_FIELD(srctype), MCX_FIELD(autopilot), MCX_FIELD(outputtype), MCX_FIELD(minenergy), MCX_FIELD(unitinmm),
    MCX_FIELD(flog), MCX_FIELD(his), MCX_FIELD(energytot), MCX_FIELD(energyabs), MCX_FIELD(energyesc),
    MCX_FIELD(maxvoidstep), MCX_FIELD(voidtime), MCX_FIELD(srcparam1), MCX_FIELD(srcparam2), MCX_FIELD(srcnum),
    MCX_FIELD(srcpattern), MCX_FIELD(deviceid), MCX_FIELD(workload), MCX_FIELD(exportfield),
    MCX_FIELD(exportdetected), MCX_FIELD(debuglevel), MCX_FIELD(normalizer), MCX_FIELD(seeddata), MCX_FIELD(gscatter),
    MCX_FIELD(savedetflag), MCX_FIELD(detectedcount), MCX_FIELD(runtime), MCX_FIELD(parentid), MCX_FIELD(mediabyte),
    MCX_FIELD(bc), MCX_FIELD(nphase), MCX_FIELD(invcdf), MCX_FIELD(nangle), MCX_FIELD(angleinvcdf), MCX_FIELD(srcid),
    MCX_FIELD(extrasrclen), MCX_FIELD(srcdata), MCX_FIELD(replay), MCX_FIELD(replaydet), MCX_FIELD(detdir), MCX_FIELD(exportjacob), MCX_FIELD(exactmath), MCX_FIELD(kernelms), MCX_FIELD(eventcount),
    MCX_FIELD(failedlaunch), MCX_FIELD(threadused), MCX_FIELD(exportenergy), MCX_FIELD(savethreadenergy),
    MCX_FIELD(autotune), MCX_FIELD(savedetweight), MCX_FIELD(exportdetweight), MCX_FIELD(replaysiteown), MCX_FIELD(omega),
    MCX_FIELD(polprop), MCX_FIELD(polmedianum), {"lambda_", offsetof(Config, lambda)}, MCX_FIELD(srciquv),
    MCX_FIELD(smatrix), MCX_FIELD(maxjumpdebug), MCX_FIELD(debugdatalen), MCX_FIELD(exportdebugdata), MCX_FIELD(errorcode), MCX_FIELD(errormsg),
};

size_t mcx_config_sizeof(void) {
    return sizeof(Config);
}

/* offset of a named Config field, or (size_t)-1 */
size_t mcx_config_offsetof(const char* name) {
    for (size_t i = 0; i < sizeof(g_cfg_fields) / sizeof(g_cfg_fields[0]); i++) {
        if (!strcmp(g_cfg_fields[i].name, name)) {
            return g_cfg_fields[i].off;
        }
    }
    return (size_t)-1;
}
