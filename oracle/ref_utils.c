/*
 * ref_utils.c -- drives the reference's host configuration layer and its
 * detected-photon writers for pinning (src/mcx_utils.c and the sources it
 * needs, compiled in place by `make ref`; nothing of them is copied here).
 *
 * TEST INFRASTRUCTURE ONLY.  Built into oracle/_ref/ when the reference
 * sources are present; never committed, never shipped.
 *
 *  - mcxref_readconfig: the reference's mcx_readconfig on a JSON input file
 *    (mcx_loadjson, shapes, mcx_prepdomain / mcx_preprocess, detector mask),
 *    with the loaded configuration summarised into plain arrays, so the
 *    library's own JSON reader can be pinned to it.
 *  - mcxref_savedet: the reference's mcx_savedetphoton, which writes the
 *    .mch file (History header, records, seeds) or, for the JNIfTI output
 *    formats, the .jdat file (mcx_savejdet), so the library's writers can be
 *    pinned to its bytes / structure.
 *
 * zmat is built with zlib (miniz) and base64 only: the writers here use no
 * other codec.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mcx_utils.h"

typedef struct {
    unsigned int dim[3], medianum, detnum, maxgate, srcnum, extrasrclen, savedetflag, debuglevel, maxdetphoton;
    int srctype, seed, isreflect, issavedet, issave2pt, isnormalized, outputtype, mediabyte, issrcfrom0;
    int issaveseed, issaveexit, issaveref, ismomentum, isspecular, autopilot, srcid;
    double nphoton;
    float tstart, tstep, tend, unitinmm, minenergy, steps[3];
    float srcpos[4], srcdir[4], srcparam1[4], srcparam2[4];
    char bc[13];
    char session[64];
} refcfg_summary;

static Config g_cfg;
static int g_loaded = 0;

static void f4(float* out, const float4* v) {
    out[0] = v->x;
    out[1] = v->y;
    out[2] = v->z;
    out[3] = v->w;
}

/* load a JSON input with the reference's reader; the configuration stays
   until the next call or mcxref_release */
int mcxref_readconfig(const char* fname, refcfg_summary* s) {
    if (g_loaded) {
        mcx_clearcfg(&g_cfg);
        g_loaded = 0;
    }
    mcx_initcfg(&g_cfg);
    g_cfg.flog = stderr;
    char name[MAX_PATH_LENGTH];
    snprintf(name, sizeof(name), "%s", fname);
    mcx_readconfig(name, &g_cfg);
    g_loaded = 1;
    memset(s, 0, sizeof(*s));
    s->dim[0] = g_cfg.dim.x;
    s->dim[1] = g_cfg.dim.y;
    s->dim[2] = g_cfg.dim.z;
    s->medianum = g_cfg.medianum;
    s->detnum = g_cfg.detnum;
    s->maxgate = g_cfg.maxgate;
    s->srcnum = g_cfg.srcnum;
    s->extrasrclen = g_cfg.extrasrclen;
    s->savedetflag = g_cfg.savedetflag;
    s->debuglevel = g_cfg.debuglevel;
    s->maxdetphoton = g_cfg.maxdetphoton;
    s->srctype = g_cfg.srctype;
    s->seed = g_cfg.seed;
    s->isreflect = g_cfg.isreflect;
    s->issavedet = g_cfg.issavedet;
    s->issave2pt = g_cfg.issave2pt;
    s->isnormalized = g_cfg.isnormalized;
    s->outputtype = g_cfg.outputtype;
    s->mediabyte = g_cfg.mediabyte;
    s->issrcfrom0 = g_cfg.issrcfrom0;
    s->issaveseed = g_cfg.issaveseed;
    s->issaveexit = g_cfg.issaveexit;
    s->issaveref = g_cfg.issaveref;
    s->ismomentum = g_cfg.ismomentum;
    s->isspecular = g_cfg.isspecular;
    s->autopilot = g_cfg.autopilot;
    s->srcid = g_cfg.srcid;
    s->nphoton = (double)g_cfg.nphoton;
    s->tstart = g_cfg.tstart;
    s->tstep = g_cfg.tstep;
    s->tend = g_cfg.tend;
    s->unitinmm = g_cfg.unitinmm;
    s->minenergy = g_cfg.minenergy;
    s->steps[0] = g_cfg.steps.x;
    s->steps[1] = g_cfg.steps.y;
    s->steps[2] = g_cfg.steps.z;
    f4(s->srcpos, &g_cfg.srcpos);
    f4(s->srcdir, &g_cfg.srcdir);
    f4(s->srcparam1, &g_cfg.srcparam1);
    f4(s->srcparam2, &g_cfg.srcparam2);
    memcpy(s->bc, g_cfg.bc, sizeof(s->bc));
    snprintf(s->session, sizeof(s->session), "%s", g_cfg.session);
    return 0;
}

/* the loaded configuration's media (medianum x 4), detectors (detnum x 4)
   and volume words (nx ny nz, x fastest) */
int mcxref_copyconfig(float* prop, float* detpos, unsigned int* vol) {
    if (!g_loaded) {
        return -1;
    }
    if (prop) {
        memcpy(prop, g_cfg.prop, sizeof(float) * 4 * g_cfg.medianum);
    }
    if (detpos && g_cfg.detnum) {
        memcpy(detpos, g_cfg.detpos, sizeof(float) * 4 * g_cfg.detnum);
    }
    if (vol) {
        memcpy(vol, g_cfg.vol, sizeof(unsigned int) * (size_t)g_cfg.dim.x * g_cfg.dim.y * g_cfg.dim.z);
    }
    return 0;
}

void mcxref_release(void) {
    if (g_loaded) {
        mcx_clearcfg(&g_cfg);
        g_loaded = 0;
    }
}

/* The reference's writer on count records of colcount floats and their
   16-byte seeds, with the History header built field by field from hist[]:
   {version, maxmedia, detnum, colcount, totalphoton, detected, savedphoton,
   seedbyte, respin, srcnum, savedetflag, totalsource} and the floats
   {unitinmm, normalizer}; prop: maxmedia + 1 media rows {mua, mus, g, n}.
   jdat = 1 writes <session>_detp.jdat, else <session>.mch (or .mct), into
   the current directory. */
int mcxref_savedet(const char* session, const unsigned int* hist, const float* histf, const float* prop,
                   float* ppath, void* seeds, int count, int issaveseed, int jdat) {
    Config cfg;
    mcx_initcfg(&cfg);
    cfg.flog = stderr;
    cfg.isdumpjson = 1;            /* quiet: no compression messages */
    snprintf(cfg.session, sizeof(cfg.session), "%s", session);
    cfg.rootpath[0] = '\0';
    cfg.issaveseed = (char)issaveseed;
    cfg.outputformat = jdat ? ofJNifti : ofMC2;
    memcpy(cfg.his.magic, "MCXH", 4);
    cfg.his.version = hist[0];
    cfg.his.maxmedia = hist[1];
    cfg.his.detnum = hist[2];
    cfg.his.colcount = hist[3];
    cfg.his.totalphoton = hist[4];
    cfg.his.detected = hist[5];
    cfg.his.savedphoton = hist[6];
    cfg.his.seedbyte = hist[7];
    cfg.his.respin = (int)hist[8];
    cfg.his.srcnum = hist[9];
    cfg.his.savedetflag = hist[10];
    cfg.his.totalsource = hist[11];
    cfg.his.unitinmm = histf[0];
    cfg.his.normalizer = histf[1];
    cfg.medianum = hist[1] + 1;
    cfg.detnum = hist[2];
    cfg.savedetflag = hist[10];
    cfg.unitinmm = histf[0];
    cfg.prop = (Medium*)malloc(sizeof(Medium) * cfg.medianum);      /* the .jdat Info lists the media */
    memcpy(cfg.prop, prop, sizeof(Medium) * cfg.medianum);
    mcx_savedetphoton(ppath, seeds, count, 0, &cfg);
    mcx_clearcfg(&cfg);
    return 0;
}

/* The reference's JNIfTI volume writer (mcx_savejnii, src/mcx_utils.c:761-884)
   on a float volume of ndim dims (x fastest), into <name>.jnii; the header
   takes the session name, the gate count and the output type from cfg. */
int mcxref_savejnii(float* vol, int ndim, unsigned int* dims, float* voxelsize, const char* name, const char* session,
                    unsigned int maxgate, int outputtype) {
    Config cfg;
    mcx_initcfg(&cfg);
    cfg.flog = stderr;
    cfg.isdumpjson = 1;
    snprintf(cfg.session, sizeof(cfg.session), "%s", session);
    cfg.maxgate = maxgate;
    cfg.outputtype = (char)outputtype;
    char fname[MAX_PATH_LENGTH];
    snprintf(fname, sizeof(fname), "%s", name);
    mcx_savejnii(vol, ndim, dims, voxelsize, fname, 1, 1, &cfg);
    mcx_clearcfg(&cfg);
    return 0;
}
