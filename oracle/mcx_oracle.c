/*
 * mcx_oracle.c -- CPU oracle for the MCX-CL photon-transport path.
 *
 * TEST INFRASTRUCTURE ONLY (see mcx_oracle.h).  The product never links this.
 *
 * A plain-C restatement of the reference algorithm.  Citations are to the
 * reference project's files (src/mcx_core.cl, src/mcx_host.cpp,
 * src/mcx_utils.c).  Expressions keep the reference's operand order so that,
 * compiled with -ffp-contract=off, the oracle reproduces the reference kernel
 * (compiled on the host from its own sources) bit for bit; see oracle/Makefile.
 *
 * One reference thread ("virtual thread", vt) owns one xorshift128+ stream
 * and simulates threadphoton (+1 for the first oddphoton threads) photons in
 * sequence.  The oracle runs the threads in index order (serially, or in
 * contiguous chunks per OpenMP worker), so its outputs do not depend on the
 * worker count except for the summation order of the FP64 field.
 */
#define _GNU_SOURCE
#include "mcx_oracle.h"
#include "oracle_pmath.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* kernel-side constants, mcx_core.cl:457-516 */
#define K_EPS            FLT_EPSILON
#define K_VERY_BIG       (1.f / FLT_EPSILON)
#define K_ONE_PI         3.1415926535897932f
#define K_TWO_PI         6.28318530717959f
#define K_JUST_BELOW_ONE 0.9998f
#define K_R_C0           3.335640951981520e-12f
#define K_MAX_ACCUM      1000.f
#define K_ROULETTE_SIZE  10.f
#define H_EPS            1e-10f          /* host EPS, mcx_const.h:30 */
#define K_VERY_BIG_H     1e10f           /* host VERY_BIG, mcx_const.h:35 */
#define OUT_MIN          0xFFFFFFFFu
#define OUT_MAX          0x7FFFFFFFu
#define DET_MASK         0x80000000u
#define MED_MASK         0x7FFFFFFFu
#define FILL_MAXDET      3
#define MEDIA_MUA_FLOAT  101
#define MEDIA_2LABEL_SPLIT 97
/* split-voxel state (mcx_core.cl:577-587): lower and upper labels, whether the
   voxel is split and which side the photon is on */
#define SV_LOWER(sv)     ((sv) & 0xFFu)
#define SV_UPPER(sv)     (((sv) >> 8) & 0xFFu)
#define SV_ISSPLIT(sv)   (((sv) >> 16) & 1u)
#define SV_ISUPPER(sv)   (((sv) >> 17) & 1u)
#define SV_CURLABEL(sv)  (SV_ISUPPER(sv) ? SV_UPPER(sv) : SV_LOWER(sv))
#define LAUNCH_ATTEMPT_CAP (1u << 16)  /* guard against a source that never yields weight */
#define CONE_DRAW_CAP      (1u << 16)  /* guard against a cone of zero half-angle */

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
#define K_NANGLES     181
#define K_R_PI        0.318309886183791f

typedef struct { float x, y, z, w; } f4;
typedef struct { f4 pos, dir, p1, p2; } osrc;

/* Restated kernel constant block (MCXParam, mcx_host.h:106-166), only the
   fields the path reads. */
typedef struct {
    osrc src;
    unsigned int extrasrclen;
    int srcid;
    f4 maxidx;
    unsigned int dimlen[4];
    float twin0, twin1, oneoverc0, Rtstep, minenergy, minaccumtime;
    unsigned int save2pt, doreflect, savedet, maxdetphoton, maxmedia, detnum, voidtime;
    unsigned int srctype, maxvoidstep, issaveseed, issaveref, isspecular, maxgate, outputtype;
    unsigned int threadphoton, savedetflag, reclen, partialdata, w0offset, mediaformat;
    unsigned int gscatter, is2d, srcnum, nphase, nangle;
    int oddphoton;
    unsigned char bc[12];
    int dorefl_compiled;          /* MCX_DO_REFLECTION, mcx_host.cpp:945-956 */
    const f4* gprop;              /* medianum rows, then 4 float4 per extra source */
    const f4* gdet;
    const uint32_t* media;
    const float* srcpattern;
    const float* invcdf;          /* nphase entries */
    const float* angleinvcdf;     /* nangle entries */
    int mathmode, variant, fieldmode;
    float omega;
    int rfmode;                   /* 0 real, 1 RF forward (complex weights), 2 RF replay output */
    const f4* smatrix;            /* polarised transport: 181 Mueller rows per medium */
    unsigned int maxpol;
    f4 s0;
    unsigned int nthread;
    /* replay */
    int replay, replaydet, replaysiteown;
    unsigned int nreplay;
    const uint64_t* rseed;
    const float* rweight;
    const float* rtof;
    const int* rdetid;
    /* trajectory capture */
    int debugmove;
    unsigned int maxtraj;
    float* traj;
    unsigned int* ntraj;
} ocfg;

typedef struct {
    const ocfg* c;
    float* ff;            /* FLOAT_SPILL: 2*fieldlen */
    double* fd;           /* DOUBLE: fieldlen */
    float* detp;          /* record buffer for this worker */
    float* detw;          /* weight and time of flight of each record when detected, or NULL */
    uint64_t* dseed;
    unsigned int detcap;  /* records this worker may store */
    unsigned int detcount;
    uint64_t nstep, nscatter, nlaunch, nreflect, nfailed;
    unsigned int tid;
} octx;

typedef struct {
    f4 p, v, f, prop;
    short fid[4];                 /* flipdir {x, y, z, face} */
    uint32_t idx1d, mediaid, isdet;
    float w0, Lmove, pathlen, n1;
    uint64_t t[2];
    uint64_t photonseed[2];
    float* ppath;                 /* w0offset + srcnum (+ 2 for an RF replay) floats */
    float wre, wim, w0re, w0im;   /* RF forward: complex weight now and at the last voxel change */
    f4 st;                        /* polarised transport: Stokes vector {I, Q, U, V} */
    float nv[3], pd;              /* split voxel: plane normal (pointing away from the photon's side), offset */
    uint32_t sv;
} ostate;

/* ---------------------------------------------------------------- helpers */

static inline float bits2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t f2bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static inline float m_log(const ocfg* c, float x) { return c->mathmode ? opm_logf(x) : logf(x); }
static inline float m_exp(const ocfg* c, float x) { return c->mathmode ? opm_expf(x) : expf(x); }
static inline float m_acos(const ocfg* c, float x) { return c->mathmode ? opm_acosf(x) : acosf(x); }
static inline float m_sin(const ocfg* c, float x) { return c->mathmode ? opm_sinf(x) : sinf(x); }
static inline float m_cos(const ocfg* c, float x) { return c->mathmode ? opm_cosf(x) : cosf(x); }
static inline void m_sincos(const ocfg* c, float x, float* s, float* co) {
    if (c->mathmode) {
        opm_sincosf(x, s, co);
    } else {
        sincosf(x, s, co);
    }
}
static inline float m_rsqrt(float x) { return 1.f / sqrtf(x); }

/* xorshift128+ draw, mcx_core.cl:684-698: low 32 bits of the sum become the
   mantissa of a float in [1,2) */
static inline float rng_next(uint64_t t[2]) {
    uint64_t s1 = t[0];
    const uint64_t s0 = t[1];
    uint64_t r;
    t[0] = s0;
    s1 ^= s1 << 23;
    t[1] = s1 ^ s0 ^ (s1 >> 18) ^ (s0 >> 5);
    r = t[1] + s0;
    return bits2f(0x3F800000u | ((uint32_t)r >> 9)) - 1.0f;
}

/* mcx_core.cl:720-722 */
static inline float rng_scatlen(const ocfg* c, uint64_t t[2]) {
    return -m_log(c, rng_next(t) + K_EPS);
}

/* mcx_core.cl:965-973 */
static inline float nextafter_ref(float a, int dir) {
    uint32_t i = f2bits(a + 1000.f);
    i += (uint32_t)dir ^ (i & 0x80000000U);
    return bits2f(i) - 1000.f;
}

/* returns 1 when the float accumulator spilled */
static inline int field_add(octx* X, size_t i, float w) {
    const ocfg* c = X->c;
    if (c->fieldmode == MCXO_FIELD_FLOAT_SPILL) {
        float old = X->ff[i];
        X->ff[i] = old + w;
        if (fabsf(old) > K_MAX_ACCUM) {
            X->ff[i] += ((old > 0.f) ? -K_MAX_ACCUM : K_MAX_ACCUM);
            X->ff[i + c->dimlen[3]] += ((old > 0.f) ? K_MAX_ACCUM : -K_MAX_ACCUM);
            return 1;
        }
    } else {
        X->fd[i >= c->dimlen[3] ? i - c->dimlen[3] : i] += (double)w;
    }
    return 0;
}

/* RF deposits of the imaginary part (mcx_core.cl:2887-2898, 2609-2617): the
   forward run and the rfmus scattering sites write the third quarter of the
   field with its own +-1000 spill into the fourth; the rf replay output
   writes the second half without a spill.  In FP64 the imaginary part is the
   second fieldlen block. */
static inline void field_add_im(octx* X, size_t i, float w, int quarter) {
    const ocfg* c = X->c;
    const size_t F = c->dimlen[3];
    if (c->fieldmode == MCXO_FIELD_FLOAT_SPILL) {
        if (quarter) {
            float old = X->ff[i + 2 * F];
            X->ff[i + 2 * F] = old + w;
            if (fabsf(old) > K_MAX_ACCUM) {
                X->ff[i + 2 * F] += ((old > 0.f) ? -K_MAX_ACCUM : K_MAX_ACCUM);
                X->ff[i + 3 * F] += ((old > 0.f) ? K_MAX_ACCUM : -K_MAX_ACCUM);
            }
        } else {
            X->ff[i + F] += w;
        }
    } else {
        X->fd[F + (i >= F ? i - F : i)] += (double)w;
    }
}

/* the rf replay output's real part has no spill (mcx_core.cl:2884) */
static inline void field_add_nospill(octx* X, size_t i, float w) {
    const ocfg* c = X->c;
    if (c->fieldmode == MCXO_FIELD_FLOAT_SPILL) {
        X->ff[i] += w;
    } else {
        X->fd[i >= c->dimlen[3] ? i - c->dimlen[3] : i] += (double)w;
    }
}

/* updatestokes (mcx_core.cl:792-835) with rotsphi (792-799) */
static void update_stokes(const ocfg* c, ostate* s, float theta, float phi, const f4* u, const f4* u2) {
    float costheta = m_cos(c, theta);
    float sin2phi, cos2phi, temp, sini, cosi, sin22, cos22;
    f4 s2, m;
    uint32_t imedia, ithedeg;
    m_sincos(c, 2.f * phi, &sin2phi, &cos2phi);
    s2.x = s->st.x;
    s2.y = s->st.y * cos2phi + s->st.z * sin2phi;
    s2.z = -s->st.y * sin2phi + s->st.z * cos2phi;
    s2.w = s->st.w;
    imedia = K_NANGLES * ((s->mediaid & MED_MASK) - 1);
    ithedeg = (uint32_t)(theta * K_NANGLES * (K_R_PI - K_EPS));
    m = c->smatrix[imedia + ithedeg];
    s->st.x = m.x * s2.x + m.y * s2.y;
    s->st.y = m.y * s2.x + m.x * s2.y;
    s->st.z = m.z * s2.z + m.w * s2.w;
    s->st.w = -m.w * s2.z + m.z * s2.w;
    temp = (u2->z > -1.f && u2->z < 1.f) ? m_rsqrt((1.f - costheta * costheta) * (1.f - u2->z * u2->z)) : 0.f;
    cosi = (temp == 0.f) ? 0.f : (((phi > K_ONE_PI && phi < K_TWO_PI) ? 1.f : -1.f) * (u2->z * costheta - u->z) * temp);
    cosi = fmaxf(-1.f, fminf(cosi, 1.f));
    sini = sqrtf(1.f - cosi * cosi);
    cos22 = 2.f * cosi * cosi - 1.f;
    sin22 = 2.f * sini * cosi;
    s2.x = s->st.x;
    s2.y = s->st.y * cos22 - s->st.z * sin22;
    s2.z = s->st.y * sin22 + s->st.z * cos22;
    s2.w = s->st.w;
    temp = 1.f / s2.x;
    s->st.y = s2.y * temp;
    s->st.z = s2.z * temp;
    s->st.w = s2.w * temp;
    s->st.x = 1.f;
}

/* updateproperty_svmc (mcx_core.cl:1231-1280): the properties of the side of
   the voxel's plane the photon is on; the plane's reference point and normal
   decode from the second volume plane */
static void updateprop_svmc(const ocfg* c, f4* prop, uint32_t mediaid, uint32_t idx1d, const f4* p, ostate* s,
                            const short fid[4]) {
    uint32_t i0, i1, sv;
    unsigned char b[8];
    if (idx1d == OUT_MIN || idx1d == OUT_MAX) {
        *prop = c->gprop[0];
        return;
    }
    i0 = c->media[idx1d + c->dimlen[2]];
    i1 = mediaid & MED_MASK;
    b[0] = i0 & 0xFF, b[1] = (i0 >> 8) & 0xFF, b[2] = (i0 >> 16) & 0xFF, b[3] = (i0 >> 24) & 0xFF;
    b[4] = i1 & 0xFF, b[5] = (i1 >> 8) & 0xFF, b[6] = (i1 >> 16) & 0xFF, b[7] = (i1 >> 24) & 0xFF;
    sv = (uint32_t)b[7] | ((uint32_t)b[6] << 8);
    if (b[6]) {
        float rx = b[5] * (1.f / 255.f) + (float)fid[0];
        float ry = b[4] * (1.f / 255.f) + (float)fid[1];
        float rz = b[3] * (1.f / 255.f) + (float)fid[2];
        float nx = b[2] * (2.f / 255.f) - 1.f, ny = b[1] * (2.f / 255.f) - 1.f, nz = b[0] * (2.f / 255.f) - 1.f;
        float r = m_rsqrt(nx * nx + ny * ny + nz * nz);
        nx = nx * r, ny = ny * r, nz = nz * r;
        s->pd = rx * nx + ry * ny + rz * nz;
        if (p->x * nx + p->y * ny + p->z * nz > s->pd) {
            *prop = c->gprop[SV_UPPER(sv)];
            sv |= 1u << 17;
            nx = -nx, ny = -ny, nz = -nz;
            s->pd = -s->pd;
        } else {
            *prop = c->gprop[SV_LOWER(sv)];
            sv &= ~(1u << 17);
        }
        s->nv[0] = nx, s->nv[1] = ny, s->nv[2] = nz;
        sv |= 1u << 16;
    } else {
        *prop = c->gprop[b[7]];
        sv &= 0xFFFFu;
    }
    s->sv = sv;
}

/* ray_plane_intersect (1282-1303): clip the step at the voxel's plane when
   the photon moves towards it and crosses it within the step */
static int ray_plane_intersect(const ocfg* c, const ostate* s, float* len, float* slen) {
    float vdotn = s->v.x * s->nv[0] + s->v.y * s->nv[1] + s->v.z * s->nv[2];
    float d0, d1, len0;
    if (vdotn <= 0.f) {
        return 0;
    }
    d0 = s->p.x * s->nv[0] + s->p.y * s->nv[1] + s->p.z * s->nv[2] - s->pd;
    d1 = d0 + (*len) * vdotn;
    if (d0 * d1 > 0.f) {
        return 0;
    }
    len0 = ((*len) * d0) / (d0 - d1);
    *len = (len0 > 0.f) ? len0 : *len;
    *slen = (*len) * s->prop.y * (s->v.w + 1.f > (float)c->gscatter ? (1.f - s->prop.z) : 1.f);
    return 1;
}

/* reflectray_svmc (1305-1343): Fresnel reflection or refraction at the
   voxel's plane; 1 when the photon refracts into a background half */
static int reflectray_svmc(const ocfg* c, float n1, float* c0, ostate* s) {
    float Icos, Re, Im, Rtotal, tmp0, tmp1, tmp2, n2;
    Icos = fabsf(c0[0] * s->nv[0] + c0[1] * s->nv[1] + c0[2] * s->nv[2]);
    n2 = SV_ISUPPER(s->sv) ? c->gprop[SV_UPPER(s->sv)].w : c->gprop[SV_LOWER(s->sv)].w;
    tmp0 = n1 * n1;
    tmp1 = n2 * n2;
    tmp2 = 1.f - tmp0 / tmp1 * (1.f - Icos * Icos);
    if (tmp2 > 0.f) {
        Re = tmp0 * Icos * Icos + tmp1 * tmp2;
        tmp2 = sqrtf(tmp2);
        Im = 2.f * n1 * n2 * Icos * tmp2;
        Rtotal = (Re - Im) / (Re + Im);
        Re = tmp1 * Icos * Icos + tmp0 * tmp2 * tmp2;
        Rtotal = (Rtotal + (Re - Im) / (Re + Im)) * 0.5f;
        if (rng_next(s->t) <= Rtotal) {
            c0[0] += (-2.f * Icos) * s->nv[0], c0[1] += (-2.f * Icos) * s->nv[1], c0[2] += (-2.f * Icos) * s->nv[2];
            s->sv ^= 1u << 17;
        } else {
            int k;
            c0[0] += (-Icos) * s->nv[0], c0[1] += (-Icos) * s->nv[1], c0[2] += (-Icos) * s->nv[2];
            for (k = 0; k < 3; k++) {
                c0[k] = tmp2 * s->nv[k] + (n1 / n2) * c0[k];
            }
            s->nv[0] = -s->nv[0], s->nv[1] = -s->nv[1], s->nv[2] = -s->nv[2];
            s->pd = -s->pd;
            if (SV_CURLABEL(s->sv) == 0) {
                return 1;
            }
            s->prop = c->gprop[SV_CURLABEL(s->sv)];
        }
    } else {
        c0[0] += (-2.f * Icos) * s->nv[0], c0[1] += (-2.f * Icos) * s->nv[1], c0[2] += (-2.f * Icos) * s->nv[2];
        s->sv ^= 1u << 17;
    }
    tmp0 = m_rsqrt(c0[0] * c0[0] + c0[1] * c0[1] + c0[2] * c0[2]);
    c0[0] = c0[0] * tmp0, c0[1] = c0[1] * tmp0, c0[2] = c0[2] * tmp0;
    return 0;
}

/* a deposit with photon sharing (mcx_core.cl:1527-1538, 2902-2911, the
   kernel built for pattern sources): each pattern with a non-zero share adds
   weight x share at element i * srcnum + k; one pattern adds weight at i */
static inline int share_add(octx* X, const ostate* s, size_t i, float w) {
    const ocfg* c = X->c;
    unsigned int k;
    if (c->srcnum <= 1) {
        return field_add(X, i, w);
    }
    for (k = 0; k < c->srcnum; k++) {
        float pw = s->ppath[c->w0offset + k];
        if (fabsf(pw) > 0.f) {
            field_add(X, i * c->srcnum + k, w * pw);
        }
    }
    return 0;
}

/* the scattering-site deposit of the replay outputs moves a saturated value
   whole into the shadow half (mcx_core.cl:2597-2604) */
static inline void field_add_site(octx* X, size_t i, float w) {
    const ocfg* c = X->c;
    if (c->fieldmode == MCXO_FIELD_FLOAT_SPILL) {
        float old = X->ff[i];
        X->ff[i] = old + w;
        if (fabsf(old) > K_MAX_ACCUM) {
            float r = X->ff[i];
            X->ff[i] = r - old;
            if (r < 0.f) {
                X->ff[i] += old;
            } else {
                X->ff[i + c->dimlen[3]] += old;
            }
        }
    } else {
        X->fd[i >= c->dimlen[3] ? i - c->dimlen[3] : i] += (double)w;
    }
}

/* index of the photon a replay quantity is read for: the reference's
   idx*threadphoton + min(idx, oddphoton-1) + offset (mcx_core.cl:1591, 2571, 2847) */
static inline long long replay_index(const ocfg* c, unsigned int tid, long long offset) {
    long long m = (long long)c->oddphoton - 1;
    long long t = (long long)tid;
    return t * (long long)c->threadphoton + (t < m ? t : m) + offset;
}

/* IEEE half -> float (exact) */
static inline float half2f(uint32_t h) {
    uint32_t s = (h & 0x8000u) << 16, e = (h >> 10) & 0x1Fu, m = h & 0x3FFu;
    if (e == 0) {
        float v = (float)m * (1.f / 16777216.f);     /* m * 2^-24, exact */
        return s ? -v : v;
    }
    if (e == 31) {
        return bits2f(s | 0x7F800000u | (m << 13));
    }
    return bits2f(s | ((e + 112u) << 23) | (m << 13));
}

/* updateproperty, mcx_core.cl:1079-1187: labels, float mua, half mua/mus,
   label + one half-precision property, byte and short mixtures of rows 1-2 */
static inline void updateprop(const ocfg* c, f4* prop, uint32_t mediaid) {
    const uint32_t w = mediaid & MED_MASK;
    if (c->mediaformat <= 4) {
        *prop = c->gprop[w];
    } else if (c->mediaformat == MEDIA_MUA_FLOAT) {
        prop->x = fabsf(bits2f(mediaid));
        prop->w = c->gprop[(!w) == 0].w;
    } else if (c->mediaformat == 100 || c->mediaformat == 102) {
        prop->x = fabsf(half2f(w & 0xFFFFu));
        prop->y = fabsf(half2f(w >> 16));
        prop->w = c->gprop[(!w) == 0].w;
    } else if (c->mediaformat == 99) {
        float* p = (float*)prop;
        *prop = c->gprop[w & 0x3FFFu];
        p[(w & 0xC000u) >> 14] = fabsf(half2f(w >> 16));
    } else if (c->mediaformat == 103) {
        const f4 a = c->gprop[1], b = c->gprop[2];
        prop->x = (float)(w & 0xFF) * (1.f / 255.f) * (b.x - a.x) + a.x;
        prop->y = (float)((w >> 8) & 0xFF) * (1.f / 255.f) * (b.y - a.y) + a.y;
        prop->z = (float)((w >> 16) & 0xFF) * (1.f / 255.f) * (b.z - a.z) + a.z;
        prop->w = (float)(w >> 24) * (1.f / 127.f) * (b.w - a.w) + a.w;
    } else if (c->mediaformat == 104) {
        const f4 a = c->gprop[1], b = c->gprop[2];
        prop->x = (float)(w & 0xFFFF) * (1.f / 65535.f) * (b.x - a.x) + a.x;
        prop->y = (float)(w >> 16) * (1.f / 65535.f) * (b.y - a.y) + a.y;
        prop->w = c->gprop[(!w) == 0].w;
    }
}

/* hitgrid, mcx_core.cl:975-995 */
static float hitgrid(const ocfg* c, const f4* p, const f4* v, short fid[4]) {
    float hx, hy, hz, dist;
    if (c->variant == MCXO_VARIANT_NVCC) {
        float gx = v->x > 0.f ? 1.f : 0.f, gy = v->y > 0.f ? 1.f : 0.f, gz = v->z > 0.f ? 1.f : 0.f;
        hx = v->x == 0.f ? K_VERY_BIG : fabsf(((float)fid[0] + gx - p->x) * (1.f / v->x));
        hy = v->y == 0.f ? K_VERY_BIG : fabsf(((float)fid[1] + gy - p->y) * (1.f / v->y));
        hz = v->z == 0.f ? K_VERY_BIG : fabsf(((float)fid[2] + gz - p->z) * (1.f / v->z));
    } else {
        /* OpenCL: isgreater() is -1 for true, so id - isgreater = id + (v>0) */
        hx = fabsf((float)fid[0] - (v->x > 0.f ? -1.f : 0.f) - p->x);
        hy = fabsf((float)fid[1] - (v->y > 0.f ? -1.f : 0.f) - p->y);
        hz = fabsf((float)fid[2] - (v->z > 0.f ? -1.f : 0.f) - p->z);
        hx = fabsf((hx + K_EPS) / v->x);
        hy = fabsf((hy + K_EPS) / v->y);
        hz = fabsf((hz + K_EPS) / v->z);
    }
    dist = fminf(fminf(hx, hy), hz);
    fid[3] = (dist == hx ? 0 : (dist == hy ? 1 : 2));
    return dist;
}

/* rotatevector, mcx_core.cl:1025-1042 */
static void rotatevector(const ocfg* c, f4* v, float st, float ct, float sp, float cp) {
    (void)c;
    if (v->z > -1.f + K_EPS && v->z < 1.f - K_EPS) {
        float tmp0 = 1.f - v->z * v->z;
        float tmp1 = st * m_rsqrt(tmp0);
        f4 n;
        n.x = tmp1 * (v->x * v->z * cp - v->y * sp) + v->x * ct;
        n.y = tmp1 * (v->y * v->z * cp + v->x * sp) + v->y * ct;
        n.z = -tmp1 * tmp0 * cp + v->z * ct;
        n.w = v->w;
        *v = n;
    } else {
        f4 n;
        n.x = st * cp;
        n.y = st * sp;
        n.z = (v->z > 0.f) ? ct : -ct;
        n.w = v->w;
        *v = n;
    }
    v->x *= m_rsqrt(v->x * v->x + v->y * v->y + v->z * v->z);
    v->y *= m_rsqrt(v->x * v->x + v->y * v->y + v->z * v->z);
    v->z *= m_rsqrt(v->x * v->x + v->y * v->y + v->z * v->z);
}

/* rotatevector2d, mcx_core.cl:1008-1023 */
static void rotatevector2d(f4* v, float st, float ct, unsigned int is2d) {
    f4 n = *v;
    if (is2d == 1) {
        n.x = 0.f;
        n.y = v->y * ct - v->z * st;
        n.z = v->y * st + v->z * ct;
    } else if (is2d == 2) {
        n.x = v->x * ct - v->z * st;
        n.y = 0.f;
        n.z = v->x * st + v->z * ct;
    } else if (is2d == 3) {
        n.x = v->x * ct - v->y * st;
        n.y = v->x * st + v->y * ct;
        n.z = 0.f;
    }
    *v = n;
    {
        float tmp0 = m_rsqrt(v->x * v->x + v->y * v->y + v->z * v->z);
        v->x *= tmp0;
        v->y *= tmp0;
        v->z *= tmp0;
    }
}

/* rotate_perpendicular_vector, mcx_core.cl:997-1006 */
static void rotate_perp(f4* d, float ax, float ay, float az, float st, float ct) {
    float cx = ay * d->z - az * d->y;
    float cy = az * d->x - ax * d->z;
    float cz = ax * d->y - ay * d->x;
    d->x = d->x * ct + cx * st;
    d->y = d->y * ct + cy * st;
    d->z = d->z * ct + cz * st;
}

static inline float vcomp(const f4* v, int k) { return k == 0 ? v->x : (k == 1 ? v->y : v->z); }

/* transmit, mcx_core.cl:1044-1055 */
static void transmit(f4* v, float n1, float n2, short fw) {
    float tmp0 = n1 / n2;
    v->x *= tmp0;
    v->y *= tmp0;
    v->z *= tmp0;
    if (fw == 0) {
        v->x = sqrtf(1.f - v->y * v->y - v->z * v->z) * (float)((v->x > 0.f) - (v->x < 0.f));
    } else if (fw == 1) {
        v->y = sqrtf(1.f - v->x * v->x - v->z * v->z) * (float)((v->y > 0.f) - (v->y < 0.f));
    } else {
        v->z = sqrtf(1.f - v->x * v->x - v->y * v->y) * (float)((v->z > 0.f) - (v->z < 0.f));
    }
}

/* reflectcoeff, mcx_core.cl:1057-1075 */
static float reflectcoeff(const f4* v, float n1, float n2, short fw) {
    float Icos = fabsf(vcomp(v, fw));
    float tmp0 = n1 * n1;
    float tmp1 = n2 * n2;
    float tmp2 = 1.f - tmp0 / tmp1 * (1.f - Icos * Icos);
    if (tmp2 > 0.f) {
        float Re, Im, Rtotal;
        Re = tmp0 * Icos * Icos + tmp1 * tmp2;
        tmp2 = sqrtf(tmp2);
        Im = 2.f * n1 * n2 * Icos * tmp2;
        Rtotal = (Re - Im) / (Re + Im);
        Re = tmp1 * Icos * Icos + tmp0 * tmp2 * tmp2;
        Rtotal = (Rtotal + (Re - Im) / (Re + Im)) * 0.5f;
        return Rtotal;
    }
    return 1.f;
}

static inline int inside_u(const ocfg* c, short x, short y, short z) {
    return (float)(unsigned short)x < c->maxidx.x && (float)(unsigned short)y < c->maxidx.y &&
           (float)(unsigned short)z < c->maxidx.z;
}

static inline uint32_t vox_index(const ocfg* c, short x, short y, short z) {
    return (uint32_t)((int)z * (int)c->dimlen[1] + (int)y * (int)c->dimlen[0] + (int)x);
}

/* skipvoid, mcx_core.cl:1350-1455 */
static int skipvoid(const ocfg* c, f4* p, f4* v, f4* f, short fid[4]) {
    int count = 1;
    fid[0] = (short)floorf(p->x);
    fid[1] = (short)floorf(p->y);
    fid[2] = (short)floorf(p->z);
    fid[3] = -1;
    for (;;) {
        if (inside_u(c, fid[0], fid[1], fid[2])) {
            int idx1d = (int)vox_index(c, fid[0], fid[1], fid[2]);
            if (c->media[idx1d] & MED_MASK) {
                p->x -= v->x;
                p->y -= v->y;
                p->z -= v->z;
                fid[0] = (short)floorf(p->x);
                fid[1] = (short)floorf(p->y);
                fid[2] = (short)floorf(p->z);
                f->y -= c->minaccumtime;
                idx1d = (int)vox_index(c, fid[0], fid[1], fid[2]);
                count = 0;
                while (!inside_u(c, fid[0], fid[1], fid[2]) || !(c->media[idx1d] & MED_MASK)) {
                    float dist = hitgrid(c, p, v, fid);
                    f->y += c->minaccumtime * dist;
                    p->x = p->x + dist * v->x;
                    p->y = p->y + dist * v->y;
                    p->z = p->z + dist * v->z;
                    if (fid[3] == 0) {
                        fid[0] += (v->x > 0.f ? 1 : -1);
                    }
                    if (fid[3] == 1) {
                        fid[1] += (v->y > 0.f ? 1 : -1);
                    }
                    if (fid[3] == 2) {
                        fid[2] += (v->z > 0.f ? 1 : -1);
                    }
                    idx1d = (int)vox_index(c, fid[0], fid[1], fid[2]);
                    if (count++ > 3) {
                        break;
                    }
                }
                f->y = (c->voidtime) ? f->y : 0.f;
                {
                    f4 htime = {0.f, 0.f, 0.f, 0.f};
                    if (c->mediaformat == MEDIA_2LABEL_SPLIT) {
                        /* the side of the entry voxel's plane (1404-1420); the launch then
                           sets the photon's split state again, and the specular test uses
                           that side's index where the reference reads the property table
                           at the packed voxel word */
                        ostate tmp;
                        memset(&tmp, 0, sizeof(tmp));
                        updateprop_svmc(c, &htime, c->media[idx1d], (uint32_t)idx1d, p, &tmp, fid);
                    } else {
                        updateprop(c, &htime, c->media[idx1d]);
                    }
                    /* htime.w equals gproperty[label].w of mcx_core.cl:1425-1429 for labels;
                       for float-mua volumes the reference indexes past the table there */
                    if (c->isspecular && htime.w != c->gprop[0].w) {
                        p->w *= 1.f - reflectcoeff(v, c->gprop[0].w, htime.w, fid[3]);
                        if (p->w > K_EPS) {
                            transmit(v, c->gprop[0].w, htime.w, fid[3]);
                        }
                    }
                }
                return idx1d;
            }
        }
        if (((p->x < 0.f) && (v->x <= 0.f)) || ((p->x >= c->maxidx.x) && (v->x >= 0.f)) ||
            ((p->y < 0.f) && (v->y <= 0.f)) || ((p->y >= c->maxidx.y) && (v->y >= 0.f)) ||
            ((p->z < 0.f) && (v->z <= 0.f)) || ((p->z >= c->maxidx.z) && (v->z >= 0.f))) {
            return -1;
        }
        p->x = p->x + v->x;
        p->y = p->y + v->y;
        p->z = p->z + v->z;
        fid[0] = (short)floorf(p->x);
        fid[1] = (short)floorf(p->y);
        fid[2] = (short)floorf(p->z);
        f->y += c->minaccumtime;
        if ((unsigned int)count++ > c->maxvoidstep) {
            return -1;
        }
    }
}

/* finddetector, mcx_core.cl:838-850 */
static unsigned int finddetector(const ocfg* c, const f4* p) {
    unsigned int i;
    for (i = 0; i < c->detnum; i++) {
        const f4* d = &c->gdet[i];
        if ((d->x - p->x) * (d->x - p->x) + (d->y - p->y) * (d->y - p->y) + (d->z - p->z) * (d->z - p->z) <
                d->w * d->w) {
            return i + 1;
        }
    }
    return 0;
}

/* savedetphoton, mcx_core.cl:867-926 */
static void savedetphoton(octx* X, ostate* s, uint32_t isdet) {
    const ocfg* c = X->c;
    int detid = (isdet == OUT_MIN) ? -1 : (int)finddetector(c, &s->p);
    if (detid) {
        unsigned int slot = X->detcount++;
        if (slot < X->detcap) {
            unsigned int i, base;
            if (c->issaveseed) {
                X->dseed[slot * 2] = s->photonseed[0];
                X->dseed[slot * 2 + 1] = s->photonseed[1];
            }
            if (X->detw) {
                X->detw[slot * 2] = s->p.w;
                X->detw[slot * 2 + 1] = s->f.y;
            }
            base = slot * c->reclen;
            if (SAVE_DETID(c->savedetflag)) {
                if (c->extrasrclen && (c->srcid <= 0)) {
                    detid |= (((int)s->ppath[c->w0offset - 1]) << 16);
                }
                X->detp[base++] = (float)detid;
            }
            for (i = 0; i < c->partialdata; i++) {
                X->detp[base++] = s->ppath[i];
            }
            if (SAVE_PEXIT(c->savedetflag)) {
                X->detp[base++] = s->p.x;
                X->detp[base++] = s->p.y;
                X->detp[base++] = s->p.z;
            }
            if (SAVE_VEXIT(c->savedetflag)) {
                X->detp[base++] = s->v.x;
                X->detp[base++] = s->v.y;
                X->detp[base++] = s->v.z;
            }
            if (SAVE_W0(c->savedetflag)) {
                X->detp[base++] = s->ppath[c->w0offset - 2];
            }
            if (SAVE_IQUV(c->savedetflag)) {
                X->detp[base++] = s->st.x;
                X->detp[base++] = s->st.y;
                X->detp[base++] = s->st.z;
                X->detp[base++] = s->st.w;
            }
        } else if (c->savedet == FILL_MAXDET) {
            X->detcount--;
        }
    }
}

static inline void set_launch_voxel(const ocfg* c, ostate* s) {
    s->idx1d = (uint32_t)((int)(floorf(s->p.z)) * (int)c->dimlen[1] + (int)(floorf(s->p.y)) * (int)c->dimlen[0] +
                          (int)(floorf(s->p.x)));
    if (s->p.x < 0.f || s->p.y < 0.f || s->p.z < 0.f || s->p.x >= c->maxidx.x || s->p.y >= c->maxidx.y ||
            s->p.z >= c->maxidx.z) {
        s->mediaid = 0;
    } else {
        s->mediaid = c->media[s->idx1d];
    }
}

/*
 * launchnewphoton, mcx_core.cl:1463-2275: close the current photon
 * (escaped weight, saved reflectance, detection) and launch the next one.
 * Returns 0 on launch, 1 when this thread's quota is done, -1 on failure.
 */
/* savedebugdata (mcx_core.cl:929-948): one trajectory record at a slot taken
   from a shared counter; the photon id is the thread's launch counter plus
   the thread's photon offset, which the close record (1501) computes with
   min(tid, oddphoton) and the launch and scattering records (2247, 2630)
   with min(tid, (tid < oddphoton) tid) */
static void save_traj(octx* X, const ostate* s, int closing) {
    const ocfg* c = X->c;
    const int tid = (int)X->tid, odd = c->oddphoton;
    const int off = closing ? (tid < odd ? tid : odd) : (tid < (tid < odd) * tid ? tid : (tid < odd) * tid);
    const uint32_t id = (uint32_t)s->f.w + (uint32_t)(tid * (int)c->threadphoton) + (uint32_t)off;
    unsigned int pos;
#pragma omp atomic capture
    pos = (*c->ntraj)++;
    if (pos < c->maxtraj) {
        float* r = c->traj + (size_t)pos * 6;
        memcpy(r, &id, sizeof(id));
        r[1] = s->p.x;
        r[2] = s->p.y;
        r[3] = s->p.z;
        r[4] = s->p.w;
        r[5] = (float)(int)s->ppath[c->w0offset - 1];
    }
}

static int launchnewphoton(octx* X, ostate* s, uint32_t isdet) {
    const ocfg* c = X->c;
    const osrc* ls = &c->src;
    float* pp;
    unsigned int attempts = 0;

    s->w0 = 1.f;
    s->Lmove = -1.f;

    if (c->savedet == FILL_MAXDET && X->detcount >= c->maxdetphoton) {
        return 1;
    }

    if (fabsf(s->p.w) >= 0.f) {
        s->ppath[c->partialdata] += s->p.w;
        if (c->debugmove) {
            save_traj(X, s, 1);
        }
        if (s->mediaid == 0 && s->idx1d != OUT_MIN && s->idx1d != OUT_MAX && c->issaveref && s->p.w > 0.f) {
            if (c->issaveref == 1) {
                int tshift = (int)floorf((s->f.y - c->twin0) * c->Rtstep);
                if ((int)c->maxgate - 1 < tshift) {
                    tshift = (int)c->maxgate - 1;
                }
                if (c->extrasrclen && (c->srcid < 0)) {
                    tshift += ((int)s->ppath[c->w0offset - 1] - 1) * (int)c->maxgate;
                }
                share_add(X, s, (size_t)s->idx1d + (size_t)tshift * c->dimlen[2], -s->p.w);
            }
        }
        if ((isdet & DET_MASK) == DET_MASK &&
                (s->mediaid == 0 || (c->mediaformat == MEDIA_2LABEL_SPLIT && SV_CURLABEL(s->sv) == 0)) &&
                c->issaveref < 2) {
            savedetphoton(X, s, isdet);
        }
    }

    memset(s->ppath, 0, sizeof(float) * c->partialdata);

    if (s->f.w >= (float)(c->threadphoton + (X->tid < (unsigned int)c->oddphoton))) {
        return 1;
    }

    if (c->replay) {
        /* the saved launch state of this photon, mcx_core.cl:1590-1596 */
        long long k = replay_index(c, X->tid, (long long)((int)s->f.w > 0 ? (int)s->f.w : 0));
        if (k < 0 || k >= (long long)c->nreplay) {
            X->nfailed++;
            return 1;
        }
        s->t[0] = c->rseed[2 * k];
        s->t[1] = c->rseed[2 * k + 1];
    }

    if (c->issaveseed) {
        s->photonseed[0] = s->t[0];
        s->photonseed[1] = s->t[1];
    }

    if (c->extrasrclen && (c->srcid != 1)) {
        const osrc* extra = (const osrc*)(c->gprop + c->maxmedia + 1);
        if (c->srcid > 1) {
            ls = extra + (c->srcid - 2);
        } else {
            s->ppath[c->w0offset - 1] = (float)((int)(rng_next(s->t) * K_JUST_BELOW_ONE * (float)(c->extrasrclen + 1)) + 1);
            if ((int)s->ppath[c->w0offset - 1] > 1) {
                ls = extra + ((int)(s->ppath[c->w0offset - 1] - 2));
            }
        }
    }

    if (c->replay && c->srcid >= 1) {
        /* keeps the stream in step with a run that picked a source, 1614-1616 */
        rng_next(s->t);
    }

    pp = s->ppath + c->partialdata;

    for (;;) {
        if (++attempts > LAUNCH_ATTEMPT_CAP) {
            return -1;
        }
        s->p = ls->pos;
        if (c->mediaformat == MEDIA_2LABEL_SPLIT) {
            s->sv = 0;        /* 1640-1642 */
        }
        s->v = ls->dir;
        s->f.x = 0.f;
        s->f.y = 0.f;
        s->f.z = c->minaccumtime;
        s->idx1d = f2bits(ls->p2.z);
        s->mediaid = f2bits(ls->p2.w);
        if (c->maxpol > 0) {
            s->st = c->s0;    /* 1633-1638 */
        }
        s->prop.x = ls->pos.x;
        s->prop.y = ls->pos.y;
        s->prop.z = ls->pos.z;
        s->prop.w = 0.f;

        switch (c->srctype) {
            case S_PENCIL:
                break;
            case S_PLANAR:
            case S_PATTERN:
            case S_PATTERN3D:
            case S_FOURIER:
            case S_PENCILARRAY: {
                /* mcx_core.cl:1662-1762 */
                float rx = rng_next(s->t);
                float ry = rng_next(s->t);
                float rz = 0.f;
                if (c->srctype == S_PATTERN3D) {
                    rz = rng_next(s->t);
                    s->p.x = s->p.x + rx * ls->p1.x;
                    s->p.y = s->p.y + ry * ls->p1.y;
                    s->p.z = s->p.z + rz * ls->p1.z;
                } else {
                    s->p.x = s->p.x + rx * ls->p1.x + ry * ls->p2.x;
                    s->p.y = s->p.y + rx * ls->p1.y + ry * ls->p2.y;
                    s->p.z = s->p.z + rx * ls->p1.z + ry * ls->p2.z;
                }
                if (c->srctype == S_PATTERN || c->srctype == S_PATTERN3D) {
                    int pix;
                    if (c->srctype == S_PATTERN) {
                        pix = (int)(ry * K_JUST_BELOW_ONE * ls->p2.w) * (int)(ls->p1.w) + (int)(rx * K_JUST_BELOW_ONE * ls->p1.w);
                    } else {
                        pix = (int)(rz * K_JUST_BELOW_ONE * ls->p1.z) * (int)(ls->p1.y) * (int)(ls->p1.x) +
                              (int)(ry * K_JUST_BELOW_ONE * ls->p1.y) * (int)(ls->p1.x) + (int)(rx * K_JUST_BELOW_ONE * ls->p1.x);
                    }
                    if (c->srcnum <= 1) {
                        s->p.w = ls->pos.w * c->srcpattern[pix];
                        pp[4] = s->p.w;
                    } else {
                        /* photon sharing, 1697-1704 / 1718-1726: weight 1, one weight per
                           pattern, the pixel index in the initial-weight slot */
                        unsigned int k;
                        uint32_t upix = (uint32_t)pix;
                        memcpy(&pp[2], &upix, sizeof(upix));
                        for (k = 0; k < c->srcnum; k++) {
                            pp[4 + k] = c->srcpattern[(size_t)pix * c->srcnum + k];
                        }
                        s->p.w = 1.f;
                    }
                } else if (c->srctype == S_FOURIER) {
                    s->p.w = ls->pos.w * (m_cos(c, (floorf(ls->p1.w) * rx + floorf(ls->p2.w) * ry + ls->p1.w - floorf(ls->p1.w)) * K_TWO_PI) *
                                          (1.f - ls->p2.w + floorf(ls->p2.w)) + 1.f) * 0.5f;
                } else if (c->srctype == S_PENCILARRAY) {
                    s->p.x = ls->pos.x + floorf(rx * ls->p1.w) * ls->p1.x / (ls->p1.w - 1.f) + floorf(ry * ls->p2.w) * ls->p2.x / (ls->p2.w - 1.f);
                    s->p.y = ls->pos.y + floorf(rx * ls->p1.w) * ls->p1.y / (ls->p1.w - 1.f) + floorf(ry * ls->p2.w) * ls->p2.y / (ls->p2.w - 1.f);
                    s->p.z = ls->pos.z + floorf(rx * ls->p1.w) * ls->p1.z / (ls->p1.w - 1.f) + floorf(ry * ls->p2.w) * ls->p2.z / (ls->p2.w - 1.f);
                }
                set_launch_voxel(c, s);
                s->prop.x = s->prop.x + (ls->p1.x + ls->p2.x) * 0.5f;
                s->prop.y = s->prop.y + (ls->p1.y + ls->p2.y) * 0.5f;
                s->prop.z = s->prop.z + (ls->p1.z + ls->p2.z) * 0.5f;
                s->prop.w = 0.f;
                break;
            }
            case S_FOURIERX:
            case S_FOURIERX2D: {
                /* mcx_core.cl:1771-1813 */
                float rx = rng_next(s->t);
                float ry = rng_next(s->t);
                f4 v2 = ls->p1;
                v2.w *= m_rsqrt(ls->p1.x * ls->p1.x + ls->p1.y * ls->p1.y + ls->p1.z * ls->p1.z);
                v2.x = v2.w * (ls->dir.y * ls->p1.z - ls->dir.z * ls->p1.y);
                v2.y = v2.w * (ls->dir.z * ls->p1.x - ls->dir.x * ls->p1.z);
                v2.z = v2.w * (ls->dir.x * ls->p1.y - ls->dir.y * ls->p1.x);
                s->p.x = s->p.x + rx * ls->p1.x + ry * v2.x;
                s->p.y = s->p.y + rx * ls->p1.y + ry * v2.y;
                s->p.z = s->p.z + rx * ls->p1.z + ry * v2.z;
                if (c->srctype == S_FOURIERX2D) {
                    s->p.w = ls->pos.w * (m_sin(c, (ls->p2.x * rx + ls->p2.z) * K_TWO_PI) * m_sin(c, (ls->p2.y * ry + ls->p2.w) * K_TWO_PI) + 1.f) * 0.5f;
                } else {
                    s->p.w = ls->pos.w * (m_cos(c, (ls->p2.x * rx + ls->p2.y * ry + ls->p2.z) * K_TWO_PI) * (1.f - ls->p2.w) + 1.f) * 0.5f;
                }
                set_launch_voxel(c, s);
                s->prop.x = s->prop.x + (ls->p1.x + v2.x) * 0.5f;
                s->prop.y = s->prop.y + (ls->p1.y + v2.y) * 0.5f;
                s->prop.z = s->prop.z + (ls->p1.z + v2.z) * 0.5f;
                s->prop.w = 0.f;
                break;
            }
            case S_HYPERBOLOID: {
                /* mcx_core.cl:1821-1852 */
                float sphi, cphi, r;
                r = K_TWO_PI * rng_next(s->t);
                m_sincos(c, r, &sphi, &cphi);
                r = sqrtf(0.5f * rng_scatlen(c, s->t)) * ls->p1.x;
                s->prop.x = -ls->p1.y / ls->p1.z;
                s->prop.y = m_rsqrt(r * r + ls->p1.z * ls->p1.z);
                s->p.x = r * (cphi - s->prop.x * sphi);
                s->p.y = r * (sphi + s->prop.x * cphi);
                s->p.z = 0.f;
                {
                    f4 np;
                    np.x = -r * sphi * s->prop.y;
                    np.y = r * cphi * s->prop.y;
                    np.z = ls->p1.z * s->prop.y;
                    np.w = 0.f;
                    s->prop = np;
                }
                if (s->v.z > -1.f + K_EPS && s->v.z < 1.f - K_EPS) {
                    float st;
                    f4 np, nv;
                    r = 1.f - s->v.z * s->v.z;
                    st = sqrtf(r);
                    r = m_rsqrt(r);
                    cphi = s->v.x * r;
                    sphi = s->v.y * r;
                    np.x = s->p.x * cphi * s->v.z - s->p.y * sphi;
                    np.y = s->p.x * sphi * s->v.z + s->p.y * cphi;
                    np.z = -s->p.x * st;
                    np.w = s->p.w;
                    s->p = np;
                    nv.x = s->prop.x * cphi * s->v.z - s->prop.y * sphi + s->prop.z * cphi * st;
                    nv.y = s->prop.x * sphi * s->v.z + s->prop.y * cphi + s->prop.z * sphi * st;
                    nv.z = -s->prop.x * st + s->prop.z * s->v.z;
                    nv.w = s->v.w;
                    s->v = nv;
                } else {
                    f4 nv;
                    nv.x = s->prop.x;
                    nv.y = s->prop.y;
                    nv.z = (s->v.z > 0.f) ? s->prop.z : -s->prop.z;
                    nv.w = s->v.w;
                    s->v = nv;
                }
                s->p.x = s->p.x + ls->pos.x;
                s->p.y = s->p.y + ls->pos.y;
                s->p.z = s->p.z + ls->pos.z;
                s->prop.x = ls->pos.x;
                s->prop.y = ls->pos.y;
                s->prop.z = ls->pos.z;
                s->prop.w = 0.f;
                s->Lmove = 0.f;
                break;
            }
            case S_DISK:
            case S_GAUSSIAN:
            case S_RING: {
                /* mcx_core.cl:1861-1935 */
                float sphi, cphi, phi, r;
                if (c->srctype == S_DISK || c->srctype == S_RING) {
                    if (ls->p1.z > 0.f || ls->p1.w > 0.f) {
                        phi = fabsf(ls->p1.z - ls->p1.w) * rng_next(s->t) + fminf(ls->p1.z, ls->p1.w);
                    } else {
                        phi = K_TWO_PI * rng_next(s->t);
                    }
                } else {
                    phi = K_TWO_PI * rng_next(s->t);
                }
                m_sincos(c, phi, &sphi, &cphi);
                if (c->srctype == S_DISK || c->srctype == S_RING) {
                    r = sqrtf(rng_next(s->t) * fabsf(ls->p1.x * ls->p1.x - ls->p1.y * ls->p1.y) + ls->p1.y * ls->p1.y);
                } else {
                    if (fabsf(ls->dir.w) < 1e-5f || fabsf(ls->p1.y) < 1e-5f) {
                        r = sqrtf(-0.5f * m_log(c, rng_next(s->t))) * ls->p1.x;
                    } else {
                        r = ls->p1.x * ls->p1.x * K_ONE_PI / ls->p1.y;
                        r = sqrtf(-0.5f * m_log(c, rng_next(s->t)) * (1.f + (ls->dir.w * ls->dir.w / (r * r)))) * ls->p1.x;
                    }
                }
                if (s->v.z > -1.f + K_EPS && s->v.z < 1.f - K_EPS) {
                    float tmp0 = 1.f - s->v.z * s->v.z;
                    float tmp1 = r * m_rsqrt(tmp0);
                    s->p.x = s->p.x + tmp1 * (s->v.x * s->v.z * cphi - s->v.y * sphi);
                    s->p.y = s->p.y + tmp1 * (s->v.y * s->v.z * cphi + s->v.x * sphi);
                    s->p.z = s->p.z - tmp1 * tmp0 * cphi;
                } else {
                    s->p.x += r * cphi;
                    s->p.y += r * sphi;
                }
                set_launch_voxel(c, s);
                break;
            }
            case S_CONE:
            case S_ISOTROPIC:
            case S_ARCSINE: {
                /* mcx_core.cl:1944-1979 */
                float ang, st, ct, sphi, cphi;
                ang = K_TWO_PI * rng_next(s->t);
                m_sincos(c, ang, &sphi, &cphi);
                if (c->srctype == S_CONE) {
                    unsigned int tries = 0;
                    do {
                        ang = (ls->p1.y > 0) ? K_TWO_PI * rng_next(s->t) : m_acos(c, 2.f * rng_next(s->t) - 1.f);
                    } while (ang > ls->p1.x && ++tries < CONE_DRAW_CAP);
                } else if (c->srctype == S_ISOTROPIC || c->variant == MCXO_VARIANT_NVCC) {
                    ang = m_acos(c, 2.f * rng_next(s->t) - 1.f);
                } else {
                    ang = K_ONE_PI * rng_next(s->t);
                }
                m_sincos(c, ang, &st, &ct);
                rotatevector(c, &s->v, st, ct, sphi, cphi);
                s->Lmove = 0.f;
                break;
            }
            case S_ZGAUSSIAN: {
                /* mcx_core.cl:1987-1995 */
                float ang, st, ct, sphi, cphi;
                ang = K_TWO_PI * rng_next(s->t);
                m_sincos(c, ang, &sphi, &cphi);
                ang = sqrtf(-2.f * m_log(c, rng_next(s->t))) * (1.f - 2.f * rng_next(s->t)) * ls->p1.x;
                m_sincos(c, ang, &st, &ct);
                rotatevector(c, &s->v, st, ct, sphi, cphi);
                s->Lmove = 0.f;
                break;
            }
            case S_LINE:
            case S_SLIT: {
                /* mcx_core.cl:2003-2083 */
                float r_l = rng_next(s->t);
                s->p.x = s->p.x + r_l * ls->p1.x;
                s->p.y = s->p.y + r_l * ls->p1.y;
                s->p.z = s->p.z + r_l * ls->p1.z;
                if (c->srctype == S_LINE) {
                    float sphi_l, cphi_l;
                    r_l = m_rsqrt(ls->p1.x * ls->p1.x + ls->p1.y * ls->p1.y + ls->p1.z * ls->p1.z);
                    if (ls->p2.x > 0.f) {
                        float lx = ls->p1.x * r_l, ly = ls->p1.y * r_l, lz = ls->p1.z * r_l;
                        float vd = s->v.x * lx + s->v.y * ly + s->v.z * lz;
                        float vn;
                        s->v.x = s->v.x - vd * lx;
                        s->v.y = s->v.y - vd * ly;
                        s->v.z = s->v.z - vd * lz;
                        vn = m_rsqrt(s->v.x * s->v.x + s->v.y * s->v.y + s->v.z * s->v.z);
                        s->v.x = s->v.x * vn;
                        s->v.y = s->v.y * vn;
                        s->v.z = s->v.z * vn;
                        r_l = ls->p2.x * (2.f * rng_next(s->t) - 1.f);
                        m_sincos(c, r_l, &sphi_l, &cphi_l);
                        rotate_perp(&s->v, lx, ly, lz, sphi_l, cphi_l);
                    } else {
                        s->v.x = ls->p1.x * r_l;
                        s->v.y = ls->p1.y * r_l;
                        s->v.z = ls->p1.z * r_l;
                        r_l = K_TWO_PI * rng_next(s->t);
                        m_sincos(c, r_l, &sphi_l, &cphi_l);
                        rotatevector(c, &s->v, 1.f, 0.f, sphi_l, cphi_l);
                    }
                    s->Lmove = 0.f;
                } else {
                    if (ls->p2.x > 0.f || ls->p2.y > 0.f) {
                        float sphi_s, cphi_s;
                        r_l = K_TWO_PI * rng_next(s->t);
                        m_sincos(c, r_l, &sphi_s, &cphi_s);
                        r_l = sqrtf(2.f * rng_scatlen(c, s->t));
                        cphi_s *= ls->p2.x * r_l;
                        sphi_s *= ls->p2.y * r_l;
                        sphi_s *= m_rsqrt(ls->p1.x * ls->p1.x + ls->p1.y * ls->p1.y + ls->p1.z * ls->p1.z);
                        s->prop.x = ls->p1.y * s->v.z - ls->p1.z * s->v.y;
                        s->prop.y = ls->p1.z * s->v.x - ls->p1.x * s->v.z;
                        s->prop.z = ls->p1.x * s->v.y - ls->p1.y * s->v.x;
                        s->prop.w = 0.f;
                        cphi_s *= m_rsqrt(s->prop.x * s->prop.x + s->prop.y * s->prop.y + s->prop.z * s->prop.z);
                        s->v.x += cphi_s * s->prop.x + sphi_s * ls->p1.x;
                        s->v.y += cphi_s * s->prop.y + sphi_s * ls->p1.y;
                        s->v.z += cphi_s * s->prop.z + sphi_s * ls->p1.z;
                        r_l = m_rsqrt(s->v.x * s->v.x + s->v.y * s->v.y + s->v.z * s->v.z);
                        s->v.x *= r_l;
                        s->v.y *= r_l;
                        s->v.z *= r_l;
                    }
                    s->Lmove = -1.f;
                }
                set_launch_voxel(c, s);
                s->prop.x = ls->pos.x + (ls->p1.x) * 0.5f;
                s->prop.y = ls->pos.y + (ls->p1.y) * 0.5f;
                s->prop.z = ls->pos.z + (ls->p1.z) * 0.5f;
                s->prop.w = 0.f;
                s->Lmove = -1.f;
                break;
            }
            default:
                break;
        }

        if (fabsf(s->p.w) <= c->minenergy) {
            continue;       /* the reference's `continue` re-tests the loop condition, which fails again */
        }

        if (c->nangle) {
            /* launch-angle inverse CDF, mcx_core.cl:2102-2124 */
            float ang, st, ct, sphi, cphi;
            if (ls->dir.w > 0.f) {
                ang = fminf(rng_next(s->t) * (float)c->nangle, (float)c->nangle - K_EPS);
                cphi = c->angleinvcdf[(int)(ang)];
            } else {
                unsigned int a0, a1;
                ang = fminf(rng_next(s->t) * (float)(c->nangle - 1), (float)(c->nangle - 1) - K_EPS);
                sphi = ang - (float)((int)ang);
                a0 = ((unsigned int)ang >= c->nangle - 1 ? c->nangle - 1 : (unsigned int)(int)(ang));
                a1 = ((unsigned int)ang + 1 >= c->nangle - 1 ? c->nangle - 1 : (unsigned int)((int)(ang) + 1));
                cphi = ((1.f - sphi) * c->angleinvcdf[a0] + sphi * c->angleinvcdf[a1]);
            }
            cphi *= K_ONE_PI;
            m_sincos(c, cphi, &st, &ct);
            ang = K_TWO_PI * rng_next(s->t);
            m_sincos(c, ang, &sphi, &cphi);
            if (ls->dir.w < 1.5f && ls->dir.w >= 0.f) {
                s->v = ls->dir;
            }
            rotatevector(c, &s->v, st, ct, sphi, cphi);
        } else if (s->Lmove < 0.f) {
            /* focus / divergence, mcx_core.cl:2125-2153 */
            if (isnan(ls->dir.w)) {
                float ang, st, ct, sphi, cphi;
                ang = K_TWO_PI * rng_next(s->t);
                m_sincos(c, ang, &sphi, &cphi);
                ang = m_acos(c, 2.f * rng_next(s->t) - 1.f);
                m_sincos(c, ang, &st, &ct);
                rotatevector(c, &s->v, st, ct, sphi, cphi);
            } else if (ls->dir.w < 0.f && isinf(ls->dir.w)) {
                float ang, st, ct, sphi, cphi;
                ang = K_TWO_PI * rng_next(s->t);
                m_sincos(c, ang, &sphi, &cphi);
                st = sqrtf(rng_next(s->t));
                ct = sqrtf(1.f - st * st);
                rotatevector(c, &s->v, st, ct, sphi, cphi);
            } else if (ls->dir.w != 0.f) {
                float Rn2 = (float)((ls->dir.w > 0.f) - (ls->dir.w < 0.f));
                s->prop.x += ls->dir.w * s->v.x;
                s->prop.y += ls->dir.w * s->v.y;
                s->prop.z += ls->dir.w * s->v.z;
                s->v.x = Rn2 * (s->prop.x - s->p.x);
                s->v.y = Rn2 * (s->prop.y - s->p.y);
                s->v.z = Rn2 * (s->prop.z - s->p.z);
                Rn2 = m_rsqrt(s->v.x * s->v.x + s->v.y * s->v.y + s->v.z * s->v.z);
                s->v.x *= Rn2;
                s->v.y *= Rn2;
                s->v.z *= Rn2;
            }
        }

        if ((s->mediaid & MED_MASK) == 0) {
            int idx = skipvoid(c, &s->p, &s->v, &s->f, s->fid);
            if (idx >= 0) {
                s->idx1d = (uint32_t)idx;
                s->mediaid = c->media[s->idx1d];
            }
        }
        s->fid[0] = (short)floorf(s->p.x);
        s->fid[1] = (short)floorf(s->p.y);
        s->fid[2] = (short)floorf(s->p.z);

        s->w0 += 1.f;
        if (s->w0 > (float)c->maxvoidstep) {
            X->nfailed++;
            return -1;
        }
        if (!((s->mediaid & MED_MASK) == 0 || fabsf(s->p.w) <= c->minenergy)) {
            break;
        }
    }

    s->f.w += 1.f;
    s->prop = c->gprop[1];
    if (c->mediaformat == MEDIA_2LABEL_SPLIT) {
        updateprop_svmc(c, &s->prop, s->mediaid, s->idx1d, &s->p, s, s->fid);
    } else {
        updateprop(c, &s->prop, s->mediaid);
    }
    if (c->debugmove) {
        save_traj(X, s, 0);      /* 2243-2249: the source slot is the launched photon's */
    }
    pp[1] += s->p.w;
    s->w0 = s->p.w;
    pp[2] = ((c->srcnum > 1) ? pp[2] : s->p.w);
    s->v.w = K_EPS;
    s->Lmove = 0.f;
    if (c->rfmode == 1) {
        /* the complex weight restarts with every launch (2427-2430, 3011, 3054, ...) */
        s->wre = s->w0re = s->p.w;
        s->wim = s->w0im = 0.f;
    } else if (c->rfmode == 2) {
        /* rf replay (2257-2262): the phase of the detected time of flight, read
           with the launch counter itself (the next photon, as the scattering
           sites do); the last photon reads the arrays' start-time pad.  The
           reference stores it through the partial-data-shifted pointer of its
           launch (1621), partialdata floats past the slots its deposits read,
           which therefore stay zero: the float (reference-faithful) mode
           reproduces that, the FP64 mode stores where the deposits read. */
        long long k = replay_index(c, X->tid, (long long)(int)s->f.w - (c->replaysiteown ? 1 : 0));
        float tof = (k >= 0 && k < (long long)c->nreplay) ? c->rtof[k] : c->twin0;
        float rs, rc;
        float* slot = s->ppath + c->w0offset + c->srcnum + (c->fieldmode == MCXO_FIELD_FLOAT_SPILL ? c->partialdata : 0);
        m_sincos(c, c->omega * tof, &rs, &rc);
        slot[0] = rc;
        slot[1] = rs;
    }
    X->nlaunch++;
    return 0;
}

/* relaunch after an exit: a detecting face marks the photon OUTSIDE_VOLUME_MIN
   (mcx_core.cl:3001, 3181) */
static inline uint32_t exit_detflag(const ocfg* c, const ostate* s, uint32_t mediaidold) {
    return (((s->idx1d == OUT_MAX && c->bc[9 + s->fid[3]]) || (s->idx1d == OUT_MIN && c->bc[6 + s->fid[3]]))
            ? OUT_MIN : (mediaidold & DET_MASK));
}

/* one reference thread: mcx_main_loop, mcx_core.cl:2307-3307 */
static void run_thread(octx* X, const uint32_t* seedwords, float* energy, unsigned int tid) {
    const ocfg* c = X->c;
    ostate s;
    uint32_t idx1dold, mediaidold = 0;
    float ppbuf[4096];
    const int svmc = (c->mediaformat == MEDIA_2LABEL_SPLIT);
    int testint = 0, hitintf = 0;      /* split voxels: test the plane this step / the step ended on it */
    memset(&s, 0, sizeof(s));
    s.p.w = NAN;
    s.mediaid = f2bits(c->src.p2.w);
    s.fid[3] = -1;
    s.ppath = ppbuf;
    memset(ppbuf, 0, sizeof(float) * (c->w0offset + c->srcnum + 2));
    X->tid = tid;

    if ((unsigned long long)tid >= (unsigned long long)c->threadphoton * c->nthread + (unsigned int)c->oddphoton) {
        return;
    }
    s.ppath[c->partialdata] = energy[tid * 2];
    s.ppath[c->partialdata + 1] = energy[tid * 2 + 1];
    s.t[0] = (uint64_t)seedwords[tid * 4] << 32 | seedwords[tid * 4 + 1];
    s.t[1] = (uint64_t)seedwords[tid * 4 + 2] << 32 | seedwords[tid * 4 + 3];

    if (launchnewphoton(X, &s, 0)) {
        return;
    }
    s.isdet = s.mediaid & DET_MASK;
    s.mediaid &= MED_MASK;

    while (s.f.w <= (float)(c->threadphoton + (tid < (unsigned int)c->oddphoton))) {
        X->nstep++;
        if (s.f.x <= 0.f) {
            s.f.x = rng_scatlen(c, s.t);
            if (s.v.w != K_EPS) {
                /* scattering, mcx_core.cl:2450-2560 */
                float cphi = 1.f, sphi = 0.f, theta, stheta, ctheta, tmp0 = 0.f;
                X->nscatter++;
                if (c->maxpol > 0 && !c->is2d) {
                    /* polarised angles by rejection against the Mueller matrix, 2454-2469 */
                    const uint32_t ipol = K_NANGLES * ((s.mediaid & MED_MASK) - 1);
                    float i0, i1, sin2phi, cos2phi;
                    do {
                        uint32_t ith;
                        theta = m_acos(c, 2.f * rng_next(s.t) - 1.f);
                        tmp0 = K_TWO_PI * rng_next(s.t);
                        m_sincos(c, 2.f * tmp0, &sin2phi, &cos2phi);
                        i0 = c->smatrix[ipol].x * s.st.x + c->smatrix[ipol].y * (s.st.y * cos2phi + s.st.z * sin2phi);
                        ith = (uint32_t)(theta * K_NANGLES * (K_R_PI - K_EPS));
                        i1 = c->smatrix[ipol + ith].x * s.st.x + c->smatrix[ipol + ith].y * (s.st.y * cos2phi + s.st.z * sin2phi);
                    } while (rng_next(s.t) * i0 >= i1);
                    m_sincos(c, tmp0, &sphi, &cphi);
                    m_sincos(c, theta, &stheta, &ctheta);
                } else {
                if (!c->is2d) {
                    tmp0 = K_TWO_PI * rng_next(s.t);
                    m_sincos(c, tmp0, &sphi, &cphi);
                }
                if (c->nphase > 2) {
                    unsigned int i0, i1;
                    tmp0 = rng_next(s.t) * (float)(c->nphase - 1);
                    theta = tmp0 - (float)((int)tmp0);
                    i0 = (unsigned int)tmp0 >= c->nphase ? c->nphase - 1 : (unsigned int)(int)(tmp0);
                    i1 = (unsigned int)tmp0 + 1 >= c->nphase ? c->nphase - 1 : (unsigned int)((int)(tmp0) + 1);
                    tmp0 = (1.f - theta) * c->invcdf[i0] + theta * c->invcdf[i1];
                    theta = m_acos(c, tmp0);
                    stheta = m_sin(c, theta);
                    ctheta = tmp0;
                } else {
                    tmp0 = (s.v.w > (float)c->gscatter) ? 0.f : s.prop.z;
                    if (fabsf(tmp0) > K_EPS) {
                        tmp0 = (1.f - s.prop.z * s.prop.z) / (1.f - s.prop.z + 2.f * s.prop.z * rng_next(s.t));
                        tmp0 *= tmp0;
                        tmp0 = (1.f + s.prop.z * s.prop.z - tmp0) / (2.f * s.prop.z);
                        tmp0 = fmaxf(-1.f, fminf(1.f, tmp0));
                        theta = m_acos(c, tmp0);
                        stheta = m_sin(c, theta);
                        ctheta = tmp0;
                    } else {
                        theta = m_acos(c, 2.f * rng_next(s.t) - 1.f);
                        m_sincos(c, theta, &stheta, &ctheta);
                    }
                }
                }
                /* per-medium slots exist for labels 1..maxmedia; the reference indexes
                   outside them for label 0 and for label-half words */
                {
                    /* split voxels record under the label of the photon's side (2507-2535) */
                    const uint32_t lab = svmc ? SV_CURLABEL(s.sv) : (s.mediaid & MED_MASK);
                    if (SAVE_NSCAT(c->savedetflag) && lab - 1u < c->maxmedia) {
                        uint32_t n = f2bits(s.ppath[lab - 1]) + 1u;
                        s.ppath[lab - 1] = bits2f(n);
                    }
                    if (SAVE_MOM(c->savedetflag) && lab - 1u < c->maxmedia) {
                        s.ppath[c->maxmedia * (SAVE_NSCAT(c->savedetflag) + SAVE_PPATH(c->savedetflag)) + lab - 1] += 1.f - ctheta;
                    }
                }
                {
                    const f4 olddir = s.v;
                    if (c->is2d) {
                        rotatevector2d(&s.v, (rng_next(s.t) > 0.5f ? stheta : -stheta), ctheta, c->is2d);
                    } else {
                        rotatevector(c, &s.v, stheta, ctheta, sphi, cphi);
                    }
                    s.v.w += 1.f;
                    if (c->maxpol > 0) {
                        update_stokes(c, &s, theta, tmp0, &olddir, &s.v);
                    }
                }
                if (c->replay && (c->outputtype == otWP || c->outputtype == otDCS || c->outputtype == otWPTOF ||
                                  c->outputtype == otRFmus)) {
                    /* replay deposit at the scattering site, mcx_core.cl:2567-2604; the
                       reference indexes these with the launch counter itself (no -1) */
                    long long k = replay_index(c, tid, (long long)(int)s.f.w - (c->replaysiteown ? 1 : 0));
                    if (k >= 0 && k < (long long)c->nreplay) {
                        int tshift;
                        float tim = 0.f;
                        tmp0 = (c->outputtype == otDCS) ? (1.f - ctheta) : 1.f;
                        if (c->outputtype == otRFmus) {
                            tmp0 = c->rweight[k] * s.ppath[c->w0offset + c->srcnum];
                            tim = c->rweight[k] * s.ppath[c->w0offset + c->srcnum + 1];
                        } else if (c->outputtype == otWPTOF) {
                            tmp0 = c->rtof[k];
                            tmp0 *= c->rweight[k];
                        } else {
                            tmp0 *= c->rweight[k];
                        }
                        tshift = (int)(floorf((c->rtof[k] - c->twin0) * c->Rtstep)) +
                                 ((c->replaydet == -1) ? (((c->rdetid[k] & 0xFFFF) - 1) * (int)c->maxgate) : 0);
                        if (c->extrasrclen && (c->srcid < 0)) {
                            tshift += ((int)s.ppath[c->w0offset - 1] - 1) * ((c->replaydet == -1) ? (int)c->detnum : 1) * (int)c->maxgate;
                        }
                        tshift = ((int)c->maxgate - 1 < tshift) ? (int)c->maxgate - 1 : tshift;
                        field_add_site(X, (size_t)s.idx1d + (size_t)(long long)tshift * c->dimlen[2], tmp0);
                        if (c->outputtype == otRFmus) {
                            field_add_im(X, (size_t)s.idx1d + (size_t)(long long)tshift * c->dimlen[2], tim, 1);
                        }
                    }
                }
                if (c->debugmove) {
                    save_traj(X, &s, 0);      /* 2625-2634: scattering sites, not the first draw */
                }
            }
            s.v.w = (float)(int)s.v.w;
            if (svmc) {
                testint = 1;      /* 2641-2647 */
            }
        }

        s.n1 = s.prop.w;
        if (svmc) {
            updateprop_svmc(c, &s.prop, s.mediaid, s.idx1d, &s.p, &s, s.fid);
        } else {
            updateprop(c, &s.prop, s.mediaid);
        }

        /* advance to the next voxel face or the end of the free path, 2677-2765 */
        s.f.z = hitgrid(c, &s.p, &s.v, s.fid);
        {
            float slen = s.f.z * s.prop.y * (s.v.w + 1.f > (float)c->gscatter ? (1.f - s.prop.z) : 1.f);
            slen = fminf(slen, s.f.x);
            s.f.z = slen / (s.prop.y * (s.v.w + 1.f > (float)c->gscatter ? (1.f - s.prop.z) : 1.f));
            hitintf = 0;
            if (svmc && SV_ISSPLIT(s.sv) && testint) {
                /* the voxel's plane cuts the step short (2687-2702) */
                float tmplen = s.f.z;
                hitintf = ray_plane_intersect(c, &s, &tmplen, &slen);
                s.f.z = tmplen;
            }

            s.pathlen += s.f.z;
            s.p.x = s.p.x + s.f.z * s.v.x;
            s.p.y = s.p.y + s.f.z * s.v.y;
            s.p.z = s.p.z + s.f.z * s.v.z;
            if (s.fid[3] == 0) {
                s.fid[0] += (slen == s.f.x || hitintf) ? 0 : (s.v.x > 0.f ? 1 : -1);
            }
            if (s.fid[3] == 1) {
                s.fid[1] += (slen == s.f.x || hitintf) ? 0 : (s.v.y > 0.f ? 1 : -1);
            }
            if (s.fid[3] == 2) {
                s.fid[2] += (slen == s.f.x || hitintf) ? 0 : (s.v.z > 0.f ? 1 : -1);
            }
            if (c->rfmode == 1) {
                /* RF forward, 2750-2760: w <- w exp(-(mua + i omega n / c0) ds) */
                float att = m_exp(c, -s.prop.x * s.f.z);
                float rs, rc, tre, tim;
                m_sincos(c, c->omega * s.prop.w * c->oneoverc0 * s.f.z, &rs, &rc);
                tre = att * (s.wre * rc + s.wim * rs);
                tim = att * (-s.wre * rs + s.wim * rc);
                s.wre = tre;
                s.wim = tim;
                s.p.w = sqrtf(s.wre * s.wre + s.wim * s.wim);
            } else {
                s.p.w *= m_exp(c, -s.prop.x * s.f.z);
            }
            s.f.x -= slen;
            s.f.y += s.f.z * s.prop.w * c->oneoverc0;
        }
        if (c->savedet && SAVE_PPATH(c->savedetflag) &&
                (svmc ? SV_CURLABEL(s.sv) : (s.mediaid & MED_MASK)) - 1u < c->maxmedia) {
            s.ppath[c->maxmedia * (SAVE_NSCAT(c->savedetflag)) + (svmc ? SV_CURLABEL(s.sv) : (s.mediaid & MED_MASK)) - 1] += s.f.z;
        }

        /* new voxel, 2795-2811 */
        mediaidold = s.mediaid | s.isdet;
        idx1dold = s.idx1d;
        s.idx1d = vox_index(c, s.fid[0], s.fid[1], s.fid[2]);
        if (!inside_u(c, s.fid[0], s.fid[1], s.fid[2])) {
            s.mediaid = 0;
            s.idx1d = (s.fid[0] < 0 || s.fid[1] < 0 || s.fid[2] < 0) ? OUT_MIN : OUT_MAX;
            s.isdet = c->bc[(s.idx1d == OUT_MAX) * 3 + s.fid[3]];
            s.isdet = ((s.isdet & 0xF) == bcUnknown) ? (c->doreflect ? bcReflect : bcAbsorb) : s.isdet;
        } else {
            s.mediaid = c->media[s.idx1d];
            s.isdet = s.mediaid & DET_MASK;
            s.mediaid &= MED_MASK;
        }

        /* deposit on a voxel change (or at a split voxel's plane), 2816-2929 */
        if ((s.idx1d != idx1dold || hitintf) && idx1dold < c->dimlen[2] && mediaidold) {
            if (c->save2pt && s.f.y >= c->twin0 && s.f.y < c->twin1) {
                float weight = 0.f, weight_im = 0.f;
                int tshift = (int)(floorf((s.f.y - c->twin0) * c->Rtstep));
                if (c->rfmode == 1) {
                    /* RF forward, 2833-2840: (w0 - w) / (mua + i omega n / c0) */
                    float dre = s.w0re - s.wre, dim = s.w0im - s.wim;
                    float aim = c->omega * s.prop.w * c->oneoverc0;
                    float am2 = s.prop.x * s.prop.x + aim * aim;
                    weight = (am2 < K_EPS) ? (s.w0re * s.pathlen) : (dre * s.prop.x + dim * aim) / am2;
                    weight_im = (am2 < K_EPS) ? (s.w0im * s.pathlen) : (dim * s.prop.x - dre * aim) / am2;
                } else if (c->outputtype == otEnergy) {
                    weight = s.w0 - s.p.w;
                } else if (c->outputtype == otFluence || c->outputtype == otFlux || c->outputtype >= otAdjoint) {
                    weight = (s.prop.x < K_EPS) ? (s.w0 * s.pathlen) : ((s.w0 - s.p.w) / (s.prop.x));
                } else if (c->replay) {
                    /* replay Jacobian deposit, mcx_core.cl:2845-2858: the detected
                       weight times the path length in the voxel, in the gate of the
                       photon's detected time of flight */
                    if (c->outputtype == otJacobian || c->outputtype == otRF || c->outputtype == otWLTOF) {
                        long long k = replay_index(c, tid, (long long)(int)s.f.w - 1);
                        if (k >= 0 && k < (long long)c->nreplay) {
                            weight = c->rweight[k] * s.pathlen;
                            tshift = (int)(floorf((c->rtof[k] - c->twin0) * c->Rtstep)) +
                                     ((c->replaydet == -1) ? (((c->rdetid[k] & 0xFFFF) - 1) * (int)c->maxgate) : 0);
                            if (c->outputtype == otRF) {
                                /* 2853-2855, 2875-2877: times cos / sin of the launch phase */
                                weight = -weight * s.ppath[c->w0offset + c->srcnum];
                                weight_im = -c->rweight[k] * s.pathlen * s.ppath[c->w0offset + c->srcnum + 1];
                            } else if (c->outputtype == otWLTOF) {
                                weight = weight * c->rtof[k];
                            }
                        }
                    }
                } else if (c->outputtype == otL) {
                    weight = s.w0 * s.pathlen;
                }
                if (c->extrasrclen && (c->srcid < 0)) {
                    tshift += ((int)s.ppath[c->w0offset - 1] - 1) * ((c->replay && c->replaydet == -1) ? (int)c->detnum : 1) *
                              (int)c->maxgate;
                }
                if (c->outputtype == otRF && c->replay) {
                    size_t at = (size_t)idx1dold + (size_t)(long long)tshift * c->dimlen[2];
                    field_add_nospill(X, at, weight);
                    if (c->omega > 0.f) {
                        field_add_im(X, at, weight_im, 0);
                    }
                } else if (fabsf(weight) > 0.f) {
                    int spilled = share_add(X, &s, (size_t)idx1dold + (size_t)(long long)tshift * c->dimlen[2], weight);
                    if (c->rfmode == 1 && !spilled) {
                        /* the reference deposits the imaginary part only when the real
                           accumulator did not spill (its else-branch, 2887) */
                        field_add_im(X, (size_t)idx1dold + (size_t)(long long)tshift * c->dimlen[2], weight_im, 1);
                    }
                }
            }
            s.w0 = s.p.w;
            if (c->rfmode == 1) {
                s.w0re = s.wre;
                s.w0im = s.wim;
            }
            s.pathlen = 0.f;
        } else {
            s.mediaid = mediaidold;
        }
        if (svmc) {
            /* the side of the plane after a voxel change or a plane crossing (2934-2950) */
            if (s.idx1d != idx1dold) {
                updateprop_svmc(c, &s.prop, s.mediaid, s.idx1d, &s.p, &s, s.fid);
                testint = 1;
            } else if (hitintf) {
                s.nv[0] = -s.nv[0], s.nv[1] = -s.nv[1], s.nv[2] = -s.nv[2];
                s.pd = -s.pd;
                s.sv ^= 1u << 17;
                testint = 0;
            }
        }

        /* exit, time-out or cyclic boundary (and a background half of a split voxel), 2958-3028 */
        if ((s.mediaid == 0 && ((s.isdet & 0xF) == bcAbsorb || (s.isdet & 0xF) == bcCyclic ||
                                ((s.isdet & 0xF) == bcReflect && s.n1 == c->gprop[0].w))) ||
                (svmc && ((s.idx1d != idx1dold || hitintf) && !SV_ISUPPER(s.sv) && !SV_LOWER(s.sv) &&
                          (!c->doreflect || s.n1 == c->gprop[0].w))) ||
                s.f.y > c->twin1) {
            if (s.isdet == bcCyclic) {
                if (s.fid[3] == 0) {
                    s.p.x = nextafter_ref(rintf(((s.idx1d == OUT_MIN) ? c->maxidx.x : 0)), (s.v.x > 0.f) - (s.v.x < 0.f));
                    s.fid[0] = (short)floorf(s.p.x);
                }
                if (s.fid[3] == 1) {
                    s.p.y = nextafter_ref(rintf(((s.idx1d == OUT_MIN) ? c->maxidx.y : 0)), (s.v.y > 0.f) - (s.v.y < 0.f));
                    s.fid[1] = (short)floorf(s.p.y);
                }
                if (s.fid[3] == 2) {
                    s.p.z = nextafter_ref(rintf(((s.idx1d == OUT_MIN) ? c->maxidx.z : 0)), (s.v.z > 0.f) - (s.v.z < 0.f));
                    s.fid[2] = (short)floorf(s.p.z);
                }
                if (inside_u(c, s.fid[0], s.fid[1], s.fid[2])) {
                    s.idx1d = vox_index(c, s.fid[0], s.fid[1], s.fid[2]);
                    s.mediaid = c->media[s.idx1d];
                    s.isdet = s.mediaid & DET_MASK;
                    s.mediaid &= MED_MASK;
                    continue;
                }
            }
            if (launchnewphoton(X, &s, exit_detflag(c, &s, mediaidold))) {
                break;
            }
            s.isdet = s.mediaid & DET_MASK;
            s.mediaid &= MED_MASK;
            if (svmc) {
                testint = 1;      /* 3019-3023 */
            }
            continue;
        }

        /* Russian roulette, 3031-3061 */
        if (fabsf(s.p.w) < c->minenergy) {
            if (rng_next(s.t) * K_ROULETTE_SIZE <= 1.f) {
                s.p.w *= K_ROULETTE_SIZE;
                if (c->rfmode == 1) {
                    s.wre *= K_ROULETTE_SIZE;
                    s.wim *= K_ROULETTE_SIZE;
                    s.w0re *= K_ROULETTE_SIZE;
                    s.w0im *= K_ROULETTE_SIZE;
                }
            } else {
                if (launchnewphoton(X, &s, (mediaidold & DET_MASK))) {
                    break;
                }
                s.isdet = s.mediaid & DET_MASK;
                s.mediaid &= MED_MASK;
                continue;
            }
        }

        /* Fresnel at a split voxel's plane (3065-3115, the OpenCL kernel) */
        if (c->dorefl_compiled && svmc && hitintf) {
            if (c->gprop[SV_LOWER(s.sv)].w != c->gprop[SV_UPPER(s.sv)].w) {
                float c0[3];
                s.nv[0] = -s.nv[0], s.nv[1] = -s.nv[1], s.nv[2] = -s.nv[2];
                s.pd = -s.pd;
                c0[0] = s.v.x, c0[1] = s.v.y, c0[2] = s.v.z;
                if (reflectray_svmc(c, s.n1, c0, &s)) {
                    if (launchnewphoton(X, &s, (mediaidold & DET_MASK))) {
                        break;
                    }
                    s.isdet = s.mediaid & DET_MASK;
                    s.mediaid &= MED_MASK;
                    testint = 1;
                    continue;
                }
                s.v.x = c0[0], s.v.y = c0[1], s.v.z = c0[2];
            } else {
                s.prop = c->gprop[SV_CURLABEL(s.sv)];
            }
        } else if (c->dorefl_compiled) {
            /* Fresnel reflection / refraction, 3126-3278; in a split-voxel volume the
               photon's side already holds the properties (the OpenCL kernel's label
               update is empty there) */
            if (!svmc) {
                updateprop(c, &s.prop, s.mediaid);
            }
            if (((s.mediaid && c->doreflect) ||
                 (s.mediaid == 0 && (((s.isdet & 0xF) == bcUnknown && c->doreflect) || ((s.isdet & 0xF) == bcReflect ||
                                                                                         (s.isdet & 0xF) == bcMirror)))) &&
                (((s.isdet & 0xF) == bcMirror) ||
                 s.n1 != ((c->mediaformat < 100) ? (s.prop.w) : (c->gprop[(s.mediaid > 0 && c->mediaformat >= 100) ? 1 : s.mediaid].w)))) {
                float Rtotal = 1.f;
                float cphi, sphi, stheta, ctheta, tmp0, tmp1;
                X->nreflect++;
                if (!svmc) {
                    updateprop(c, &s.prop, s.mediaid);
                }
                tmp0 = s.n1 * s.n1;
                tmp1 = s.prop.w * s.prop.w;
                cphi = fabsf(vcomp(&s.v, s.fid[3]));
                sphi = 1.f - cphi * cphi;
                s.f.z = 1.f - tmp0 / tmp1 * sphi;
                if (s.f.z > 0.f && (s.isdet & 0xF) != bcMirror) {
                    ctheta = tmp0 * cphi * cphi + tmp1 * s.f.z;
                    stheta = 2.f * s.n1 * s.prop.w * cphi * sqrtf(s.f.z);
                    Rtotal = (ctheta - stheta) / (ctheta + stheta);
                    ctheta = tmp1 * cphi * cphi + tmp0 * s.f.z;
                    Rtotal = (Rtotal + (ctheta - stheta) / (ctheta + stheta)) * 0.5f;
                }
                if (Rtotal < 1.f && (!(s.mediaid == 0 && ((s.isdet & 0xF) == bcMirror))) && rng_next(s.t) > Rtotal) {
                    transmit(&s.v, s.n1, s.prop.w, s.fid[3]);
                    if (s.mediaid == 0) {
                        if (launchnewphoton(X, &s, exit_detflag(c, &s, mediaidold))) {
                            break;
                        }
                        s.isdet = s.mediaid & DET_MASK;
                        s.mediaid &= MED_MASK;
                        continue;
                    }
                } else {
                    int fw = s.fid[3];
                    if (fw == 0) {
                        s.v.x = -s.v.x;
                        s.p.x = nextafter_ref(rintf(s.p.x), (int)((float)(s.v.x > 0.f) - 0.5f));
                        s.fid[0] = (short)rintf(s.p.x);
                    } else if (fw == 1) {
                        s.v.y = -s.v.y;
                        s.p.y = nextafter_ref(rintf(s.p.y), (int)((float)(s.v.y > 0.f) - 0.5f));
                        s.fid[1] = (short)rintf(s.p.y);
                    } else {
                        s.v.z = -s.v.z;
                        s.p.z = nextafter_ref(rintf(s.p.z), (int)((float)(s.v.z > 0.f) - 0.5f));
                        s.fid[2] = (short)rintf(s.p.z);
                    }
                    s.idx1d = idx1dold;
                    s.mediaid = (c->media[s.idx1d] & MED_MASK);
                    /* The reference leaves isdet holding the boundary code of the face
                       it just reflected from, which the next step ORs into the medium
                       index (2796) and can turn label 2 into 3.  Both the oracle and
                       the product take the detector bit of the voxel it is back in. */
                    s.isdet = c->media[s.idx1d] & DET_MASK;
                    if (svmc) {
                        /* back in the voxel it came from: its side of the plane (3218-3236);
                           only the CUDA branch tests the plane after the relaunch (3240-3243) */
                        updateprop_svmc(c, &s.prop, s.mediaid, s.idx1d, &s.p, &s, s.fid);
                        if (SV_CURLABEL(s.sv) == 0) {
                            if (launchnewphoton(X, &s, (mediaidold & DET_MASK))) {
                                break;
                            }
                            s.isdet = s.mediaid & DET_MASK;
                            s.mediaid &= MED_MASK;
                            if (c->variant == MCXO_VARIANT_NVCC) {
                                testint = 1;
                            }
                            continue;
                        }
                    } else {
                        updateprop(c, &s.prop, s.mediaid);
                    }
                    s.n1 = s.prop.w;
                }
            }
        }
    }

    energy[tid * 2] = s.ppath[c->partialdata];
    energy[tid * 2 + 1] = s.ppath[c->partialdata + 1];
}

/* ------------------------------------------------------------ host steps */

/* mcx_maskdet, mcx_utils.c:4085-4198 */
static void maskdet(uint32_t* vol, unsigned int nx, unsigned int ny, unsigned int nz, const float* detpos,
                    unsigned int detnum, int svmc) {
    unsigned int dx = nx + 2, dy = ny + 2, dz = nz + 2;
    int isonecube = (nx == 1) && (ny == 1) && (nz == 1);
    static const float corners[8][3] = {{0.f, 0.f, 0.f}, {1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f},
        {1.f, 1.f, 0.f}, {1.f, 0.f, 1.f}, {0.f, 1.f, 1.f}, {1.f, 1.f, 1.f}
    };
    uint32_t* pad = (uint32_t*)calloc((size_t)dx * dy * dz, sizeof(uint32_t));
    unsigned int zi, yi, d;
    for (zi = 1; zi <= nz; zi++) {
        for (yi = 1; yi <= ny; yi++) {
            memcpy(pad + (size_t)zi * dy * dx + yi * dx + 1, vol + (size_t)(zi - 1) * ny * nx + (yi - 1) * nx, nx * sizeof(uint32_t));
        }
    }
    for (d = 0; d < detnum; d++) {
        const float* dp = detpos + d * 4;
        float d2max = (dp[3] + 1.7321f) * (dp[3] + 1.7321f);
        float x, y, z;
        for (z = -dp[3] - 1.f; z <= dp[3] + 1.f; z += 0.5f) {
            float iz = z + dp[2];
            for (y = -dp[3] - 1.f; y <= dp[3] + 1.f; y += 0.5f) {
                float iy = y + dp[1];
                for (x = -dp[3] - 1.f; x <= dp[3] + 1.f; x += 0.5f) {
                    float ix = x + dp[0];
                    float mind2 = K_VERY_BIG_H;
                    unsigned int cc, idx1d;
                    if (iz < 0 || ix < 0 || iy < 0 || ix >= nx || iy >= ny || iz >= nz ||
                            x * x + y * y + z * z > (dp[3] + 1.f) * (dp[3] + 1.f)) {
                        continue;
                    }
                    for (cc = 0; cc < 8; cc++) {
                        float rx = (int)ix - dp[0] + corners[cc][0];
                        float ry = (int)iy - dp[1] + corners[cc][1];
                        float rz = (int)iz - dp[2] + corners[cc][2];
                        float d2 = rx * rx + ry * ry + rz * rz;
                        if (d2 > d2max) {
                            mind2 = K_VERY_BIG_H;
                            break;
                        }
                        if (d2 < mind2) {
                            mind2 = d2;
                        }
                    }
                    if (mind2 == K_VERY_BIG_H ||
                            mind2 >= (dp[3] + 0.5f * (1.f + isonecube)) * (dp[3] + 0.5f * (1.f + isonecube))) {
                        continue;
                    }
                    idx1d = ((int)(iz + 1.f) * dy * dx + (int)(iy + 1.f) * dx + (int)(ix + 1.f));
                    if (svmc) {
                        /* split voxels with a background lower half (4155-4165) */
                        uint32_t lower = (pad[idx1d] & 0xFF000000u) >> 24, upper = (pad[idx1d] & 0x00FF0000u) >> 16;
                        if ((lower || upper) && !lower && upper) {
                            vol[(int)iz * ny * nx + (int)iy * nx + (int)ix] |= DET_MASK;
                        }
                    } else if (pad[idx1d]) {
                        if (!(pad[idx1d + 1] && pad[idx1d - 1] && pad[idx1d + dx] && pad[idx1d - dx] &&
                                pad[idx1d + dy * dx] && pad[idx1d - dy * dx] &&
                                pad[idx1d + dx + 1] && pad[idx1d + dx - 1] && pad[idx1d - dx + 1] && pad[idx1d - dx - 1] &&
                                pad[idx1d + dy * dx + 1] && pad[idx1d + dy * dx - 1] && pad[idx1d - dy * dx + 1] &&
                                pad[idx1d - dy * dx - 1] &&
                                pad[idx1d + dy * dx + dx] && pad[idx1d + dy * dx - dx] && pad[idx1d - dy * dx + dx] &&
                                pad[idx1d - dy * dx - dx] &&
                                pad[idx1d + dy * dx + dx + 1] && pad[idx1d + dy * dx + dx - 1] &&
                                pad[idx1d + dy * dx - dx + 1] && pad[idx1d + dy * dx - dx - 1] &&
                                pad[idx1d - dy * dx + dx + 1] && pad[idx1d - dy * dx + dx - 1] &&
                                pad[idx1d - dy * dx - dx + 1] && pad[idx1d - dy * dx - dx - 1])) {
                            vol[(int)iz * ny * nx + (int)iy * nx + (int)ix] |= DET_MASK;
                        }
                    }
                }
            }
        }
    }
    free(pad);
}

static unsigned int gates_of(const mcxo_input* in) {
    return (unsigned int)(int)((in->tend - in->tstart) / in->tstep + 0.5);
}

static int is_replay(const mcxo_input* in) {
    return in->seed == MCXO_SEED_FROM_FILE;
}

static unsigned int savedetflag_eff(const mcxo_input* in) {
    /* mcx_preprocess, mcx_utils.c:1631-1638, 1763-1791 */
    unsigned int f = in->savedetflag;
    int issavedet = in->issavedet;
    int hasbcdet = 0, i;
    for (i = 6; i < 12; i++) {
        if (in->bc[i] == '1') {
            hasbcdet = 1;
        }
    }
    if (issavedet && in->detnum == 0 && !hasbcdet) {
        issavedet = 0;
    }
    if (!issavedet) {
        /* a replay keeps the flags that describe its input records, mcx_utils.c:1619-1625 */
        return (is_replay(in) ? (f & ~0x80u) : 0u) & ((in->mediabyte >= 100) ? ~(0x2u | 0x4u | 0x8u) : ~0u);
    }
    if (in->ismomentum) {
        f |= 0x8;
    }
    if (in->issaveexit) {
        f |= 0x10 | 0x20;
    }
    if (in->polmedianum && in->smatrix) {
        f |= 0x4 | 0x20 | 0x40 | 0x80;    /* mcx_utils.c:1777-1784 */
    } else {
        f &= ~0x80u;
    }
    if (f == 0) {
        f = 0x5;
    }
    if (in->mediabyte >= 100) {
        f &= ~(0x2u | 0x4u | 0x8u);
    }
    return f;
}

static int savedet_eff(const mcxo_input* in) {
    int i, hasbcdet = 0;
    for (i = 6; i < 12; i++) {
        if (in->bc[i] == '1') {
            hasbcdet = 1;
        }
    }
    if (in->issavedet && in->detnum == 0 && !hasbcdet) {
        return 0;
    }
    return in->issavedet;
}

unsigned int mcxo_reclen(const mcxo_input* in) {
    unsigned int f = savedetflag_eff(in);
    unsigned int partial = (in->medianum - 1) * (SAVE_NSCAT(f) + SAVE_PPATH(f) + SAVE_MOM(f));
    return partial + SAVE_DETID(f) + 3 * (SAVE_PEXIT(f) + SAVE_VEXIT(f)) + SAVE_W0(f) + 4 * SAVE_IQUV(f);
}

/* complex-weight transport (omega > 0, not a replay: mcx_host.cpp:473) or a
   complex replay output (rf, rfmus) */
static int rf_mode(const mcxo_input* in) {
    if (in->omega > 0.f && !is_replay(in)) {
        return 1;
    }
    return (is_replay(in) && (in->outputtype == otRF || in->outputtype == otRFmus)) ? 2 : 0;
}

unsigned int mcxo_fieldcomp(const mcxo_input* in) {
    return rf_mode(in) ? 2u : 1u;
}

unsigned int mcxo_fieldlen(const mcxo_input* in) {
    unsigned int mult = (in->extrasrclen && in->srcid < 0) ? (in->extrasrclen + 1) : 1;
    if (in->srcnum > 1 && (in->srctype == S_PATTERN || in->srctype == S_PATTERN3D)) {
        mult *= in->srcnum;    /* one field per shared pattern, patterns innermost (mcx_host.cpp:474, 679) */
    }
    if (is_replay(in) && in->replaydet == -1) {
        mult *= in->detnum;    /* one block of gates per detector, mcx_host.cpp:684-687 */
    }
    return in->dimx * in->dimy * in->dimz * gates_of(in) * mult;
}

static unsigned char bc_code(char ch, int isdetflag) {
    /* mcx_lookupindex, mcx_utils.c:5292-5305 */
    if (isdetflag) {
        return (unsigned char)(ch == '1' ? 1 : 0);
    }
    switch (ch) {
        case 'r': case 'R': return bcReflect;
        case 'a': case 'A': return bcAbsorb;
        case 'm': case 'M': return bcMirror;
        case 'c': case 'C': return bcCyclic;
        default: return bcUnknown;
    }
}

/* launch voxel and medium of a point source, mcx_utils.c:1722-1748 */
static void point_src_voxel(const float pos[4], unsigned int nx, unsigned int ny, unsigned int nz, const uint32_t* vol,
                            float* p2z, float* p2w) {
    if (pos[0] < 0.f || pos[1] < 0.f || pos[2] < 0.f || pos[0] >= nx || pos[1] >= ny || pos[2] >= nz) {
        *p2z = bits2f(0);
        *p2w = bits2f(0);
    } else {
        uint32_t u = (uint32_t)((int)(floorf(pos[2])) * (ny * nx) + (int)(floorf(pos[1])) * nx + (int)(floorf(pos[0])));
        *p2z = bits2f(u);
        *p2w = bits2f(vol[u] & MED_MASK);
    }
}

/* Preprocessing and kernel constants shared by the oracle and the reference
   harness: mcx_validatecfg/mcx_preprocess (mcx_utils.c:1822-1964,
   1521-1809), parameter packing (mcx_host.cpp:494-524, 647-693), work split
   (1101-1102) and seeding (696-700, 759-768). */
typedef struct {
    ocfg c;
    f4* gprop;
    f4* gdet;
    uint32_t* media;
    uint32_t* seedwords;
    unsigned int nvox, gates, fieldlen, hostreclen;
    float steps;
} oprep;

static int prepare(const mcxo_input* in, oprep* P) {
    ocfg c;
    unsigned int nvox, gates, fieldlen, i, savedetflag, partialdata, hostreclen;
    f4* gprop;
    f4* gdet = NULL;
    uint32_t* media;
    uint32_t* seedwords;
    float fullload, tp_f;
    size_t nph = (size_t)in->nphoton;
    int isbcdet = 0;
    float steps;

    memset(P, 0, sizeof(*P));
    memset(&c, 0, sizeof(c));
    if (in->dimx == 0 || in->dimy == 0 || in->dimz == 0 || in->medianum == 0 || in->nthread == 0) {
        return -1;
    }
    if (in->mediabyte != 1 && in->mediabyte != 2 && in->mediabyte != 4 && in->mediabyte != MEDIA_2LABEL_SPLIT &&
            !(in->mediabyte >= 99 && in->mediabyte <= 104)) {
        return -2;
    }
    if (in->issaveref > 1 || (in->srcnum > 1 && is_replay(in)) ||
            (rf_mode(in) && in->srcnum > 1 && (in->srctype == S_PATTERN || in->srctype == S_PATTERN3D))) {
        return -3;
    }
    nvox = in->dimx * in->dimy * in->dimz;
    gates = gates_of(in);
    fieldlen = mcxo_fieldlen(in);
    savedetflag = savedetflag_eff(in);
    partialdata = (in->medianum - 1) * (SAVE_NSCAT(savedetflag) + SAVE_PPATH(savedetflag) + SAVE_MOM(savedetflag));
    hostreclen = mcxo_reclen(in);

    /* --- preprocessing (mcx_validatecfg / mcx_preprocess) --- */
    steps = in->unitinmm;
    gprop = (f4*)calloc(in->medianum + 4 * in->extrasrclen + 8, sizeof(f4));
    for (i = 0; i < in->medianum; i++) {
        gprop[i].x = in->prop[i * 4];
        gprop[i].y = in->prop[i * 4 + 1];
        gprop[i].z = in->prop[i * 4 + 2];
        gprop[i].w = in->prop[i * 4 + 3];
        if (in->unitinmm != 1.f && i >= 1) {
            gprop[i].y *= in->unitinmm;
            gprop[i].x *= in->unitinmm;
        }
    }
    for (i = 0; i < in->medianum; i++) {
        if (gprop[i].y == 0.f) {
            gprop[i].y = H_EPS;
        }
    }
    /* split-voxel volumes carry a second plane: reference point and normal */
    media = (uint32_t*)malloc((size_t)nvox * sizeof(uint32_t) * (in->mediabyte == MEDIA_2LABEL_SPLIT ? 2 : 1));
    memcpy(media, in->vol, (size_t)nvox * sizeof(uint32_t) * (in->mediabyte == MEDIA_2LABEL_SPLIT ? 2 : 1));

    {
        float off = in->issrcfrom0 ? 0.f : 1.f;
        float sp[4], sd[4];
        double norm;
        memcpy(sp, in->srcpos, sizeof(sp));
        memcpy(sd, in->srcdir, sizeof(sd));
        sp[0] -= off;
        sp[1] -= off;
        sp[2] -= off;
        if (sp[3] == 0.f) {
            sp[3] = 1.f;
        }
        norm = sqrt(sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2]);
        if (norm < H_EPS) {
            free(gprop);
            free(media);
            return -4;
        }
        norm = 1.f / norm;
        sd[0] *= norm;
        sd[1] *= norm;
        sd[2] *= norm;
        c.src.pos = (f4){sp[0], sp[1], sp[2], sp[3]};
        c.src.dir = (f4){sd[0], sd[1], sd[2], sd[3]};
        c.src.p1 = (f4){in->srcparam1[0], in->srcparam1[1], in->srcparam1[2], in->srcparam1[3]};
        c.src.p2 = (f4){in->srcparam2[0], in->srcparam2[1], in->srcparam2[2], in->srcparam2[3]};
        for (i = 0; i < in->extrasrclen; i++) {
            f4* e = gprop + in->medianum + i * 4;
            const float* s = in->srcdata + i * 16;
            e[0] = (f4){s[0] - off, s[1] - off, s[2] - off, s[3] == 0.f ? 1.f : s[3]};
            e[1] = (f4){s[4], s[5], s[6], s[7]};
            e[2] = (f4){s[8], s[9], s[10], s[11]};
            e[3] = (f4){s[12], s[13], s[14], s[15]};
        }
        if (in->detnum) {
            gdet = (f4*)calloc(in->detnum, sizeof(f4));
            for (i = 0; i < in->detnum; i++) {
                gdet[i] = (f4){in->detpos[i * 4] - off, in->detpos[i * 4 + 1] - off, in->detpos[i * 4 + 2] - off, in->detpos[i * 4 + 3]};
            }
        }
    }
    if (in->srctype <= S_CONE || in->srctype == S_ARCSINE || in->srctype == S_ZGAUSSIAN) {
        float pos[4] = {c.src.pos.x, c.src.pos.y, c.src.pos.z, c.src.pos.w};
        point_src_voxel(pos, in->dimx, in->dimy, in->dimz, media, &c.src.p2.z, &c.src.p2.w);
        for (i = 0; i < in->extrasrclen; i++) {
            f4* e = gprop + in->medianum + i * 4;
            float epos[4] = {e[0].x, e[0].y, e[0].z, e[0].w};
            point_src_voxel(epos, in->dimx, in->dimy, in->dimz, media, &e[3].z, &e[3].w);
        }
    }
    for (i = 6; i < 12; i++) {
        if (in->bc[i] == '1') {
            isbcdet = 1;
        }
    }
    if (savedet_eff(in)) {
        float* dp = (float*)malloc(sizeof(float) * 4 * (in->detnum + 1));
        for (i = 0; i < in->detnum; i++) {
            dp[i * 4] = gdet[i].x;
            dp[i * 4 + 1] = gdet[i].y;
            dp[i * 4 + 2] = gdet[i].z;
            dp[i * 4 + 3] = gdet[i].w;
        }
        maskdet(media, in->dimx, in->dimy, in->dimz, dp, in->detnum, in->mediabyte == MEDIA_2LABEL_SPLIT);
        free(dp);
    }

    /* --- kernel constants (mcx_host.cpp:494-524, 647-693) --- */
    c.extrasrclen = in->extrasrclen;
    c.srcid = in->srcid;
    c.maxidx = (f4){(float)in->dimx, (float)in->dimy, (float)in->dimz, 0.f};
    c.dimlen[0] = in->dimx;
    c.dimlen[1] = in->dimx * in->dimy;
    c.dimlen[2] = nvox;
    c.dimlen[3] = fieldlen;
    c.maxgate = gates;
    c.twin0 = in->tstart;
    c.twin1 = in->tstart + in->tstep * (float)gates;
    c.oneoverc0 = K_R_C0 * in->unitinmm;
    c.Rtstep = 1.f / in->tstep;
    c.minenergy = in->minenergy;
    c.minaccumtime = steps * K_R_C0 * in->unitinmm;
    c.save2pt = 1;
    c.doreflect = (unsigned int)in->isreflect;
    c.savedet = (unsigned int)savedet_eff(in);
    c.maxdetphoton = in->maxdetphoton;
    c.maxmedia = in->medianum - 1;
    c.detnum = in->detnum;
    c.voidtime = (unsigned int)in->voidtime;
    c.srctype = (unsigned int)in->srctype;
    c.maxvoidstep = (unsigned int)in->maxvoidstep;
    c.issaveseed = in->issaveseed > 0;
    c.issaveref = (unsigned int)in->issaveref;
    c.isspecular = in->isspecular > 0;
    c.outputtype = (unsigned int)in->outputtype;
    c.savedetflag = savedetflag;
    c.reclen = hostreclen;
    c.partialdata = partialdata;
    c.w0offset = partialdata + 4;
    c.mediaformat = (unsigned int)in->mediabyte;
    c.gscatter = in->gscatter;
    c.srcnum = (in->srcnum > 1 && (in->srctype == S_PATTERN || in->srctype == S_PATTERN3D)) ? in->srcnum : 1;
    c.nphase = in->nphase;
    c.nangle = in->nangle;
    c.invcdf = in->invcdf;
    c.angleinvcdf = in->angleinvcdf;
    c.srcpattern = in->srcpattern;
    c.gprop = gprop;
    c.gdet = gdet;
    c.media = media;
    c.mathmode = in->mathmode;
    c.variant = in->variant;
    c.debugmove = in->debugmove;
    c.maxtraj = in->maxtraj;
    c.traj = in->traj_out;
    c.ntraj = in->ntraj_out;
    if (c.debugmove && (!c.traj || !c.ntraj)) {
        return -3;
    }
    c.fieldmode = in->fieldmode;
    c.nthread = in->nthread;
    c.omega = in->omega;
    c.rfmode = rf_mode(in);
    c.smatrix = (const f4*)in->smatrix;
    c.maxpol = in->smatrix ? in->polmedianum : 0u;
    c.s0 = (f4){in->s0[0], in->s0[1], in->s0[2], in->s0[3]};
    if (is_replay(in)) {
        if (!in->replayseed || !in->replayweight || !in->replaytof || !in->replaydetid ||
                (double)in->nreplay != in->nphoton) {
            free(gprop);
            free(gdet);
            free(media);
            return -5;
        }
        c.replay = 1;
        c.replaydet = in->replaydet;
        c.replaysiteown = in->replaysiteown;
        c.nreplay = in->nreplay;
        c.rseed = in->replayseed;
        c.rweight = in->replayweight;
        c.rtof = in->replaytof;
        c.rdetid = in->replaydetid;
    }
    {
        unsigned int is2d = (in->dimx == 1 ? 1 : (in->dimy == 1 ? 2 : (in->dimz == 1 ? 3 : 0)));
        if (is2d) {
            is2d = is2d * (((in->dimx > 1) + (in->dimy > 1) + (in->dimz > 1)) == 2);
        }
        c.is2d = is2d;
    }
    for (i = 0; i < 12; i++) {
        c.bc[i] = bc_code(in->bc[i], i >= 6);
    }
    {
        int allabsorb = 1, allunknown = 1;
        for (i = 0; i < 6; i++) {
            if (c.bc[i] != bcAbsorb) {
                allabsorb = 0;
            }
            if (c.bc[i] != bcUnknown) {
                allunknown = 0;
            }
        }
        c.dorefl_compiled = in->isreflect || (!allabsorb && !allunknown);
        if (!c.dorefl_compiled) {
            for (i = 0; i < 6; i++) {
                if (c.bc[i] == bcReflect || c.bc[i] == bcMirror) {
                    c.dorefl_compiled = 1;
                }
            }
        }
    }
    (void)isbcdet;

    /* work split, mcx_host.cpp:1101-1102, in the reference's float arithmetic */
    fullload = (float)in->core;
    tp_f = (float)nph * (float)in->core / (fullload * (float)in->nthread * 1);
    c.threadphoton = (unsigned int)(int)tp_f;
    c.oddphoton = (int)((float)nph * (float)in->core / (fullload * 1) - (float)((size_t)c.threadphoton * in->nthread));

    /* seeds, mcx_host.cpp:696-700, 759-768 */
    seedwords = (uint32_t*)malloc(sizeof(uint32_t) * 4 * (size_t)in->nthread);
    srand(in->seed > 0 ? (unsigned int)in->seed : 0u);
    for (i = 0; i < in->seedskip; i++) {
        (void)rand();
    }
    for (i = 0; i < in->nthread * 4; i++) {
        seedwords[i] = (uint32_t)rand();
    }

    P->c = c;
    P->gprop = gprop;
    P->gdet = gdet;
    P->media = media;
    P->seedwords = seedwords;
    P->nvox = nvox;
    P->gates = gates;
    P->fieldlen = fieldlen;
    P->hostreclen = hostreclen;
    P->steps = steps;
    return 0;
}

int mcxo_run(const mcxo_input* in, double* field_out, float* fieldnorm, float* energy_out, float* detp_out,
             uint64_t* seeds_out, uint32_t* masked_out, mcxo_stats* st) {
    oprep P;
    ocfg c;
    unsigned int nvox, gates, fieldlen, i, hostreclen;
    f4* gprop;
    f4* gdet;
    uint32_t* media;
    uint32_t* seedwords;
    float* energy;
    float steps;
    mcxo_stats stats;
    float* ffield = NULL;
    unsigned int ncomp = 1;
    double* dfield = NULL;
    unsigned int nworkers = 1;
    float* wdetp = NULL;
    uint64_t* wdseed = NULL;
    float* wdetw = NULL;
    unsigned int total_det = 0, saved = 0;
    uint64_t cnt[5] = {0, 0, 0, 0, 0};
    int rc = prepare(in, &P);

    if (rc) {
        return rc;
    }
    memset(&stats, 0, sizeof(stats));
    c = P.c;
    gprop = P.gprop;
    gdet = P.gdet;
    media = P.media;
    seedwords = P.seedwords;
    nvox = P.nvox;
    gates = P.gates;
    fieldlen = P.fieldlen;
    hostreclen = P.hostreclen;
    steps = P.steps;
    c.gprop = gprop;
    c.gdet = gdet;
    c.media = media;
    if (masked_out) {
        memcpy(masked_out, media, (size_t)nvox * sizeof(uint32_t));
    }
    energy = energy_out ? energy_out : (float*)malloc(sizeof(float) * 2 * in->nthread);
    memset(energy, 0, sizeof(float) * 2 * in->nthread);

    /* complex fields: real and imaginary blocks; in float mode the four
       quarters the RF deposits address (re, re spill, im, im spill) */
    ncomp = c.rfmode ? 2u : 1u;
    if (c.fieldmode == MCXO_FIELD_FLOAT_SPILL || in->debugrng) {
        ffield = (float*)calloc((size_t)fieldlen * (c.rfmode ? 4 : 2), sizeof(float));
        c.fieldmode = MCXO_FIELD_FLOAT_SPILL;
    }

    if (in->debugrng) {
        /* -D R: each thread writes its stream into the field, mcx_core.cl:2408-2414 */
        for (i = 0; i < in->nthread; i++) {
            uint64_t t[2];
            unsigned int j;
            if ((unsigned long long)i >= (unsigned long long)c.threadphoton * c.nthread + (unsigned int)c.oddphoton) {
                continue;
            }
            t[0] = (uint64_t)seedwords[i * 4] << 32 | seedwords[i * 4 + 1];
            t[1] = (uint64_t)seedwords[i * 4 + 2] << 32 | seedwords[i * 4 + 3];
            for (j = i; j < fieldlen; j += in->nthread) {
                ffield[j] = rng_next(t);
            }
        }
        for (i = 0; i < fieldlen; i++) {
            if (field_out) {
                field_out[i] = (double)ffield[i];
            }
            if (fieldnorm) {
                fieldnorm[i] = ffield[i];
            }
        }
        free(ffield);
        free(seedwords);
        if (!energy_out) {
            free(energy);
        }
        free(gprop);
        free(gdet);
        free(media);
        if (st) {
            memset(st, 0, sizeof(*st));
            st->threadphoton = c.threadphoton;
            st->oddphoton = c.oddphoton;
            st->fieldlen = fieldlen;
            st->maxgate = gates;
            st->reclen = hostreclen;
        }
        return 0;
    }

    if (c.fieldmode == MCXO_FIELD_FLOAT_SPILL) {
        /* serial, in thread order: the same accumulation order as the reference
           kernel run one thread at a time */
        octx X;
        memset(&X, 0, sizeof(X));
        X.c = &c;
        X.ff = ffield;
        X.detcap = in->maxdetphoton;
        X.detp = detp_out ? detp_out : (float*)calloc((size_t)in->maxdetphoton * (hostreclen ? hostreclen : 1), sizeof(float));
        X.dseed = seeds_out ? seeds_out : (uint64_t*)calloc((size_t)in->maxdetphoton * 2 + 2, sizeof(uint64_t));
        X.detw = in->detweight_out;
        for (i = 0; i < in->nthread; i++) {
            run_thread(&X, seedwords, energy, i);
        }
        total_det = X.detcount;
        saved = total_det < in->maxdetphoton ? total_det : in->maxdetphoton;
        cnt[0] = X.nstep;
        cnt[1] = X.nscatter;
        cnt[2] = X.nlaunch;
        cnt[3] = X.nreflect;
        cnt[4] = X.nfailed;
        if (!detp_out) {
            free(X.detp);
        }
        if (!seeds_out) {
            free(X.dseed);
        }
    } else {
        /* FP64 field, threads split into contiguous chunks per worker; records are
           concatenated in thread order so the record list does not depend on the
           worker count */
        double** wfield;
        unsigned int* wcount;
        unsigned int w, chunk;
        uint64_t (*wcnt)[5];
#ifdef _OPENMP
        nworkers = in->nworkers > 0 ? (unsigned int)in->nworkers : (unsigned int)omp_get_max_threads();
#endif
        if (nworkers > in->nthread) {
            nworkers = in->nthread;
        }
        if (nworkers == 0) {
            nworkers = 1;
        }
        chunk = (in->nthread + nworkers - 1) / nworkers;
        wfield = (double**)calloc(nworkers, sizeof(double*));
        wcount = (unsigned int*)calloc(nworkers, sizeof(unsigned int));
        wcnt = calloc(nworkers, sizeof(*wcnt));
        wdetp = (float*)calloc((size_t)nworkers * in->maxdetphoton * (hostreclen ? hostreclen : 1) + 1, sizeof(float));
        wdseed = (uint64_t*)calloc((size_t)nworkers * in->maxdetphoton * 2 + 2, sizeof(uint64_t));
        wdetw = in->detweight_out ? (float*)calloc((size_t)nworkers * in->maxdetphoton * 2 + 2, sizeof(float)) : NULL;
#ifdef _OPENMP
        #pragma omp parallel for num_threads(nworkers) schedule(static, 1)
#endif
        for (w = 0; w < nworkers; w++) {
            octx X;
            unsigned int t0 = w * chunk, t1 = (w + 1) * chunk, t;
            memset(&X, 0, sizeof(X));
            X.c = &c;
            wfield[w] = (double*)calloc((size_t)fieldlen * ncomp, sizeof(double));
            X.fd = wfield[w];
            X.detcap = in->maxdetphoton;
            X.detp = wdetp + (size_t)w * in->maxdetphoton * (hostreclen ? hostreclen : 1);
            X.dseed = wdseed + (size_t)w * in->maxdetphoton * 2;
            X.detw = wdetw ? wdetw + (size_t)w * in->maxdetphoton * 2 : NULL;
            if (t1 > in->nthread) {
                t1 = in->nthread;
            }
            for (t = t0; t < t1; t++) {
                run_thread(&X, seedwords, energy, t);
            }
            wcount[w] = X.detcount;
            wcnt[w][0] = X.nstep;
            wcnt[w][1] = X.nscatter;
            wcnt[w][2] = X.nlaunch;
            wcnt[w][3] = X.nreflect;
            wcnt[w][4] = X.nfailed;
        }
        dfield = (double*)calloc((size_t)fieldlen * ncomp, sizeof(double));
        for (w = 0; w < nworkers; w++) {
            unsigned int k, take;
            for (k = 0; k < fieldlen * ncomp; k++) {
                dfield[k] += wfield[w][k];
            }
            free(wfield[w]);
            total_det += wcount[w];
            take = wcount[w] < in->maxdetphoton ? wcount[w] : in->maxdetphoton;
            if (saved + take > in->maxdetphoton) {
                take = in->maxdetphoton - saved;
            }
            if (detp_out && hostreclen) {
                memcpy(detp_out + (size_t)saved * hostreclen, wdetp + (size_t)w * in->maxdetphoton * hostreclen,
                       sizeof(float) * take * hostreclen);
            }
            if (seeds_out && c.issaveseed) {
                memcpy(seeds_out + (size_t)saved * 2, wdseed + (size_t)w * in->maxdetphoton * 2, sizeof(uint64_t) * 2 * take);
            }
            if (wdetw) {
                memcpy(in->detweight_out + (size_t)saved * 2, wdetw + (size_t)w * in->maxdetphoton * 2, sizeof(float) * 2 * take);
            }
            saved += take;
            for (k = 0; k < 5; k++) {
                cnt[k] += wcnt[w][k];
            }
        }
        free(wfield);
        free(wcount);
        free(wcnt);
        free(wdetp);
        free(wdseed);
        free(wdetw);
    }

    /* --- merge, energies and normalisation (mcx_host.cpp:1252-1306, 1382-1465) --- */
    {
        double etot = 0.0, eesc = 0.0;
        float scale = 1.f;
        float* blockscale = NULL;
        float* sharescale = NULL;
        float Vvox = steps * steps * steps;
        for (i = 0; i < in->nthread; i++) {
            eesc += energy[i * 2];
            etot += energy[i * 2 + 1];
        }
        stats.energytot = etot;
        stats.energyesc = eesc;
        if (in->isnormalized) {
            stats.energyabs = etot - eesc;
            if (in->outputtype == otFlux || in->outputtype == otFluence || in->outputtype >= otAdjoint || c.rfmode == 1) {
                scale = (float)((double)in->unitinmm / (etot * (double)Vvox * (double)in->tstep));
                if (in->outputtype == otFluence || in->outputtype >= otAdjoint) {
                    scale *= in->tstep;
                }
            } else if (in->outputtype == otEnergy || in->outputtype == otL) {
                scale = (float)(1.0 / etot);
            } else if (c.replay && (in->outputtype == otJacobian || in->outputtype == otWP || in->outputtype == otDCS ||
                                    in->outputtype == otRF || in->outputtype == otRFmus ||
                                    in->outputtype == otWLTOF || in->outputtype == otWPTOF)) {
                /* replay outputs, mcx_host.cpp:1396-1431: unitinmm over the replayed
                   detected weight, per detector when each has its own block */
                unsigned int d, nd = (c.replaydet == -1) ? c.detnum : 1;
                for (d = 1; d <= nd; d++) {
                    float sw = 0.f;
                    unsigned int k;
                    for (k = 0; k < c.nreplay; k++) {
                        if (nd == 1 || (c.rdetid[k] & 0xFFFF) == (int)d) {
                            sw += c.rweight[k];
                        }
                    }
                    scale = (sw > 0.f) ? in->unitinmm / sw : 0.f;
                    if (nd > 1) {
                        if (!blockscale) {
                            blockscale = (float*)calloc(nd, sizeof(float));
                        }
                        blockscale[d - 1] = scale;
                    }
                }
            }
            if (c.srcnum > 1) {
                /* per-pattern scale, 1436-1447: the pattern's pixel count over its
                   float Kahan-summed weight */
                unsigned int k;
                int psize = (in->srctype == S_PATTERN3D)
                            ? (int)in->srcparam1[0] * (int)in->srcparam1[1] * (int)in->srcparam1[2]
                            : (int)in->srcparam1[3] * (int)in->srcparam2[3];
                float scaleref = scale;
                sharescale = (float*)calloc(c.srcnum, sizeof(float));
                for (k = 0; k < c.srcnum; k++) {
                    float sum = 0.f, comp = 0.f;
                    int j;
                    for (j = 0; j < psize; j++) {
                        float y = in->srcpattern[(size_t)j * c.srcnum + k] - comp;
                        float t = sum + y;
                        comp = t - sum - y;
                        sum = t;
                    }
                    sharescale[k] = psize / sum * scaleref;
                }
                scale = sharescale[0];
            }
            if (in->extrasrclen && in->srcid < 0) {
                scale *= (float)(in->extrasrclen + 1);
            }
            stats.normalizer = scale;
        }
        for (i = 0; i < fieldlen * ncomp; i++) {
            double raw;
            float merged;
            const unsigned int j = i % fieldlen;
            if (ffield) {
                /* the reference host's merge (mcx_host.cpp:1251-1274): the spill half
                   is added except for the rf replay outputs, whose imaginary part is
                   the second half; the forward run's imaginary part is the third
                   quarter plus its spill */
                if (i < fieldlen) {
                    merged = (c.rfmode == 2) ? ffield[i] : ffield[i] + ffield[i + fieldlen];
                } else {
                    merged = (c.rfmode == 1) ? ffield[j + 2 * (size_t)fieldlen] + ffield[j + 3 * (size_t)fieldlen]
                                             : ffield[j + fieldlen];
                }
                raw = (double)merged;
            } else {
                raw = dfield[i];
                merged = (float)raw;
            }
            if (field_out) {
                field_out[i] = raw;
            }
            if (fieldnorm) {
                float sc = blockscale ? blockscale[j / (fieldlen / c.detnum)] : (sharescale ? sharescale[j % c.srcnum] : scale);
                fieldnorm[i] = in->isnormalized ? merged * sc : merged;
            }
        }
        free(blockscale);
        free(sharescale);
    }
    stats.detected = total_det;
    stats.saved = saved;
    stats.threadphoton = c.threadphoton;
    stats.oddphoton = c.oddphoton;
    stats.reclen = hostreclen;
    stats.fieldlen = fieldlen;
    stats.maxgate = gates;
    stats.nstep = cnt[0];
    stats.nscatter = cnt[1];
    stats.nlaunch = cnt[2];
    stats.nreflect = cnt[3];
    stats.nfailed = cnt[4];
    if (st) {
        *st = stats;
    }
    free(ffield);
    free(dfield);
    free(seedwords);
    if (!energy_out) {
        free(energy);
    }
    free(gprop);
    free(gdet);
    free(media);
    (void)nworkers;
    return 0;
}

int mcxo_replayinit(const mcxo_input* in, const float* detp, unsigned int reclen, unsigned int ndet,
                    const uint64_t* seeds, uint64_t* seed_out, float* weight, float* tof, int* detid) {
    /* mcx_replayinit, mcx_utils.c:1355-1421, after mcx_preprocess has fixed
       savedetflag and scaled mua by unitinmm */
    unsigned int f = savedetflag_eff(in);
    int hasdetid = SAVE_DETID(f);
    unsigned int offset = SAVE_NSCAT(f) * (in->medianum - 1);
    unsigned int i, j, n = 0;
    if (!detp || !seeds || reclen == 0) {
        return -6;
    }
    if (((!hasdetid) && in->detnum > 1) || !SAVE_PPATH(f)) {
        return -7;      /* the baseline run must save detector ids and partial paths ('dp') */
    }
    for (i = 0; i < ndet; i++) {
        const float* rec = detp + (size_t)i * reclen;
        int did = (int)rec[0];
        if (!(in->replaydet <= 0 || in->replaydet == (did & 0xFFFF))) {
            continue;
        }
        if (!(in->srcid <= 0 || ((did & 0xFFFF0000) && in->srcid == ((did & 0xFFFF0000) >> 16)))) {
            continue;
        }
        seed_out[2 * n] = seeds[2 * (size_t)i];
        seed_out[2 * n + 1] = seeds[2 * (size_t)i + 1];
        weight[n] = 1.f;
        tof[n] = 0.f;
        detid[n] = hasdetid ? did : 1;
        for (j = (unsigned int)hasdetid; j < in->medianum - 1 + (unsigned int)hasdetid; j++) {
            float mua = in->prop[(j - hasdetid + 1) * 4];
            float plen = rec[offset + j];
            if (in->unitinmm != 1.f) {
                mua *= in->unitinmm;
            }
            weight[n] *= expf(-mua * plen);
            plen *= in->unitinmm;
            tof[n] += plen * K_R_C0 * in->prop[(j - hasdetid + 1) * 4 + 3];
        }
        if (tof[n] < in->tstart || tof[n] > in->tend) {
            continue;
        }
        n++;
    }
    return (int)n;
}

/* Prepared inputs for the reference-kernel harness (oracle/ref_harness.cpp). */
int mcxo_prepare_ref(const mcxo_input* in, mcxo_refprep* R) {
    oprep P;
    int rc = prepare(in, &P);
    unsigned int i;
    if (rc) {
        return rc;
    }
    memset(R, 0, sizeof(*R));
    memcpy(R->srcpos, &P.c.src.pos, 16);
    memcpy(R->srcdir, &P.c.src.dir, 16);
    memcpy(R->srcparam1, &P.c.src.p1, 16);
    memcpy(R->srcparam2, &P.c.src.p2, 16);
    R->extrasrclen = P.c.extrasrclen;
    R->srcid = P.c.srcid;
    memcpy(R->maxidx, &P.c.maxidx, 16);
    memcpy(R->dimlen, P.c.dimlen, 16);
    R->twin0 = P.c.twin0;
    R->twin1 = P.c.twin1;
    R->oneoverc0 = P.c.oneoverc0;
    R->Rtstep = P.c.Rtstep;
    R->minenergy = P.c.minenergy;
    R->minaccumtime = P.c.minaccumtime;
    R->save2pt = P.c.save2pt;
    R->doreflect = P.c.doreflect;
    R->savedet = P.c.savedet;
    R->maxdetphoton = P.c.maxdetphoton;
    R->maxmedia = P.c.maxmedia;
    R->detnum = P.c.detnum;
    R->voidtime = P.c.voidtime;
    R->srctype = P.c.srctype;
    R->maxvoidstep = P.c.maxvoidstep;
    R->issaveseed = P.c.issaveseed;
    R->issaveref = P.c.issaveref;
    R->isspecular = P.c.isspecular;
    R->maxgate = P.c.maxgate;
    R->outputtype = P.c.outputtype;
    R->threadphoton = P.c.threadphoton;
    R->oddphoton = P.c.oddphoton;
    R->savedetflag = P.c.savedetflag;
    R->reclen = P.c.reclen;
    R->partialdata = P.c.partialdata;
    R->w0offset = P.c.w0offset;
    R->mediaformat = P.c.mediaformat;
    R->gscatter = P.c.gscatter;
    R->is2d = P.c.is2d;
    R->srcnum = P.c.srcnum;
    R->nphase = P.c.nphase;
    R->nangle = P.c.nangle;
    for (i = 0; i < 12; i++) {
        R->bc[i] = (char)P.c.bc[i];
    }
    R->dorefl_compiled = P.c.dorefl_compiled;
    R->nprop = in->medianum + 4 * in->extrasrclen;
    R->gprop = (float*)P.gprop;
    R->gdet = (float*)P.gdet;
    R->media = P.media;
    R->seedwords = P.seedwords;
    R->nvox = P.nvox;
    R->fieldlen = P.fieldlen;
    R->omega = P.c.omega;
    R->rfmode = P.c.rfmode;
    R->maxpolmedia = P.c.maxpol;
    R->smatrix = in->smatrix;
    for (i = 0; i < 4; i++) {
        R->s0[i] = in->s0[i];
    }
    return 0;
}

void mcxo_free_ref(mcxo_refprep* R) {
    free(R->gprop);
    free(R->gdet);
    free(R->media);
    free(R->seedwords);
    memset(R, 0, sizeof(*R));
}

float mcxo_pm_logf(float x) { return opm_logf(x); }
float mcxo_pm_expf(float x) { return opm_expf(x); }
void mcxo_pm_sincosf(float x, float* s, float* c) { opm_sincosf(x, s, c); }
float mcxo_pm_acosf(float x) { return opm_acosf(x); }
