/*
 * ref_harness.cpp -- runs the reference photon-transport kernel
 * (src/mcx_core.cl, compiled in place as host C++ through ref_shim.hpp) on
 * the CPU with the same prepared inputs as the oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile into oracle/_ref/ only
 * when the reference sources are present; never committed, never shipped.
 *
 * Threads are run block by block, thread by thread, in global-index order,
 * exactly one reference thread at a time, so the deposits happen in the same
 * order as the oracle's serial mode and the outputs compare bit for bit.
 */
#include "ref_shim.hpp"
#define MCX_ADJOINT_MODE       /* the adjoint post-kernels (mcx_core.cl:3313-3514) */
#include "mcx_core.cl"

#include "mcx_oracle.h"

#include <algorithm>
#include <vector>

struct ReplayBufs {
    float* weight = nullptr;
    float* tof = nullptr;
    int* detid = nullptr;
    unsigned int* jump = nullptr;      /* trajectory capture (-D M): record counter and records */
    float* debug = nullptr;
};

template <int ispencil, int isreflect, int issvmc>
static void run_blocks(const mcxo_refprep& R, unsigned int nblock, unsigned int bsize, unsigned int* media,
                       float* field, float* genergy, unsigned int* seeds, float* detp, unsigned int* detcount,
                       float* gprop, float* gdet, RandType* gseed, float* srcpattern, const float* invcdf,
                       unsigned int nphase, const float* angleinvcdf, unsigned int nangle, int nworkers,
                       const ReplayBufs& rp) {
    (void)nworkers;
    for (long b = 0; b < (long)nblock; b++) {
        unsigned int progress = 0;
        blockIdx = make_uint3((unsigned int)b, 0, 0);
        blockDim = make_uint3(bsize, 1, 1);
        gridDim = make_uint3(nblock, 1, 1);
        /* the kernel's table preload (mcx_core.cl:2354-2383) splits the copy
           across the block's threads and synchronises; run one thread at a
           time, the block's tables are filled up front instead */
        if (invcdf) {
            std::memcpy(sharedmem_raw, invcdf, sizeof(float) * nphase);
        }
        if (angleinvcdf) {
            std::memcpy(sharedmem_raw + sizeof(float) * (nphase + (nphase & 1)), angleinvcdf, sizeof(float) * nangle);
        }
        for (unsigned int t = 0; t < bsize; t++) {
            threadIdx = make_uint3(t, 0, 0);
            mcx_main_loop<ispencil, isreflect, !issvmc, issvmc, 0>(
                media, field, genergy, seeds, detp, (const float4*)gprop, srcpattern, (const float4*)gdet,
                &progress, detcount, rp.weight, rp.tof, rp.detid, gseed, rp.jump, rp.debug, (float*)invcdf, (float*)angleinvcdf,
                (RandType*)sharedmem_raw, (float4*)R.smatrix);
        }
    }
}

extern "C" int mcxref_run(const mcxo_input* in, unsigned int nblocksize, int nworkers, float* field_out,
                          float* energy_out, float* detp_out, uint64_t* seeds_out, unsigned int* detcount_out) {
    mcxo_refprep R;
    int rc = mcxo_prepare_ref(in, &R);
    if (rc) {
        return rc;
    }
    if (in->nthread % nblocksize) {
        mcxo_free_ref(&R);
        return -10;
    }
    if (in->mediabyte > 4 && in->mediabyte != 97) {
        /* the __NVCC__ launch path garbles prop.y/z for MEDIA_MUA_FLOAT (mcx_core.cl:2214-2231);
           split voxels overwrite the whole property row there */
        mcxo_free_ref(&R);
        return -11;
    }
    MCXParam& P = gcfg_const[0];
    std::memset(&P, 0, sizeof(P));
    std::memcpy(&P.src.pos, R.srcpos, 16);
    std::memcpy(&P.src.dir, R.srcdir, 16);
    std::memcpy(&P.src.param1, R.srcparam1, 16);
    std::memcpy(&P.src.param2, R.srcparam2, 16);
    P.extrasrclen = R.extrasrclen;
    P.srcid = R.srcid;
    std::memcpy(&P.maxidx, R.maxidx, 16);
    std::memcpy(&P.dimlen, R.dimlen, 16);
    P.minstep = 1.f;
    P.twin0 = R.twin0;
    P.twin1 = R.twin1;
    P.tmax = in->tend;
    P.oneoverc0 = R.oneoverc0;
    P.save2pt = R.save2pt;
    P.doreflect = R.doreflect;
    P.savedet = R.savedet;
    P.Rtstep = R.Rtstep;
    P.minenergy = R.minenergy;
    P.minaccumtime = R.minaccumtime;
    P.maxdetphoton = R.maxdetphoton;
    P.maxmedia = R.maxmedia;
    P.detnum = R.detnum;
    P.voidtime = (int)R.voidtime;
    P.srctype = (int)R.srctype;
    P.maxvoidstep = R.maxvoidstep;
    P.issaveseed = R.issaveseed;
    P.issaveref = R.issaveref;
    P.isspecular = R.isspecular;
    P.maxgate = R.maxgate;
    P.seed = in->seed;
    P.replaydet = in->replaydet;
    P.outputtype = R.outputtype;
    P.threadphoton = R.threadphoton;
    P.oddphoton = R.oddphoton;
    P.savedetflag = R.savedetflag;
    P.reclen = R.reclen;
    P.partialdata = R.partialdata;
    P.w0offset = R.w0offset;
    P.mediaformat = R.mediaformat;
    P.gscatter = R.gscatter;
    P.is2d = R.is2d;
    P.srcnum = R.srcnum;
    P.omega = R.omega;
    P.maxpolmedia = R.maxpolmedia;
    P.s0 = make_float4(R.s0[0], R.s0[1], R.s0[2], R.s0[3]);
    P.debuglevel = in->debugmove ? 2u : 0u;    /* MCX_DEBUG_MOVE */
    P.maxjumpdebug = in->maxtraj;
    P.nphase = R.nphase;
    P.nphaselen = R.nphase + (R.nphase & 1);
    P.nangle = R.nangle;
    P.nanglelen = R.nangle + (R.nangle & 1);
    std::memcpy(P.bc, R.bc, 12);

    unsigned int nblock = in->nthread / nblocksize;
    /* the __NVCC__ launch path reads media[idx + nvox] (updateproperty_asgn),
       so the volume is padded with a zero second half */
    std::vector<unsigned int> media(2 * (size_t)R.nvox, 0u);
    std::memcpy(media.data(), R.media, sizeof(unsigned int) * R.nvox * (R.mediaformat == 97 ? 2 : 1));
    /* RF: four quarters (re, re spill, im, im spill); the rfmus replay output
       writes the third quarter although the reference allocates two */
    std::vector<float> field((R.rfmode ? 4 : 2) * (size_t)R.fieldlen, 0.f);
    std::vector<float> genergy(2 * (size_t)in->nthread, 0.f);
    std::vector<unsigned int> seeds(R.seedwords, R.seedwords + 4 * (size_t)in->nthread);
    /* replay: the seed buffer holds one saved state per photon (the kernel
       also reads a start state per thread from it, which the launch then
       overwrites); one zero-weight photon pads the per-photon arrays, which
       the reference's scattering-site deposits read one photon ahead */
    const bool replay = (in->seed == MCXO_SEED_FROM_FILE);
    ReplayBufs rp;
    unsigned int jumpctr = 0;
    std::vector<float> debugdata(in->debugmove ? 6 * (size_t)in->maxtraj + 6 : 0);
    if (in->debugmove) {
        if (!in->traj_out || !in->ntraj_out) {
            mcxo_free_ref(&R);
            return -3;
        }
        rp.jump = &jumpctr;
        rp.debug = debugdata.data();
    }
    std::vector<float> rweight, rtof;
    std::vector<int> rdetid;
    if (replay) {
        size_t nw = std::max((size_t)in->nreplay * 4 + 8, (size_t)in->nthread * 4 + 8);
        seeds.assign(nw, 0u);
        std::memcpy(seeds.data(), in->replayseed, sizeof(uint64_t) * 2 * in->nreplay);
        rweight.assign(in->nreplay + 1, 0.f);
        rtof.assign(in->nreplay + 1, in->tstart);
        rdetid.assign(in->nreplay + 1, 1);
        std::memcpy(rweight.data(), in->replayweight, sizeof(float) * in->nreplay);
        std::memcpy(rtof.data(), in->replaytof, sizeof(float) * in->nreplay);
        std::memcpy(rdetid.data(), in->replaydetid, sizeof(int) * in->nreplay);
        rp.weight = rweight.data();
        rp.tof = rtof.data();
        rp.detid = rdetid.data();
    }
    size_t reclen = R.reclen ? R.reclen : 1;
    std::vector<float> detp((size_t)R.maxdetphoton * reclen + 1, 0.f);
    std::vector<RandType> gseed((size_t)R.maxdetphoton * 2 + 2, 0);
    unsigned int detcount = 0;
    std::vector<float> gprop(R.gprop, R.gprop + 4 * (size_t)R.nprop);
    std::vector<float> gdet(4 * (size_t)(R.detnum + 1), 0.f);
    if (R.detnum) {
        std::memcpy(gdet.data(), R.gdet, sizeof(float) * 4 * R.detnum);
    }

    int ispencil = (in->srctype == MCX_SRC_PENCIL);
    int isreflect = R.dorefl_compiled;
#define RUN(a, b, sv) run_blocks<a, b, sv>(R, nblock, nblocksize, media.data(), field.data(), genergy.data(), seeds.data(), \
                                   detp.data(), &detcount, gprop.data(), gdet.data(), gseed.data(), (float*)in->srcpattern, \
                                   in->invcdf, in->nphase, in->angleinvcdf, in->nangle, nworkers, rp)
    /* split-voxel volumes run the kernel built for them (issvmc) */
    if (R.mediaformat == 97) {
        if (ispencil && isreflect) {
            RUN(1, 1, 1);
        } else if (ispencil) {
            RUN(1, 0, 1);
        } else if (isreflect) {
            RUN(0, 1, 1);
        } else {
            RUN(0, 0, 1);
        }
    } else if (ispencil && isreflect) {
        RUN(1, 1, 0);
    } else if (ispencil) {
        RUN(1, 0, 0);
    } else if (isreflect) {
        RUN(0, 1, 0);
    } else {
        RUN(0, 0, 0);
    }
#undef RUN

    /* the reference host's merge, mcx_host.cpp:1251-1274 */
    const size_t F = R.fieldlen;
    for (size_t i = 0; i < F; i++) {
        field_out[i] = (R.rfmode == 2) ? field[i] : field[i] + field[i + F];
    }
    if (R.rfmode == 1) {
        for (size_t i = 0; i < F; i++) {
            field_out[F + i] = field[i + 2 * F] + field[i + 3 * F];
        }
    } else if (R.rfmode == 2) {
        for (size_t i = 0; i < F; i++) {
            field_out[F + i] = field[i + F];
        }
    }
    if (energy_out) {
        std::memcpy(energy_out, genergy.data(), sizeof(float) * 2 * in->nthread);
    }
    unsigned int saved = detcount < R.maxdetphoton ? detcount : R.maxdetphoton;
    if (detp_out && R.reclen) {
        std::memcpy(detp_out, detp.data(), sizeof(float) * saved * R.reclen);
    }
    if (seeds_out && R.issaveseed) {
        std::memcpy(seeds_out, gseed.data(), sizeof(uint64_t) * 2 * saved);
    }
    if (detcount_out) {
        *detcount_out = detcount;
    }
    if (in->debugmove) {
        *in->ntraj_out = jumpctr;
        std::memcpy(in->traj_out, debugdata.data(), sizeof(float) * 6 * (size_t)std::min(jumpctr, in->maxtraj));
    }
    mcxo_free_ref(&R);
    return 0;
}

/* The reference's Mie routine (src/mcx_mie.cpp:91), compiled from its own
   source: Mueller rows {S11, S12, S33, S34} at the 181 angles the reference's
   mcx_prep_polarized uses (mcx_utils.c:1484-1488), for pinning the polarised
   transport and checking the library's own Mie series. */
extern "C" void Mie(double x, double mx, const double* mu, float4* smatrix, double* qsca, double* g);

extern "C" void mcx_error(const int id, const char* msg, const char* file, const int linenum) {
    std::fprintf(stderr, "reference Mie error %d: %s\n", id, msg);
}

extern "C" void mcxref_mie(double x, double mrel, float* smatrix, double* qsca, double* g) {
    std::vector<double> mu(181);
    for (int i = 0; i < 181; i++) {
        mu[i] = cos((double)(3.1415926535897932f * i / (181 - 1)));
    }
    Mie(x, mrel, mu.data(), (float4*)smatrix, qsca, g);
}

/* The reference's adjoint post-kernels, one voxel per emulated thread:
   kind 0 mcx_adjoint_kernel (phi_src x phi_det), 1 mcx_adjoint_dcoeff_kernel
   (grad phi_src . grad phi_det), real fields (gfield_im NULL). */
extern "C" void mcxref_adjoint(int kind, float* field, float* out, unsigned int dimxyz, unsigned int maxgate,
                               unsigned int ns, unsigned int nd, unsigned int nx, unsigned int ny) {
    blockDim = make_uint3(1, 1, 1);
    gridDim = make_uint3(dimxyz, 1, 1);
    threadIdx = make_uint3(0, 0, 0);
    for (unsigned int v = 0; v < dimxyz; v++) {
        blockIdx = make_uint3(v, 0, 0);
        if (kind == 0) {
            mcx_adjoint_kernel(field, nullptr, out, dimxyz, maxgate, ns, nd);
        } else {
            mcx_adjoint_dcoeff_kernel(field, nullptr, out, dimxyz, maxgate, ns, nd, nx, ny);
        }
    }
}
