"""Differentiable detector readings and fluence: d/d(mua, mus) per voxel or
per label.

The forward pass runs the transport kernel on a per-voxel float mua volume
(the reference's MEDIA_MUA_FLOAT format, src/mcx_core.cl:1093-1096) and
records, for every detected photon, its detector, its launch RNG state and
its weight when detected.  The reading of detector d is

    R_d = (1/N) sum_{i detected by d} w_i,   w_i = exp(-sum_v mua_v u L_iv)

(N launched photons, u the voxel size in mm, L_iv the path length of photon
i in voxel v in voxels).  A photon's path does not depend on mua, so

    dR_d/dmua_v = -(u/N) sum_{i in d} w_i L_iv

and, by the likelihood ratio of the free-flight lengths and scattering
events (path density ~ mus^n exp(-mus u L) per medium),

    dR_d/dmus_v = (1/N) sum_{i in d} w_i (n_iv / mus_v - u L_iv).

The backward pass replays only the detected photons from their saved
states -- nothing but the seeds is stored, so memory is O(detected photons)
-- with the per-photon factor a_i = (dLoss/dR_d(i)) w_i / N as the replay
weight: the replay Jacobian output (mcx_core.cl:2845-2858) accumulates
sum a_i L_iv per voxel and the scattering-count output (2567-2604, with each
photon's own factor) sum a_i n_iv.

torch is the plumbing here: the transport runs in the CUDA library through
the pmcxcl-compatible ``run()``; tensors cross as host arrays.
"""
import numpy as np

from . import pmcxcl


def _replay_threads(n):
    """Thread layout of a replay: at least one reference thread per replayed
    photon.  The reference's replay indexes photon seeds as
    threadid * threadphoton + min(threadid, oddphoton - 1) + k
    (mcx_core.cl:1591, 2847), which, whenever the thread count does not divide
    the replayed photons, replays photon oddphoton * (threadphoton + 1) - 1
    twice and the last photon never; with threadphoton 0 every thread that
    runs a photon runs its own."""
    return dict(autopilot=0, nthread=max(64, -(-int(n) // 64) * 64), nblocksize=64)


def _window_tof(cfg, tof):
    """Detection times for a replay, inside the time window: a photon that
    leaves through a detector on the step that also passes the window's end
    is recorded with a time beyond it (as the reference records it); its
    replay deposits into the last gate."""
    t0 = np.float32(cfg.get("tstart", 0.0))
    t1 = np.nextafter(np.float32(cfg.get("tend", 5e-9)), np.float32(0))
    return np.clip(np.asarray(tof, np.float32), t0, t1)


class ReplayGradient:
    """One differentiable simulation setup: everything but the mua volume
    (and optionally the scattering coefficient of label 1) is fixed.  The
    seed is fixed too, so repeated forward passes use common random numbers.

    cfg: a ``run()`` dictionary without ``vol``; prop row 1 gives mus, g, n
    of the medium (its mua column is ignored), row 0 the outside."""

    def __init__(self, cfg, run=None):
        self.run = run or pmcxcl.run
        self.cfg = dict(cfg)
        self.cfg.pop("vol", None)
        self.cfg.update(issavedet=1, issaveseed=1, savedetweight=1, savedetflag="d")
        self.nphoton = float(self.cfg["nphoton"])
        self.ndet = int(np.asarray(self.cfg["detpos"]).reshape(-1, 4).shape[0])
        self.unitinmm = float(self.cfg.get("unitinmm", 1.0))
        self.last = None

    def _prop(self, mus):
        prop = np.array(self.cfg["prop"], np.float32).reshape(-1, 4).copy()
        if mus is not None:
            prop[1, 1] = mus
        return prop

    def forward(self, mua, mus=None):
        """mua: float32 [Nx, Ny, Nz] per mm.  Returns the readings R [ndet] (float64)."""
        mua = np.asarray(mua, np.float32)
        prop = self._prop(mus)
        res = self.run(dict(self.cfg, vol=mua[None], prop=prop))
        if "detp" in res:
            detid = res["detp"][0].astype(np.int64) & 0xFFFF
            w = res["detweight"][0].astype(np.float64)
            tof = _window_tof(self.cfg, res["detweight"][1])
            seeds = res["seeds"]
        else:
            detid = np.zeros(0, np.int64)
            w = np.zeros(0)
            tof = np.zeros(0, np.float32)
            seeds = np.zeros((16, 0), np.uint8)
        R = np.bincount(detid - 1, weights=w, minlength=self.ndet)[:self.ndet] / self.nphoton
        self.last = dict(mua=mua, prop=prop, detid=detid, w=w, tof=tof, seeds=seeds, stat=res["stat"])
        return R

    def _replay(self, a, outputtype, siteown=0):
        L = self.last
        cfg = dict(self.cfg, vol=L["mua"][None], prop=L["prop"], seed=L["seeds"],
                   replayweight=a.astype(np.float32), replaytof=L["tof"], replaydetid=L["detid"].astype(np.int32),
                   outputtype=outputtype, isnormalized=0, issaveseed=0, savedetweight=0, replaysiteown=siteown,
                   **_replay_threads(a.size))
        res = self.run(cfg)
        return res["flux"][..., 0].astype(np.float64), res

    def backward(self, grad_R, want_mus=False):
        """grad_R: dLoss/dR [ndet].  Returns dLoss/dmua [Nx, Ny, Nz] and, when
        want_mus, dLoss/dmus per voxel."""
        L = self.last
        if L is None:
            raise RuntimeError("backward() needs a forward() first")
        g = np.asarray(grad_R, np.float64).ravel()
        a = g[L["detid"] - 1] * L["w"] / self.nphoton
        shape = L["mua"].shape
        if a.size == 0:
            z = np.zeros(shape)
            return (z, z) if want_mus else z
        FJ, res = self._replay(a, "jacobian")
        self.last["redetected"] = res["stat"]["detected"]
        gmua = -self.unitinmm * FJ
        if not want_mus:
            return gmua
        FN, _ = self._replay(a, "nscat", siteown=1)
        mus = float(L["prop"][1, 1]) * self.unitinmm
        return gmua, FN / mus - self.unitinmm * FJ


class LabelReadings:
    """Detector readings of a label volume as functions of every label's mua
    and mus.  No replay is needed: a detected photon's partial path length
    and scattering count in each label -- the per-medium columns of its
    detected record (savedetflag 'dsp', mcx_core.cl:867-926, scatter counts
    kept as integer bits as the reference keeps them) -- are exactly the
    per-label sums of L_iv and n_iv:

        dR_d/dmua_k = -(u/N) sum_{i in d} w_i P_ik
        dR_d/dmus_k =  (1/N) sum_{i in d} w_i (n_ik / mus_k - u P_ik)

    (P_ik in voxels, u the voxel size in mm, mua and mus per mm).  The
    per-voxel replay Jacobian summed over a label's voxels gives the same
    mua column; the seed is fixed, so repeated forwards share random
    numbers.  cfg: a ``run()`` dictionary with a label ``vol`` and ``prop``."""

    def __init__(self, cfg, run=None):
        self.run = run or pmcxcl.run
        self.cfg = dict(cfg)
        self.cfg.update(issavedet=1, issaveseed=1, savedetweight=1, savedetflag="dsp")
        self.nphoton = float(self.cfg["nphoton"])
        self.ndet = int(np.asarray(self.cfg["detpos"]).reshape(-1, 4).shape[0])
        self.unitinmm = float(self.cfg.get("unitinmm", 1.0))
        self.prop0 = np.array(self.cfg["prop"], np.float32).reshape(-1, 4).copy()
        self.nmed = self.prop0.shape[0] - 1
        self.last = None

    def forward(self, mua=None, mus=None):
        """mua, mus: per label 1..nmed (None keeps the configuration's).
        Returns the readings R [ndet] (float64)."""
        prop = self.prop0.copy()
        if mua is not None:
            prop[1:, 0] = np.asarray(mua, np.float32)
        if mus is not None:
            prop[1:, 1] = np.asarray(mus, np.float32)
        res = self.run(dict(self.cfg, prop=prop))
        m = self.nmed
        if "detp" in res:
            d = np.asarray(res["detp"])
            detid = d[0].astype(np.int64) & 0xFFFF
            nscat = np.ascontiguousarray(d[1:1 + m]).view(np.uint32).astype(np.float64)
            ppath = d[1 + m:1 + 2 * m].astype(np.float64)
            w = res["detweight"][0].astype(np.float64)
            tof = _window_tof(self.cfg, res["detweight"][1])
            seeds = res["seeds"]
        else:
            detid = np.zeros(0, np.int64)
            nscat = ppath = np.zeros((m, 0))
            w = np.zeros(0)
            tof = np.zeros(0, np.float32)
            seeds = np.zeros((16, 0), np.uint8)
        R = np.bincount(detid - 1, weights=w, minlength=self.ndet)[:self.ndet] / self.nphoton
        self.last = dict(prop=prop, detid=detid, w=w, tof=tof, seeds=seeds, nscat=nscat, ppath=ppath,
                         stat=res["stat"])
        return R

    def jacobian(self):
        """(dR/dmua, dR/dmus), each [ndet, nmed], per mm, of the last forward."""
        L = self.last
        if L is None:
            raise RuntimeError("jacobian() needs a forward() first")
        u = self.unitinmm
        mus = L["prop"][1:, 1].astype(np.float64)
        Ja = np.zeros((self.ndet, self.nmed))
        Js = np.zeros((self.ndet, self.nmed))
        for k in range(self.nmed):
            wa = -u * L["w"] * L["ppath"][k]
            ws = L["w"] * ((L["nscat"][k] / mus[k] if mus[k] > 0 else 0.0) - u * L["ppath"][k])
            Ja[:, k] = np.bincount(L["detid"] - 1, weights=wa, minlength=self.ndet)[:self.ndet]
            Js[:, k] = np.bincount(L["detid"] - 1, weights=ws, minlength=self.ndet)[:self.ndet]
        return Ja / self.nphoton, Js / self.nphoton

    def backward(self, grad_R):
        """dLoss/dR [ndet] -> (dLoss/dmua, dLoss/dmus), each [nmed]."""
        Ja, Js = self.jacobian()
        g = np.asarray(grad_R, np.float64).ravel()
        return g @ Ja, g @ Js

    def replay_mua_gradient(self, grad_R):
        """dLoss/dmua per label from the replay Jacobian (mcx_core.cl:2845-2858):
        the detected photons relaunched from their seeds, each with replay
        weight dLoss/dR_d w_i / N, the per-voxel output summed over each
        label's voxels."""
        L = self.last
        g = np.asarray(grad_R, np.float64).ravel()
        a = g[L["detid"] - 1] * L["w"] / self.nphoton
        cfg = dict(self.cfg, prop=L["prop"], seed=L["seeds"], replayweight=a.astype(np.float32),
                   replaytof=L["tof"], replaydetid=L["detid"].astype(np.int32), outputtype="jacobian",
                   isnormalized=0, issaveseed=0, savedetweight=0, **_replay_threads(a.size))
        F = self.run(cfg)["flux"].astype(np.float64)
        F = F.reshape(F.shape[:3] + (-1,)).sum(axis=3)      # every time gate of the detected photons
        vol = np.asarray(self.cfg["vol"])
        return np.array([-self.unitinmm * F[vol == k + 1].sum() for k in range(self.nmed)])


class FluenceGradient:
    """Gradient of a loss of the fluence (flux) field with respect to every
    voxel's mua and mus, on the GPU.  A photon's path does not depend on
    mua, so the transport kernel's fluence-gradient passes (MCXG_ADJ1 /
    MCXG_ADJ2) rerun the forward photons with the same random numbers: the
    first stores each photon's loss total, the second accumulates, per voxel
    visit, the visit's own deposit derivative minus its path length times
    the loss of the photon's later deposits, and per scattering the
    likelihood-ratio term of mus.  Memory: one float per photon.  Label
    volumes give per-label gradients by summing over each label's voxels.

    cfg: a ``run()`` dictionary with ``vol`` (labels, or float mua as
    [1, Nx, Ny, Nz]) and ``prop``; outputtype flux or fluence; no Russian
    roulette (its survival draws depend on the weight)."""

    def __init__(self, cfg):
        import ctypes
        from . import _lib
        self._ct = ctypes
        self._lib = _lib
        self.L = _lib.load()
        self.cfg = dict(cfg)
        self.C = None
        self.s = None
        self.scale = None

    def close(self):
        if self.C is not None:
            self.L.mcx_clearcfg(self._ct.byref(self.C))
            self.C = None
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc:
            raise RuntimeError("%s: %s" % (what, self.L.mcxg_error_string(rc).decode()))

    def forward(self, **override):
        """Runs the forward problem (cfg updated by ``override``, e.g. a new
        ``vol`` or ``prop``); returns the normalised field [Nx, Ny, Nz, gates]
        in FP64 (the compensated accumulator merged without rounding to
        float)."""
        ct = self._ct
        self.close()
        C = self._lib.Config()
        pmcxcl.parse_config(dict(self.cfg, **override), C)
        self.L.mcx_validatecfg(ct.byref(C), None, None, 0)
        pmcxcl._check(C)
        s = self.L.mcx_prepare_simulation(ct.byref(C))
        pmcxcl._check(C)
        self.C, self.s = C, s
        ms = ct.c_float()
        self._check(self.L.mcxg_simulate(s, 2, ct.byref(ms)), "forward")
        self.forward_ms = ms.value
        esc, tot = ct.c_double(), ct.c_double()
        self._check(self.L.mcxg_get_energy(s, ct.byref(esc), ct.byref(tot)), "energies")
        vvox = float(C.steps.x * C.steps.y * C.steps.z)
        self.scale = float(C.unitinmm) / (tot.value * vvox * float(C.tstep))
        if ord(C.outputtype) == 1:             # fluence: flux times the gate width
            self.scale *= float(C.tstep)
        self.shape = (C.dim.x, C.dim.y, C.dim.z, int(C.maxgate))
        n = int(C.dim.x) * C.dim.y * C.dim.z * int(C.maxgate)
        out = np.zeros(n, np.float64)
        self._check(self.L.mcxg_get_field_f64(s, out.ctypes.data), "field")
        return out.reshape(self.shape, order="F") * self.scale

    def backward(self, dloss):
        """dloss: dLoss/dfield [Nx, Ny, Nz, gates] of the last forward.
        Returns (dLoss/dmua, dLoss/dmus), each [Nx, Ny, Nz], per mm."""
        ct = self._ct
        if self.s is None:
            raise RuntimeError("backward() needs a forward() first")
        c = (np.asarray(dloss, np.float64) * self.scale).astype(np.float32).ravel(order="F")
        self._check(self.L.mcxg_set_adjoint(self.s, c.ctypes.data, c.size), "loss gradient")
        ms1, ms2 = ct.c_float(), ct.c_float()
        self._check(self.L.mcxg_simulate(self.s, 256, ct.byref(ms1)), "gradient pass 1")
        self._check(self.L.mcxg_simulate(self.s, 512, ct.byref(ms2)), "gradient pass 2")
        self.backward_ms = ms1.value + ms2.value
        nvox = self.shape[0] * self.shape[1] * self.shape[2]
        ga, gs = np.zeros(nvox, np.float32), np.zeros(nvox, np.float32)
        self._check(self.L.mcxg_get_adjoint_grad(self.s, ga.ctypes.data, gs.ctypes.data), "gradients")
        u = float(self.C.unitinmm)
        f = self.shape[:3]
        return (ga.astype(np.float64).reshape(f, order="F") * u, gs.astype(np.float64).reshape(f, order="F") * u)


def readings(sim, mua, mus=None):
    """Detector readings as a differentiable torch function of mua (and of
    the scalar mus of label 1 when given as a tensor)."""
    import torch

    class _Readings(torch.autograd.Function):
        @staticmethod
        def forward(ctx, mua_t, mus_t):
            m = None if mus_t is None else float(mus_t.detach().cpu())
            R = sim.forward(mua_t.detach().cpu().numpy(), m)
            ctx.dev, ctx.dtype = mua_t.device, mua_t.dtype
            ctx.want_mus = mus_t is not None and mus_t.requires_grad
            return torch.as_tensor(R, dtype=torch.float64, device=mua_t.device)

        @staticmethod
        def backward(ctx, gR):
            out = sim.backward(gR.detach().cpu().numpy(), want_mus=ctx.want_mus)
            if ctx.want_mus:
                gmua, gmus = out
                gm = torch.as_tensor(gmus.sum(), dtype=torch.float64, device=ctx.dev)
            else:
                gmua, gm = out, None
            return torch.as_tensor(gmua, dtype=ctx.dtype, device=ctx.dev), gm

    return _Readings.apply(mua, mus)


def label_readings(sim, mua, mus):
    """Detector readings as a differentiable torch function of the per-label
    mua and mus tensors ([nmed] each) of a LabelReadings setup."""
    import torch

    class _LabelReadings(torch.autograd.Function):
        @staticmethod
        def forward(ctx, mua_t, mus_t):
            R = sim.forward(mua_t.detach().cpu().numpy(), mus_t.detach().cpu().numpy())
            ctx.dev, ctx.dtype = mua_t.device, mua_t.dtype
            return torch.as_tensor(R, dtype=torch.float64, device=mua_t.device)

        @staticmethod
        def backward(ctx, gR):
            ga, gs = sim.backward(gR.detach().cpu().numpy())
            return (torch.as_tensor(ga, dtype=ctx.dtype, device=ctx.dev),
                    torch.as_tensor(gs, dtype=ctx.dtype, device=ctx.dev))

    return _LabelReadings.apply(mua, mus)
