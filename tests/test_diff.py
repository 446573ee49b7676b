"""Gradients of detector readings with respect to per-voxel mua (and the
scattering coefficient) by replaying the detected photons from their seeds.

* CPU: with the oracle as the transport engine, the replay gradient of a
  log-ratio loss matches central finite differences with common random
  numbers (relative step 1e-3) on the most sensitive voxels.
* GPU, the differentiation workload (100^3 Gaussian-random-field mua, 16
  detectors, 1e7 photons): on 64 random voxels drawn among those the
  detected photons visit, the backward pass is within 2% of central
  differences; the backward pass re-detects every replayed photon and takes
  at most 1.5x the forward time; the scattering-coefficient gradient agrees
  with finite differences over a wide step; torch.autograd routes through it.
"""
import time

import numpy as np
import pytest

from mcxcl_gb300 import diff, workloads


def _oracle_engine(O):
    def run(cfg):
        nt = int(cfg["nthread"]) if cfg.get("autopilot", 1) == 0 and "nthread" in cfg else 2048
        r = O.run(cfg, nthread=nt, core=nt, mathmode=O.MATH_LIBM, fieldmode=O.FIELD_DOUBLE)
        out = {"flux": r["flux"], "stat": {"detected": r["stat"]["detected"]}}
        if r["detp"].size:
            out["detp"] = r["detp"]
            out["detweight"] = r["detweight"]
            if r["seeds"] is not None:
                out["seeds"] = np.ascontiguousarray(r["seeds"]).view(np.uint8).reshape(-1, 16).T
        return out
    return run


def _loss(R, Rt):
    return float(np.sum((np.log(R) - np.log(Rt)) ** 2))


def _dloss(R, Rt):
    return 2 * (np.log(R) - np.log(Rt)) / R


def _small(nphoton):
    cfg, mua, target = workloads.diff_config(n=30, nphoton=nphoton)
    cfg["detpos"] = [[15 + 5 * np.cos(a), 15 + 5 * np.sin(a), 0, 1]
                     for a in np.linspace(0, 2 * np.pi, 8, endpoint=False)]
    return cfg, mua, target


def test_replay_gradient_matches_fd_on_oracle(oracle_mod):
    cfg, mua, target = _small(200000)
    sim = diff.ReplayGradient(cfg, run=_oracle_engine(oracle_mod))
    Rt = sim.forward(target)
    R = sim.forward(mua)
    gm = sim.backward(_dloss(R, Rt))
    assert sim.last["redetected"] == len(sim.last["w"]) > 500
    for f in np.argsort(-np.abs(gm).ravel())[:10:2]:
        v = np.unravel_index(f, mua.shape)
        h = np.float32(1e-3) * mua[v]
        mp, mm = mua.copy(), mua.copy()
        mp[v] += h
        mm[v] -= h
        fd = (_loss(sim.forward(mp), Rt) - _loss(sim.forward(mm), Rt)) / float(mp[v] - mm[v])
        assert abs(gm[v] / fd - 1) < 0.02, (v, gm[v], fd)


def test_replay_gradient_sign_and_support(oracle_mod):
    """Raising mua anywhere can only lower a reading: dR_d/dmua <= 0, and it is
    zero where no detected photon went."""
    cfg, mua, _ = _small(50000)
    sim = diff.ReplayGradient(cfg, run=_oracle_engine(oracle_mod))
    R = sim.forward(mua)
    e = np.zeros_like(R)
    e[0] = 1.0
    g = sim.backward(e)
    assert np.all(g <= 0)
    assert 0 < np.count_nonzero(g) < g.size


# ---------------------------------------------------------------- GPU

@pytest.fixture(scope="module")
def c4():
    import mcxcl_gb300
    if not mcxcl_gb300.gpuinfo():
        pytest.fail("no CUDA device visible to the transport library")
    cfg, mua, target = workloads.diff_config()
    sim = diff.ReplayGradient(cfg)
    Rt = sim.forward(target)
    sim.forward(mua)                       # warm-up
    t0 = time.perf_counter()
    R = sim.forward(mua)
    tf = time.perf_counter() - t0
    g = _dloss(R, Rt)
    t0 = time.perf_counter()
    gm = sim.backward(g)
    tb = time.perf_counter() - t0
    return dict(cfg=cfg, mua=mua, Rt=Rt, R=R, sim=sim, gm=gm, tf=tf, tb=tb)


@pytest.mark.gpu
def test_c4_backward_matches_central_differences(c4):
    sim, mua, Rt, gm = c4["sim"], c4["mua"], c4["Rt"], c4["gm"]
    rng = np.random.default_rng(64)
    support = np.flatnonzero(np.abs(gm).ravel() > 1e-3 * np.abs(gm).max())
    picks = rng.choice(support, size=64, replace=False)
    bw, fd = [], []
    for f in picks:
        v = np.unravel_index(f, mua.shape)
        h = np.float32(1e-3) * mua[v]
        mp, mm = mua.copy(), mua.copy()
        mp[v] += h
        mm[v] -= h
        fd.append((_loss(sim.forward(mp), Rt) - _loss(sim.forward(mm), Rt)) / float(mp[v] - mm[v]))
        bw.append(gm[v])
    bw, fd = np.array(bw), np.array(fd)
    assert np.linalg.norm(bw - fd) <= 0.02 * np.linalg.norm(fd), (bw, fd)
    assert np.median(np.abs(bw / fd - 1)) < 0.02


@pytest.mark.gpu
def test_c4_backward_cost_and_redetection(c4):
    sim = c4["sim"]
    sim.forward(c4["mua"])
    sim.backward(_dloss(sim.forward(c4["mua"]), c4["Rt"]))
    assert sim.last["redetected"] == len(sim.last["w"]) > 1000
    assert c4["tb"] <= 1.5 * c4["tf"], (c4["tb"], c4["tf"])


@pytest.mark.gpu
def test_c4_mus_gradient_matches_wide_differences(c4):
    """mus changes the paths, so common random numbers only hold until the
    first discrete event that flips; the likelihood-ratio gradient is checked
    against central differences over +-10% instead."""
    sim, mua, Rt = c4["sim"], c4["mua"], c4["Rt"]
    R = sim.forward(mua, 1.0)
    _, gs = sim.backward(_dloss(R, Rt), want_mus=True)
    h = 0.1
    fd = (_loss(sim.forward(mua, 1.0 + h), Rt) - _loss(sim.forward(mua, 1.0 - h), Rt)) / (2 * h)
    assert abs(gs.sum() - fd) <= 0.1 * abs(fd), (gs.sum(), fd)


@pytest.mark.gpu
def test_torch_autograd_routes_through_replay(c4):
    import torch
    sim, mua, Rt = c4["sim"], c4["mua"], c4["Rt"]
    m = torch.tensor(mua, requires_grad=True)
    R = diff.readings(sim, m)
    loss = ((torch.log(R) - torch.log(torch.tensor(Rt))) ** 2).sum()
    loss.backward()
    ref = sim.backward(_dloss(R.detach().numpy(), Rt))
    np.testing.assert_allclose(m.grad.numpy(), ref.astype(np.float32), rtol=1e-6, atol=1e-12)


# ------------------------------------------------------- per-label gradients

def _label_cfg(nphoton):
    import cases
    cfg = cases.small_two_media(nphoton=nphoton, savedetflag="dsp", seed=31)
    cfg["detpos"] = [[20, 10, 0, 2], [10, 20, 0, 2], [30, 20, 0, 2], [20, 30, 0, 2]]
    return cfg


def test_label_gradient_matches_fd_and_replay_on_oracle(oracle_mod):
    """Per-label mua gradient from the detected records' partial paths:
    central differences with common random numbers (the paths do not move),
    and the replay Jacobian summed over each label's voxels (the replay
    output pinned to the reference's, mcx_core.cl:2845-2858)."""
    cfg = _label_cfg(100000)
    sim = diff.LabelReadings(cfg, run=_oracle_engine(oracle_mod))
    mua0 = sim.prop0[1:, 0].copy()
    Rt = sim.forward(mua0 * 1.3)
    R = sim.forward()
    g = _dloss(R, Rt)
    ga, gs = sim.backward(g)
    assert np.all(np.isfinite(gs)) and len(sim.last["w"]) > 200
    for k in range(sim.nmed):
        h = 1e-3 * mua0[k]
        mp, mm = mua0.copy(), mua0.copy()
        mp[k] += h
        mm[k] -= h
        fd = (_loss(sim.forward(mp), Rt) - _loss(sim.forward(mm), Rt)) / float(np.float32(mp[k]) - np.float32(mm[k]))
        assert abs(ga[k] / fd - 1) < 0.02, (k, ga[k], fd)
    sim.forward()
    rep = sim.replay_mua_gradient(g)
    np.testing.assert_allclose(rep, ga, rtol=1e-5)


@pytest.mark.gpu
def test_label_gradients_on_gpu():
    """The cube + sphere medium (labels 1 and 2), 4 detectors, 2e6 photons:
    per-label mua gradients against central differences with common random
    numbers (2 %) and against the replay Jacobian summed per label; per-label
    mus gradients against central differences over +-5 % (mus moves the paths,
    so those differences are statistical: gradients and differences over 4
    seeds agree within 3 standard errors); torch.autograd routes."""
    import torch
    cfg = dict(workloads.builtin("cubesph60b"), nphoton=2000000, seed=77)
    sim = diff.LabelReadings(cfg)
    mua0, mus0 = sim.prop0[1:, 0].copy(), sim.prop0[1:, 1].copy()
    Rt = sim.forward(mua0 * np.float32(1.2), mus0 * np.float32(0.9))
    R = sim.forward()
    g = _dloss(R, Rt)
    ga, gs = sim.backward(g)
    for k in range(sim.nmed):
        h = 1e-3 * mua0[k]
        mp, mm = mua0.copy(), mua0.copy()
        mp[k] += h
        mm[k] -= h
        fd = (_loss(sim.forward(mp), Rt) - _loss(sim.forward(mm), Rt)) / float(np.float32(mp[k]) - np.float32(mm[k]))
        assert abs(ga[k] / fd - 1) < 0.02, ("mua", k, ga[k], fd)
    sim.forward()
    np.testing.assert_allclose(sim.replay_mua_gradient(g), ga, rtol=1e-3)
    # mus moves the paths: the likelihood-ratio gradient and the central
    # differences are both statistical, so both are taken over 4 seeds and
    # must agree within 3 combined standard errors
    gl, fl = [], []
    for sd in range(4):
        sim.cfg["seed"] = 1000 + sd
        Rs = sim.forward()
        gl.append(sim.backward(_dloss(Rs, Rt))[1])
        row = []
        for k in range(sim.nmed):
            h = 0.1 * mus0[k]
            sp, sm = mus0.copy(), mus0.copy()
            sp[k] += h
            sm[k] -= h
            row.append((_loss(sim.forward(None, sp), Rt) - _loss(sim.forward(None, sm), Rt)) / float(2 * h))
        fl.append(row)
    gl, fl = np.array(gl), np.array(fl)
    se = np.sqrt(gl.var(0, ddof=1) / 4 + fl.var(0, ddof=1) / 4)
    assert np.all(np.abs(gl.mean(0) - fl.mean(0)) <= 3 * se), (gl.mean(0), fl.mean(0), se)
    sim.cfg["seed"] = 77
    sim.forward()
    a = torch.tensor(mua0, requires_grad=True)
    s = torch.tensor(mus0, requires_grad=True)
    Rtt = diff.label_readings(sim, a, s)
    ((torch.log(Rtt) - torch.log(torch.tensor(Rt))) ** 2).sum().backward()
    np.testing.assert_allclose(a.grad.numpy(), ga.astype(np.float32), rtol=1e-5)
    np.testing.assert_allclose(s.grad.numpy(), gs.astype(np.float32), rtol=1e-5)


# ------------------------------------------------------- fluence gradients

def _fluence_cfg(n=30, nphoton=2000000):
    cfg, mua, target = workloads.diff_config(n=n, nphoton=nphoton)
    cfg.pop("detpos")
    cfg.update(issavedet=0, isreflect=0, outputtype="flux")
    return cfg, mua, target


@pytest.mark.gpu
def test_fluence_gradient_per_voxel_mua_matches_central_differences():
    """dLoss/dmua per voxel for L = sum (Phi - Phi_target)^2 over the fluence
    field of a 30^3 float-mua volume: the two gradient passes against central
    differences with common random numbers (relative step 1e-3) on the 16
    voxels of largest gradient and 16 drawn at random among the rest of the
    support: within 2 % in norm.  Also reports the backward/forward time."""
    cfg, mua, target = _fluence_cfg()
    sim = diff.FluenceGradient(cfg)
    Ft = sim.forward(vol=target[None])
    F = sim.forward(vol=mua[None])
    ga, gs = sim.backward(2 * (F - Ft))
    ratio = sim.backward_ms / sim.forward_ms
    support = np.flatnonzero(np.abs(ga).ravel() > 1e-3 * np.abs(ga).max())
    rng = np.random.default_rng(5)
    top = np.argsort(-np.abs(ga).ravel())[:16]
    picks = np.concatenate([top, rng.choice(np.setdiff1d(support, top), size=16, replace=False)])

    def loss(m):
        return float(np.sum((sim.forward(vol=m[None]) - Ft) ** 2))
    bw, fd = [], []
    for f in picks:
        v = np.unravel_index(f, mua.shape)
        h = np.float32(1e-3) * mua[v]
        mp, mm = mua.copy(), mua.copy()
        mp[v] += h
        mm[v] -= h
        fd.append((loss(mp) - loss(mm)) / float(mp[v] - mm[v]))
        bw.append(ga[v])
    bw, fd = np.array(bw), np.array(fd)
    print("fluence gradient: backward/forward time %.2f, rel err %.4f" % (ratio, np.linalg.norm(bw - fd) / np.linalg.norm(fd)))
    assert np.linalg.norm(bw - fd) <= 0.02 * np.linalg.norm(fd), np.c_[bw, fd]
    assert np.all(np.isfinite(gs))
    sim.close()


@pytest.mark.gpu
def test_fluence_gradient_per_label_matches_central_differences():
    """A label volume (cube with a sphere): per-label dLoss/dmua (the
    per-voxel gradient summed over each label) against central differences
    with common random numbers (2 %); per-label dLoss/dmus against central
    differences over +-5 % (mus moves the paths: both over 4 seeds, within
    3 combined standard errors).

    The mus check differentiates the linear functional sum(c F) with c held
    fixed (c = dLoss/dF of one earlier run): with c taken from the same
    photons as the gradient, the likelihood-ratio estimate carries a
    covariance term of order 1/N that the central difference of the noisy
    loss does not have in the same form, so the two would differ by a bias
    that is not an error of either."""
    from mcxcl_gb300 import workloads as W
    cfg = dict(W.builtin("cubesph60b"), nphoton=2000000, seed=91, outputtype="flux", issavedet=0, isreflect=0,
               tstep=1e-9)
    cfg.pop("detpos")
    vol = cfg["vol"]
    prop0 = np.array(cfg["prop"], np.float32)
    target = prop0.copy()
    target[1:, 0] *= 1.2
    target[1:, 1] *= 0.9
    sim = diff.FluenceGradient(cfg)
    Ft = sim.forward(prop=target)
    F = sim.forward(prop=prop0)
    ga, gs = sim.backward(2 * (F - Ft))
    la = np.array([ga[vol == k].sum() for k in (1, 2)])

    def loss(p):
        return float(np.sum((sim.forward(prop=p) - Ft) ** 2))

    def central(k, col, rel):
        pp, pm = prop0.copy(), prop0.copy()
        h = np.float32(rel) * prop0[k, col]
        pp[k, col] += h
        pm[k, col] -= h
        return (loss(pp) - loss(pm)) / float(pp[k, col] - pm[k, col])
    for k in (1, 2):
        fd = central(k, 0, 1e-3)
        assert abs(la[k - 1] - fd) <= 0.02 * abs(fd), ("mua", k, la[k - 1], fd)
    # mus: likelihood-ratio gradients of sum(c F) and its central differences
    # over +-5 %, both over 4 seeds, within 3 combined standard errors
    c = 2 * (F - Ft)

    def linear(p):
        return float(np.sum(c * sim.forward(prop=p)))

    def central_lin(k, rel):
        pp, pm = prop0.copy(), prop0.copy()
        h = np.float32(rel) * prop0[k, 1]
        pp[k, 1] += h
        pm[k, 1] -= h
        return (linear(pp) - linear(pm)) / float(pp[k, 1] - pm[k, 1])
    gl, fl = [], []
    for sd in range(4):
        sim.cfg["seed"] = 500 + sd
        sim.forward(prop=prop0)
        _, gss = sim.backward(c)
        gl.append([gss[vol == k].sum() for k in (1, 2)])
        fl.append([central_lin(k, 0.05) for k in (1, 2)])
    gl, fl = np.array(gl), np.array(fl)
    se = np.sqrt(gl.var(0, ddof=1) / 4 + fl.var(0, ddof=1) / 4)
    assert np.all(np.abs(gl.mean(0) - fl.mean(0)) <= 3 * se), (gl.mean(0), fl.mean(0), se)
    sim.close()
