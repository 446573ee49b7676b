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
        r = O.run(cfg, nthread=2048, core=2048, mathmode=O.MATH_LIBM, fieldmode=O.FIELD_DOUBLE)
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
