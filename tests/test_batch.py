"""Batches: many simulations in one persistent launch (mcx_run_batch).

* A simulation's result does not depend on the batch around it: alone or in
  a batch, its per-simulation energies are the same bits and its field the
  same to the rounding of the atomics.
* The batch reproduces the reference's cube60 known answer and agrees with
  the one-simulation-per-launch kernel within the Monte Carlo noise.
* A captured CUDA graph replays the same run.
"""
import numpy as np
import pytest

import cases
from mcxcl_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import mcxcl_gb300
    info = mcxcl_gb300.gpuinfo()
    if not info:
        pytest.fail("no CUDA device visible to the transport library")
    return info[0]


def _absorbed(r):
    return r["stat"]["energyabs"] / r["stat"]["energytot"]


def test_batch_member_is_independent_of_its_batch(gpu):
    import mcxcl_gb300
    sims = workloads.batch_configs(nsim=6, master_seed=3, edge=(32, 48), photons=(1e5, 3e5))
    alone = mcxcl_gb300.run_batch([sims[2]])[0]
    together = mcxcl_gb300.run_batch(sims)
    t = together[2]
    assert t["stat"]["energytot"] == alone["stat"]["energytot"]
    assert _absorbed(t) == _absorbed(alone)
    np.testing.assert_allclose(t["flux"], alone["flux"], rtol=2e-5, atol=1e-7 * alone["flux"].max())
    for cfg, r in zip(sims, together):
        assert r["flux"].shape == cfg["vol"].shape + (1,)
        assert abs(r["stat"]["energytot"] - cfg["nphoton"]) <= 1e-6 * cfg["nphoton"] + 10


def test_batch_reference_known_answer(gpu):
    """cube60 at 1e7 photons: 0.1769 absorbed (mcx_gpu_benchmarks.m:46-69)."""
    import mcxcl_gb300
    b1 = cases.cube60(nphoton=10000000, seed=29012392, issavedet=0)
    b1.pop("detpos")
    small = workloads.batch_configs(nsim=5, master_seed=5, edge=(32, 40), photons=(1e5, 2e5))
    res = mcxcl_gb300.run_batch(small + [b1])
    assert abs(_absorbed(res[-1]) - 0.1769) <= 0.005


def test_batch_agrees_with_one_launch_per_simulation(gpu):
    """Absorbed fraction and voxel fluence of batch members against the same
    simulations run one per launch (different seeds: statistical)."""
    import mcxcl_gb300
    sims = workloads.batch_configs(nsim=4, master_seed=9, edge=(40, 60), photons=(2e6, 3e6))
    batch = mcxcl_gb300.run_batch(sims)
    for cfg, b in zip(sims, batch):
        one = mcxcl_gb300.run(dict(cfg, seed=cfg["seed"] + 1))
        a1, a2 = _absorbed(one), _absorbed(b)
        assert abs(a1 - a2) <= 0.003 + 0.01 * a1, (a1, a2)
        f1, f2 = one["flux"].sum(), b["flux"].sum()
        assert abs(f1 - f2) <= 0.01 * f1, (f1, f2)


def test_batch_graph_replay_matches_stream_run(gpu):
    import mcxcl_gb300
    sims = workloads.batch_configs(nsim=8, master_seed=11, edge=(32, 40), photons=(1e5, 2e5))
    a = mcxcl_gb300.run_batch(sims)
    g1 = mcxcl_gb300.run_batch(sims, graph=True)
    g2 = mcxcl_gb300.run_batch(sims, graph=True)
    for x, y, z in zip(a, g1, g2):
        assert x["stat"]["energytot"] == y["stat"]["energytot"] == z["stat"]["energytot"]
        assert _absorbed(x) == _absorbed(y) == _absorbed(z)
        np.testing.assert_allclose(y["flux"], x["flux"], rtol=2e-5, atol=1e-7 * x["flux"].max())


def test_batch_rejects_detectors(gpu):
    import mcxcl_gb300
    cfg = cases.cube60(nphoton=1000)
    with pytest.raises(mcxcl_gb300.MCXError, match="batch"):
        mcxcl_gb300.run_batch([cfg])


@pytest.mark.gpu
def test_batch_compensated_field_against_fp64():
    """The batched launch with every deposit also accumulated in FP64 (the
    same photons): each simulation's compensated field agrees with it to
    1e-6 relative in every non-zero element and to 1e-9 in its total."""
    import mcxcl_gb300
    from mcxcl_gb300 import workloads
    sims = workloads.batch_configs(nsim=16, master_seed=11, edge=(32, 64), photons=(1e5, 2e6))
    res = mcxcl_gb300.run_batch(sims, verify=True)
    for r in res:
        st = r["stat"]
        assert st["relerr_max"] <= 1e-6 and st["relerr_median"] <= 1e-7 and st["relerr_total"] <= 1e-9, st
