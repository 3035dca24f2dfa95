"""FP64 parity at the full sizes of the benchmark shapes: the GPU step and
the CPU oracle agree bit for bit (pair sets, multipliers, iteration counts,
rod state) on the 20,000-rod quasi-2D layer, the 50,000-rod bundle with
200,000 crosslinkers, the 200,000-rod evaluation cube and the 64-replica
ensemble, for five steps each from their seeded initial states."""
import numpy as np
import pytest

from alens_gb300 import capi, workloads
from alens_gb300.oracle_api import OracleSystem

pytestmark = pytest.mark.gpu


def run_pair(cfg, rods, steps, links=None):
    g = capi.GpuSystem(cfg)
    o = OracleSystem(cfg)
    for s in (g, o):
        s.set_rods(rods)
        if links is not None:
            s.set_links(links)
    for _ in range(steps):
        sg, so = g.step(), o.step()
        assert sg["nCollision"] == so["nCollision"] and sg["nBilateral"] == so["nBilateral"]
        assert sg["iterations"] == so["iterations"], (sg, so)
        cg, co = g.constraints(), o.constraints()
        assert np.array_equal(cg["i"], co["i"]) and np.array_equal(cg["j"], co["j"])
        assert np.array_equal(cg["image"], co["image"])
        assert np.array_equal(cg["gamma"], co["gamma"])
    pg, qg = g.get_rods()
    po, qo = o.get_rods()
    assert np.array_equal(pg, po) and np.array_equal(qg, qo)
    return sg


def test_layer_20000(gpu_lib):
    w = workloads.dense_monolayer(n=20000, side=40.0, seed=0)
    st = run_pair(w.cfg, w.rods, 5)
    assert st["nCollision"] > 10000


def test_layer_20000_fuller_blocks(gpu_lib, monkeypatch):
    """At least 24 tiles (1,536 rows) per solver block: each block's rows
    overflow its shared-memory row cache, so cached and uncached rows mix."""
    monkeypatch.setenv("ALENS_SOLVER_MIN_TILES", "24")
    w = workloads.dense_monolayer(n=20000, side=40.0, seed=0)
    run_pair(w.cfg, w.rods, 3)


def test_bundle_50000_with_200000_links(gpu_lib):
    w = workloads.crosslinked_bundle_rods(n=50000, box=20.0, seed=0)
    pairs = workloads.pair_list(capi.GpuSystem, w.cfg, w.rods, 0.05)
    links = workloads.make_links(w.cfg, w.rods, pairs, 200000, seed=1)
    st = run_pair(w.cfg, w.rods, 5, links=links)
    assert st["nBilateral"] == 200000


def test_eval_cube_200000(gpu_lib):
    w = workloads.large_eval(n=200000, box=40.0, seed=0)
    run_pair(w.cfg, w.rods, 5)


def test_ensemble_64_replicas(gpu_lib):
    reps = workloads.ensemble(nrep=64, nmin=500, nmax=8000, seed=0)
    g = capi.GpuSystem([w.cfg for w in reps])
    orcs = []
    for r, w in enumerate(reps):
        g.set_rods(w.rods, replica=r)
        o = OracleSystem(w.cfg)
        o.set_rods(w.rods)
        orcs.append(o)
    for _ in range(5):
        g.step()
        for r, o in enumerate(orcs):
            so = o.step()
            sr = g.replica_stats(r)
            assert sr["nCollision"] == so["nCollision"] and sr["iterations"] == so["iterations"], r
    for r, o in enumerate(orcs):
        pg, qg = g.get_rods(r)
        po, qo = o.get_rods()
        assert np.array_equal(pg, po) and np.array_equal(qg, qo), r
