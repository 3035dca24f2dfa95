"""The protein binding step on the GPU (alens_protein_bind_step) against the
oracle (oracle/oracle_kmc.cpp): the same proteins, rods and Philox rolls
must give the same protein states bit for bit, step after step, with the
doubly bound proteins entering the rod solve as springs (FP64: the rods
stay bit-identical too).
"""
import numpy as np
import pytest

from alens_gb300 import capi, workloads
from alens_gb300.oracle_api import OracleSystem

pytestmark = pytest.mark.gpu

KBT = 0.00411
D = 0.025


def species():
    """Four species that exercise every branch at dt = 1e-4: plain rates,
    bind volume with load-dependent unbinding and PtoAPratio < 1, fixed end
    0 with PtoAPratio > 1, and the lookupType 1 stretch; motors walking both
    ways (fast enough to walk off rod ends within a few steps), drag, bound
    diffusion, clamped ends."""
    return [
        capi.make_protein_type(tag=0, rc=0.03, ko_s=(200.0, 150.0), Ka=(0.01, 0.012), ko_d=(100.0, 80.0),
                               Ke=(0.5, 0.4), eps=400.0, kappa=200.0, lambda_=0.0, freeLength=0.025,
                               diffUnbound=1.0, vmax=(50.0, 50.0), diffBoundS=(0.01, 0.01), fstall=2.0),
        capi.make_protein_type(tag=1, rc=0.025, ko_s=(120.0, 120.0), Ka=(0.02, 0.02), ko_d=(90.0, 90.0),
                               Ke=(0.2, 0.2), eps=400.0, kappa=150.0, lambda_=0.3, freeLength=0.03,
                               useBindVol=True, PtoAPratio=0.5, diffUnbound=2.0, vmax=(-80.0, 30.0),
                               vmaxAP=(-20.0, 10.0), vdrag=(True, False), diffBoundD=(0.02, 0.0), walkOff=False),
        capi.make_protein_type(tag=2, rc=0.04, ko_s=(60.0, 60.0), Ka=(0.01, 0.01), ko_d=(50.0, 70.0),
                               Ke=(0.6, 0.6), eps=300.0, kappa=300.0, lambda_=0.25822, freeLength=0.053,
                               fixedEnd0=True, PtoAPratio=2.0, diffUnbound=0.5, vmax=(0.0, 100.0)),
        capi.make_protein_type(tag=3, rc=0.035, ko_s=(150.0, 100.0), Ka=(0.015, 0.015), ko_d=(80.0, 80.0),
                               Ke=(0.8, 0.8), eps=400.0, kappa=100.0, lambda_=0.5, freeLength=0.05,
                               lookupType=1, diffUnbound=1.0, vmax=(40.0, -40.0), fstall=1.0,
                               diffBoundS=(0.005, 0.0), diffBoundD=(0.005, 0.005)),
    ]


def same(a, b):
    for f in ("gid", "type", "idBind"):
        assert np.array_equal(a[f], b[f]), f
    for f in ("distBind", "pos", "posEnd"):
        assert np.array_equal(a[f], b[f], equal_nan=True), f


def _pair(w, nprot, seed, steps, move=True, links=None, boundaries=None, motion=True):
    pairs = workloads.pair_list(OracleSystem, w.cfg, w.rods, 0.05)
    prots = workloads.protein_population(w.cfg, w.rods, nprot, pairs=pairs, seed=seed, ntypes=4)
    g = capi.GpuSystem(w.cfg)
    o = OracleSystem(w.cfg)
    for s in (g, o):
        s.set_rods(w.rods)
        if links is not None:
            s.set_links(links)
        if boundaries is not None:
            s.set_boundaries(boundaries)
        s.set_protein_types(species(), KBT, D)
    g.set_proteins(prots)
    o.set_proteins(prots)
    same(g.get_proteins(), o.get_proteins())
    totals = np.zeros(6, dtype=np.int64)
    for _ in range(steps):
        if motion:
            # TubuleSystem::step(): motion, then binding, then the rods
            mg = g.protein_motion_step()[0]
            mo = o.protein_motion_step()
            assert mg == mo, (mg, mo)
            totals[4:] += [mg["nSU"], mg["nDS"]]
            same(g.get_proteins(), o.get_proteins())
        sg = g.protein_bind_step()[0]
        so = o.protein_bind_step()
        assert sg == so, (sg, so)
        totals[:4] += [sg["nUS"], sg["nSU"], sg["nSD"], sg["nDS"]]
        same(g.get_proteins(), o.get_proteins())
        if move:
            rg = g.step()
            ro = o.step()
            assert rg["nBilateral"] == ro["nBilateral"] == sg["nD"] + (0 if links is None else len(links["i"]))
            assert rg["iterations"] == ro["iterations"]
            pg, qg = g.get_rods()
            po, qo = o.get_rods()
            assert np.array_equal(pg, po) and np.array_equal(qg, qo)
    return g, o, totals


def test_bind_steps_match_oracle_with_rod_steps(gpu_lib):
    w = workloads.small_periodic(n=1000, box=5.0, seed=7)
    g, o, tot = _pair(w, 4000, seed=7, steps=6)
    # every transition happened
    assert np.all(tot > 0), tot
    g.close()
    o.close()


def test_protein_steps_with_a_boundary(gpu_lib):
    """Unbound proteins that diffuse or walk off below a wall are moved onto
    it; rods get the wall's contacts in the same solve."""
    w = workloads.small_periodic(n=800, box=4.5, seed=5)
    w.cfg.simBoxPBC[2] = 0   # a wall in z: z is not periodic
    wall = capi.make_boundary(capi.BOUNDARY_WALL, center=(0.0, 0.0, 0.3), axis=(0.0, 0.0, 1.0))
    g, o, tot = _pair(w, 3000, seed=5, steps=4, boundaries=[wall])
    # after a motion step every unbound protein is on the allowed side
    assert g.protein_motion_step()[0] == o.protein_motion_step()
    q = g.get_proteins()
    same(q, o.get_proteins())
    unbound = (q["idBind"] < 0).all(axis=1)
    assert unbound.sum() > 0 and np.all(q["pos"][unbound, 2] >= 0.3 - 1e-12)
    g.close()
    o.close()


def test_bind_steps_with_user_links(gpu_lib):
    """Springs follow the alens_set_links links in the block order."""
    w = workloads.small_periodic(n=800, box=4.5, seed=3)
    pairs = workloads.pair_list(OracleSystem, w.cfg, w.rods, 0.05)
    links = workloads.make_links(w.cfg, w.rods, pairs, 60, seed=3)
    g, o, _ = _pair(w, 2000, seed=3, steps=3, links=links)
    cg, co = g.constraints(), o.constraints()
    assert np.array_equal(cg["i"], co["i"]) and np.array_equal(cg["j"], co["j"])
    assert np.array_equal(cg["gamma"], co["gamma"])
    g.close()
    o.close()


def test_dense_monolayer_proteins(gpu_lib):
    """The dense monolayer (20,000 rods) with 20,000 proteins of the
    symmetric crosslinker of its example configuration: two bind steps and
    the first rod step."""
    w = workloads.dense_monolayer()
    pairs = workloads.pair_list(OracleSystem, w.cfg, w.rods, 0.05)
    prots = workloads.protein_population(w.cfg, w.rods, 20000, pairs=pairs, seed=1)
    t = [capi.make_protein_type()]
    g = capi.GpuSystem(w.cfg)
    o = OracleSystem(w.cfg)
    for s in (g, o):
        s.set_rods(w.rods)
        s.set_protein_types(t, KBT, D)
        s.set_proteins(prots)
    for k in range(2):
        sg = g.protein_bind_step()[0]
        so = o.protein_bind_step()
        assert sg == so
        same(g.get_proteins(), o.get_proteins())
        if k == 0:
            assert g.step()["nBilateral"] == o.step()["nBilateral"]
    g.close()
    o.close()


def test_replicas_are_independent(gpu_lib):
    ws = [workloads.small_periodic(n=600, box=4.0, seed=s) for s in (11, 12)]
    cfgs = [ws[0].cfg, workloads.config_with(ws[1].cfg, rngSeed=99)]
    g = capi.GpuSystem(cfgs)
    g.set_protein_types(species(), KBT, D)
    orc = []
    for r, (w, c) in enumerate(zip(ws, cfgs)):
        pairs = workloads.pair_list(OracleSystem, c, w.rods, 0.05)
        prots = workloads.protein_population(c, w.rods, 1500 + 500 * r, pairs=pairs, seed=r, ntypes=4)
        g.set_rods(w.rods, replica=r)
        g.set_proteins(prots, replica=r)
        o = OracleSystem(c)
        o.set_rods(w.rods)
        o.set_protein_types(species(), KBT, D)
        o.set_proteins(prots)
        orc.append(o)
    for _ in range(3):
        sg = g.protein_bind_step()
        for r, o in enumerate(orc):
            assert sg[r] == o.protein_bind_step()
            same(g.get_proteins(replica=r), o.get_proteins())
        g.step()
        for o in orc:
            o.step()
    for r, o in enumerate(orc):
        pg, _ = g.get_rods(replica=r)
        po, _ = o.get_rods()
        assert np.array_equal(pg, po)
        o.close()
    g.close()


def test_protein_api_edges(gpu_lib):
    w = workloads.small_periodic(n=200, box=3.0, seed=1)
    g = capi.GpuSystem(w.cfg)
    g.set_rods(w.rods)
    # no species yet
    with pytest.raises(capi.AlensError):
        g.set_proteins(capi.protein_array(1))
    with pytest.raises(capi.AlensError):
        g.set_protein_types([capi.make_protein_type(lookupType=2)])
    g.set_protein_types([capi.make_protein_type()], KBT, D)
    # no proteins: a bind step is a no-op
    assert g.protein_bind_step()[0]["nU"] == 0
    p = capi.protein_array(3)
    p["gid"] = [5, 6, 7]
    p["pos"] = 1.0
    bad = p.copy()
    bad["idBind"][1, 0] = 200       # rod index out of range
    bad["distBind"][1, 0] = 0.0
    with pytest.raises(capi.AlensError):
        g.set_proteins(bad)
    g.set_proteins(p)
    got = g.get_proteins()
    assert np.array_equal(got["gid"], [5, 6, 7])
    st = g.protein_bind_step()[0]
    assert st["nU"] + st["nS"] == 3
    # removing them
    g.set_proteins(capi.protein_array(0))
    assert g.get_proteins().shape[0] == 0
    assert g.step()["nBilateral"] == 0
    g.close()
