"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle on
identical seeded inputs.

Bars: the pair list (indices and periodic images) is bit-exact in canonical
order; FP64 gamma, Jacobian and rod state agree within 1e-9 relative (the
shared arithmetic specification makes them bit-identical in practice, which
is also checked); iteration counts are equal.
"""
import numpy as np
import pytest

from alens_gb300 import capi, workloads
from alens_gb300.oracle_api import OracleSystem

pytestmark = pytest.mark.gpu

RTOL = 1e-9


def rel_err(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


def pair(cfg, rods):
    g = capi.GpuSystem(cfg)
    o = OracleSystem(cfg)
    g.set_rods(rods)
    o.set_rods(rods)
    return g, o


def compare_constraints(g, o, exact=True):
    cg, co = g.constraints(), o.constraints()
    assert cg["ncoll"] == co["ncoll"] and cg["nbil"] == co["nbil"]
    assert np.array_equal(cg["i"], co["i"])
    assert np.array_equal(cg["j"], co["j"])
    assert np.array_equal(cg["image"], co["image"])
    assert rel_err(cg["jac"], co["jac"]) <= RTOL
    assert rel_err(cg["delta0"], co["delta0"]) <= RTOL
    if exact:
        assert np.array_equal(cg["jac"], co["jac"])
        assert np.array_equal(cg["delta0"], co["delta0"])
    return cg, co


def compare_state(g, o, exact=True):
    pg, qg = g.get_rods()
    po, qo = o.get_rods()
    assert rel_err(pg, po) <= RTOL and rel_err(qg, qo) <= RTOL
    if exact:
        assert np.array_equal(pg, po) and np.array_equal(qg, qo)


@pytest.mark.parametrize("graph", [1, 0])
def test_small_periodic_staged(gpu_lib, graph):
    w = workloads.small_periodic(n=1000, box=5.0, seed=0)
    cfg = workloads.config_with(w.cfg, useGraph=graph)
    g, o = pair(cfg, w.rods)
    for step in range(4):
        sg, so = g.detect(), o.detect()
        assert sg["nCollision"] == so["nCollision"] > 0
        compare_constraints(g, o)
        sg, so = g.solve(), o.solve()
        assert sg["iterations"] == so["iterations"]
        assert sg["residual"] == so["residual"]
        cg, co = g.constraints(), o.constraints()
        assert rel_err(cg["gamma"], co["gamma"]) <= RTOL
        assert np.array_equal(cg["gamma"], co["gamma"])
        g.advance()
        o.advance()
        compare_state(g, o)
        vg, wg = g.get_velocity()
        vo, wo = o.get_velocity()
        assert rel_err(vg, vo) <= RTOL and rel_err(wg, wo) <= RTOL


@pytest.mark.parametrize("warm", [capi.WARM_ZERO, capi.WARM_PREV])
def test_trajectory_config1(gpu_lib, warm):
    """100 steps of the 1,000-rod periodic system (graph-replayed step)."""
    w = workloads.small_periodic(n=1000, box=5.0, seed=0)
    cfg = workloads.config_with(w.cfg, warmStart=warm)
    g, o = pair(cfg, w.rods)
    for step in range(100):
        sg = g.step()
        so = o.step()
        assert sg["nCollision"] == so["nCollision"], step
        assert sg["iterations"] == so["iterations"], step
        assert sg["converged"] == 1
    compare_state(g, o)
    cg, co = g.constraints(), o.constraints()
    assert np.array_equal(cg["gamma"], co["gamma"])
    assert np.array_equal(g.con_stress(), o.con_stress())
    assert g.step_count() == o.step_count() == 100


def test_quasi2d_slab(gpu_lib):
    w = workloads.dense_monolayer(n=3000, side=15.5, seed=3)
    g, o = pair(w.cfg, w.rods)
    for step in range(6):
        sg, so = g.step(), o.step()
        assert sg["nCollision"] == so["nCollision"] > 0
        assert sg["iterations"] == so["iterations"]
    compare_state(g, o)


def test_true_monolayer_in_plane(gpu_lib):
    """monolayer flag: motion confined to x-y on both sides."""
    rng = np.random.default_rng(2)
    n = 400
    pos = np.column_stack([rng.uniform(0, 8, n), rng.uniform(0, 8, n), np.full(n, 0.5)])
    phi = rng.uniform(0, np.pi, n)
    quat = workloads.axis_to_quat(np.column_stack([np.cos(phi), np.sin(phi), np.zeros(n)]))
    rods = capi.RodState(np.arange(n), pos, quat, rng.uniform(0.3, 0.6, n), np.full(n, 0.0125))
    # in-plane crossings cannot be relieved by in-plane motion, so some
    # steps may stop at the iteration cap; parity holds either way
    cfg = capi.make_config(box_high=(8, 8, 1), pbc=(1, 1, 0), monolayer=True, max_ite=400)
    g, o = pair(cfg, rods)
    for _ in range(5):
        sg, so = g.step(), o.step()
        assert sg["iterations"] == so["iterations"]
    compare_state(g, o)
    pg, _ = g.get_rods()
    assert np.all(pg[:, 2] == 0.5)


def test_tiny_box_images_and_self_pairs(gpu_lib):
    """Boxes with 1 or 2 cells per dimension: a pair can meet through several
    periodic images and a rod can touch its own image."""
    rng = np.random.default_rng(9)
    n = 60
    pos = rng.uniform(0, 1.2, (n, 3))
    axes = workloads.isotropic_axes(rng, n)
    length = rng.uniform(0.6, 1.1, n)
    # two parallel rods along x that overlap through images 0 and -1 in x
    pos[0], axes[0], length[0] = (0.6, 0.5, 0.5), (1, 0, 0), 1.1
    pos[1], axes[1], length[1] = (0.0, 0.52, 0.5), (1, 0, 0), 1.1
    quat = workloads.axis_to_quat(axes)
    rods = capi.RodState(np.arange(n), pos, quat, length, np.full(n, 0.0125))
    # x and z hold one cell, y two; the box is never smaller than the search
    # cutoff, so a rod cannot reach its own image
    cfg = capi.make_config(box_high=(1.2, 2.5, 1.2), pbc=(1, 1, 1), max_ite=5000)
    g, o = pair(cfg, rods)
    g.detect()
    o.detect()
    cg, co = compare_constraints(g, o)
    assert len(set(zip(cg["i"], cg["j"]))) < len(cg["i"]), "expected multi-image pairs"
    assert len(set(cg["image"])) > 5
    g.solve()
    o.solve()
    g.advance()
    o.advance()
    compare_state(g, o)


def test_spheres_and_immovable(gpu_lib):
    rng = np.random.default_rng(4)
    n = 500
    pos = rng.uniform(0, 3, (n, 3))
    quat = workloads.axis_to_quat(workloads.isotropic_axes(rng, n))
    length = np.where(rng.random(n) < 0.4, 0.0, rng.uniform(0.2, 0.8, n))
    radius = np.where(length == 0.0, 0.05, 0.0125)
    imm = (rng.random(n) < 0.1).astype(np.int32)
    rods = capi.RodState(np.arange(n) * 3 + 11, pos, quat, length, radius, imm)
    cfg = capi.make_config(box_high=(3, 3, 3), pbc=(1, 1, 1), max_ite=5000, seed=77)
    g, o = pair(cfg, rods)
    for _ in range(5):
        sg, so = g.step(), o.step()
        assert sg["nCollision"] == so["nCollision"] and sg["iterations"] == so["iterations"]
    compare_state(g, o)
    pg, _ = g.get_rods()
    assert np.array_equal(pg[imm == 1], rods.pos[imm == 1])


def make_links(rods, nlinks, box, seed, kappa=100.0, ell0=0.05):
    """Random bilateral springs between nearby rods (blocks built on the host
    the way setProteinConstraints builds them)."""
    rng = np.random.default_rng(seed)
    a = workloads.quat_to_axis(rods.quat)
    blocks = []
    n = rods.n
    tries = 0
    while len(blocks) < nlinks and tries < 100 * nlinks:
        tries += 1
        i, j = rng.integers(0, n, 2)
        if i == j:
            continue
        si = rng.uniform(-0.5, 0.5) * rods.length[i]
        sj = rng.uniform(-0.5, 0.5) * rods.length[j]
        P = rods.pos[i] + si * a[i]
        Q = rods.pos[j] + sj * a[j]
        d = P - Q
        d -= box * np.round(d / box)
        L = np.linalg.norm(d)
        if L > 0.6 or L < 1e-6:
            continue
        b = capi.AlensBlock()
        b.delta0 = L - ell0
        b.gamma = -b.delta0 * kappa
        b.gidI, b.gidJ = int(rods.gid[i]), int(rods.gid[j])
        b.globalIndexI, b.globalIndexJ = int(i), int(j)
        nI = d / L
        for k in range(3):
            b.normI[k] = nI[k]
            b.normJ[k] = -nI[k]
            b.posI[k] = si * a[i][k]
            b.posJ[k] = sj * a[j][k]
            b.labI[k] = P[k]
            b.labJ[k] = P[k] - d[k]
        b.oneSide = 1 if rng.random() < 0.05 else 0
        b.bilateral = 1
        b.kappa = kappa
        blocks.append(b)
    return blocks


def test_bilateral_blocks(gpu_lib):
    w = workloads.small_periodic(n=800, box=4.0, seed=21)
    g, o = pair(w.cfg, w.rods)
    for step in range(4):
        pos, quat = g.get_rods()
        rods = capi.RodState(w.rods.gid, pos, quat, w.rods.length, w.rods.radius)
        blocks = make_links(rods, 600, 4.0, seed=step)
        g.add_bilateral(blocks)
        o.add_bilateral(blocks)
        sg, so = g.step(), o.step()
        assert sg["nBilateral"] == so["nBilateral"] == len(blocks)
        assert sg["iterations"] == so["iterations"]
    compare_state(g, o)
    cg, co = g.constraints(), o.constraints()
    assert np.array_equal(cg["gamma"], co["gamma"])


def test_empty_and_contact_free(gpu_lib):
    cfg = capi.make_config(box_high=(5, 5, 5))
    g = capi.GpuSystem(cfg)
    g.set_rods(capi.RodState(np.zeros(0, np.int64), np.zeros((0, 3)), np.zeros((0, 4)), [], []))
    st = g.step()
    assert st["nCollision"] == 0 and st["converged"] == 1
    rods = capi.RodState([0, 1], [[1, 1, 1], [3, 3, 3]], workloads.axis_to_quat([[0, 0, 1], [1, 0, 0]]),
                         [0.5, 0.5], [0.0125, 0.0125])
    g2, o2 = pair(cfg, rods)
    for _ in range(3):
        assert g2.step()["nCollision"] == 0
        o2.step()
    compare_state(g2, o2)


def test_ensemble_matches_standalone(gpu_lib):
    reps = workloads.ensemble(nrep=5, nmin=200, nmax=1500, seed=3)
    g = capi.GpuSystem([w.cfg for w in reps])
    for r, w in enumerate(reps):
        g.set_rods(w.rods, replica=r)
    orcs = []
    for w in reps:
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
        assert np.array_equal(pg, po) and np.array_equal(qg, qo)


def test_capacity_fixed_and_autogrow(gpu_lib):
    dense = workloads.small_periodic(n=800, box=1.2, seed=2, max_ite=50)
    fixed = workloads.config_with(dense.cfg, maxConstraints=100)
    g = capi.GpuSystem(fixed)
    g.set_rods(dense.rods)
    with pytest.raises(capi.AlensError) as e:
        g.step()
    assert e.value.status == capi.ALENS_CAPACITY
    # automatic growth: far more pairs than the initial 4N+1024 guess
    g2, o2 = pair(dense.cfg, dense.rods)
    sg, so = g2.step(), o2.step()
    assert sg["nCollision"] == so["nCollision"] > 4 * 800 + 1024
    compare_state(g2, o2)


def test_nan_input_detected(gpu_lib):
    w = workloads.small_periodic(n=100, box=2.0, seed=1)
    bad = w.rods.copy()
    bad.quat[3, 0] = np.inf
    g = capi.GpuSystem(w.cfg)
    g.set_rods(bad)
    with pytest.raises(capi.AlensError) as e:
        g.step()
    assert e.value.status == capi.ALENS_NAN_DETECTED


def test_not_converged_reports_iterations(gpu_lib):
    dense = workloads.small_periodic(n=200, box=1.2, seed=2, max_ite=3)
    g, o = pair(dense.cfg, dense.rods)
    sg, so = g.step(), o.step()
    assert sg["rc"] == so["rc"] == capi.ALENS_NOT_CONVERGED
    assert sg["iterations"] == so["iterations"] == 3
    compare_state(g, o)


def test_mixed_precision_close_to_fp64(gpu_lib):
    w = workloads.small_periodic(n=1000, box=5.0, seed=0)
    cfg64 = w.cfg
    cfgmx = workloads.config_with(w.cfg, precision=capi.PREC_MIXED)
    g64 = capi.GpuSystem(cfg64)
    gmx = capi.GpuSystem(cfgmx)
    g64.set_rods(w.rods)
    gmx.set_rods(w.rods)
    for _ in range(3):
        s64 = g64.step()
        smx = gmx.step()
        assert smx["converged"] == 1 and smx["residual"] <= cfg64.conResTol
    p64, _ = g64.get_rods()
    pmx, _ = gmx.get_rods()
    assert rel_err(pmx, p64) <= 1e-6


def test_delassus_operator_bit_exact(gpu_lib):
    """The assembled operator A = dt D^T M D and the QP vectors equal the
    oracle's bit for bit (bilateral rows included)."""
    w = workloads.small_periodic(n=600, box=3.5, seed=8)
    g, o = pair(w.cfg, w.rods)
    blocks = make_links(w.rods, 200, 3.5, seed=5)
    g.add_bilateral(blocks)
    o.add_bilateral(blocks)
    g.detect()
    o.detect()
    opg = g.operator()
    opo = o.operator()
    assert np.array_equal(opg["rowPtr"], opo["rowPtr"])
    assert np.array_equal(opg["cols"], opo["cols"])
    assert np.array_equal(opg["vals"], opo["vals"])
    q, diag = o.solver_data()
    assert np.array_equal(opg["q"], q)
    assert np.all(opg["lb"][: opg["q"].shape[0] - len(blocks)] == 0.0)
    assert np.all(np.isneginf(opg["lb"][-len(blocks):]))


def test_device_crosslinks(gpu_lib):
    """Pre-bound crosslinkers: blocks built on the device every step equal
    the oracle's, and the trajectory stays bit-identical."""
    from alens_gb300.oracle_api import OracleSystem as Orc
    w = workloads.crosslinked_bundle_rods(n=1500, box=5.0, seed=3)
    pairs = workloads.pair_list(Orc, w.cfg, w.rods, 0.05)
    links = workloads.make_links(w.cfg, w.rods, pairs, 3000, seed=1)
    g, o = pair(w.cfg, w.rods)
    g.set_links(links)
    o.set_links(links)
    for _ in range(4):
        sg, so = g.step(), o.step()
        assert sg["nBilateral"] == so["nBilateral"] == 3000
        assert sg["iterations"] == so["iterations"]
    compare_state(g, o)
    cg, co = g.constraints(), o.constraints()
    assert np.array_equal(cg["gamma"], co["gamma"])
    assert np.array_equal(cg["delta0"], co["delta0"])


def _gamma_rel(a, b):
    """Relative L2 distance of two multiplier vectors.  Two solves that both
    stop at the residual tolerance differ by the tolerance's effect (about
    1e-4 of the largest multiplier element-wise); the L2 measure is the
    1e-4 relative bar, with an element-wise bar of 1e-3 beside it."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    scale = max(float(np.max(np.abs(b))), 1e-30)
    assert float(np.max(np.abs(a - b))) <= 2e-3 * scale
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def fp64_residual(system, replica=0):
    """Min-map residual max_k |x_k - max(lb_k, x_k - g_k)| of the system's
    current multipliers, g = (A + diag(cinv)) x + q, evaluated in numpy from
    the operator the library exports (independent of the solver's own
    residual)."""
    op = system.operator(replica)
    x = op["gamma0"]
    n = x.shape[0]
    rows = np.repeat(np.arange(n), np.diff(op["rowPtr"]))
    g = np.bincount(rows, weights=op["vals"] * x[op["cols"]], minlength=n) + op["cinv"] * x + op["q"]
    return float(np.max(np.abs(x - np.maximum(op["lb"], x - g)))) if n else 0.0


@pytest.mark.parametrize("form", ["grid", "cluster", "resident", "fast"])
def test_mixed_forms_match_fp64(gpu_lib, monkeypatch, form):
    """Every form of the FP32-bulk solver reaches the FP64 tolerance and
    stays close to the FP64 solution of the same step (relative L2 of the
    multipliers), with crosslink springs in the solve."""
    monkeypatch.setenv("ALENS_SOLVER_FORM", form)
    w = workloads.crosslinked_bundle_rods(n=1500, box=5.0, seed=3)
    from alens_gb300.oracle_api import OracleSystem as Orc
    pairs = workloads.pair_list(Orc, w.cfg, w.rods, 0.05)
    links = workloads.make_links(w.cfg, w.rods, pairs, 1500, seed=1)
    g64 = capi.GpuSystem(w.cfg)
    gmx = capi.GpuSystem(workloads.config_with(w.cfg, precision=capi.PREC_MIXED))
    for g in (g64, gmx):
        g.set_rods(w.rods)
        g.set_links(links)
    for _ in range(3):
        # same state into both, one step each, compare the step's solution
        pos, quat = g64.get_rods()
        gmx.update_rods(pos, quat)
        s64 = g64.step()
        smx = gmx.step()
        assert smx["converged"] == 1 and smx["residual"] <= w.cfg.conResTol
        assert smx["nCollision"] == s64["nCollision"]
        # the returned multipliers meet the tolerance in FP64, checked here
        assert fp64_residual(gmx) <= w.cfg.conResTol * 1.0001
        c64, cmx = g64.constraints(), gmx.constraints()
        # springs carry multipliers of order 1 while the residual bar is an
        # absolute 1e-5 um: two solves that each meet it (checked above)
        # differ by a few 1e-4
        assert _gamma_rel(cmx["gamma"], c64["gamma"]) <= 5e-4
    p64, _ = g64.get_rods()
    pmx, _ = gmx.get_rods()
    # the update of the last step carries that step's tolerance-level
    # multiplier difference (stiff springs)
    assert rel_err(pmx, p64) <= 1e-5


def test_resident_form_ensemble(gpu_lib, monkeypatch):
    """Cluster-resident solver over uneven replicas in one launch."""
    monkeypatch.setenv("ALENS_SOLVER_FORM", "resident")
    reps = workloads.ensemble(nrep=6, nmin=300, nmax=3000, seed=5)
    cfgs = [workloads.config_with(w.cfg, precision=capi.PREC_MIXED) for w in reps]
    g = capi.GpuSystem(cfgs)
    singles = []
    for r, w in enumerate(reps):
        g.set_rods(w.rods, replica=r)
        s = capi.GpuSystem(w.cfg)
        s.set_rods(w.rods)
        singles.append(s)
    for _ in range(3):
        for r, s in enumerate(singles):
            pos, quat = g.get_rods(r)
            s.update_rods(pos, quat)
        st = g.step()
        assert st["converged"] == 1
        for r, s in enumerate(singles):
            s.step()
            cr = g.constraints(r)
            cs = s.constraints()
            assert np.array_equal(cr["i"], cs["i"])
            assert fp64_residual(g, r) <= cfgs[r].conResTol * 1.0001
            # random initial overlaps: multipliers up to ~2, absolute 1e-5 um bar
            assert _gamma_rel(cr["gamma"], cs["gamma"]) <= 5e-4


def test_resident_form_falls_back_when_too_large(gpu_lib, monkeypatch):
    """More constraints than the clusters' shared memory holds: the step is
    rerun in grid form and still meets the tolerance."""
    monkeypatch.setenv("ALENS_SOLVER_FORM", "resident")
    w = workloads.small_periodic(n=250000, box=31.5, seed=4)   # ~4.5e4 constraints
    g = capi.GpuSystem(workloads.config_with(w.cfg, precision=capi.PREC_MIXED))
    g.set_rods(w.rods)
    g64 = capi.GpuSystem(w.cfg)
    g64.set_rods(w.rods)
    st = g.step()
    s64 = g64.step()
    assert st["nCollision"] == s64["nCollision"] > 16 * 2048
    assert st["converged"] == 1 and st["residual"] <= w.cfg.conResTol
    assert _gamma_rel(g.constraints()["gamma"], g64.constraints()["gamma"]) <= 3e-4


def test_autotune_keeps_fp64_parity(gpu_lib):
    """The autotuner only changes launch shapes: the FP64 trajectory after
    tuning still equals the oracle's bit for bit, and tuning does not move
    the rods."""
    w = workloads.small_periodic(n=1000, box=5.0, seed=0)
    g, o = pair(w.cfg, w.rods)
    rep = g.autotune(reps=2)
    assert rep["chosen"] >= 0 and len(rep["candidates"]) >= 2
    assert all(c["ms"] is not None for c in rep["candidates"])
    pg, _ = g.get_rods()
    assert np.array_equal(pg, w.rods.pos)
    for _ in range(5):
        sg, so = g.step(), o.step()
        assert sg["iterations"] == so["iterations"]
    compare_state(g, o)


@pytest.mark.parametrize("box,n,pbc", [(1.3, 300, (1, 1, 1)), (1.9, 600, (1, 1, 1)), (1.3, 300, (1, 1, 0))])
def test_dense_pair_search_stencil(gpu_lib, box, n, pbc):
    """Dense boxes (more than 24 rods per cutoff-sized cell) take the
    half-cutoff cells and the 5-cell stencil; with 2 or 3 cells per side
    the +-2 offsets wrap once across the periodic boundary (and are dropped
    where that still leaves the grid, or where the side is not periodic).
    The pair sets, multipliers and trajectory equal the oracle's bit for
    bit."""
    from alens_gb300 import workloads as wl
    w = wl.small_periodic(n=n, box=box, seed=3, lmin=0.5, lmax=1.0)
    cfg = wl.config_with(w.cfg, simBoxPBC=pbc)
    g, o = pair(cfg, w.rods)
    for _ in range(3):
        sg, so = g.step(), o.step()
        assert sg["nCollision"] == so["nCollision"] > 0
        assert sg["iterations"] == so["iterations"]
        compare_constraints(g, o)
    compare_state(g, o)


@pytest.mark.parametrize("min_tiles", [2, 3, 8])
def test_min_tiles_per_block_keeps_fp64_parity(gpu_lib, monkeypatch, min_tiles):
    """Fewer, fuller solver blocks (a minimum number of 64-row tiles per
    block) change only which block updates which rows: the FP64 trajectory
    equals the oracle's bit for bit, single system and ensemble."""
    monkeypatch.setenv("ALENS_SOLVER_MIN_TILES", str(min_tiles))
    w = workloads.small_periodic(n=1000, box=5.0, seed=0)
    g, o = pair(w.cfg, w.rods)
    for _ in range(4):
        sg, so = g.step(), o.step()
        assert sg["iterations"] == so["iterations"]
    compare_state(g, o)


def test_autotune_mixed_ensemble(gpu_lib):
    reps = workloads.ensemble(nrep=8, nmin=300, nmax=3000, seed=8)
    cfgs = [workloads.config_with(w.cfg, precision=capi.PREC_MIXED) for w in reps]
    g = capi.GpuSystem(cfgs)
    for r, w in enumerate(reps):
        g.set_rods(w.rods, replica=r)
    rep = g.autotune(reps=2)
    forms = {c["form"] for c in rep["candidates"]}
    assert {"grid", "cluster", "resident"} <= forms
    assert rep["chosen"] >= 0
    for _ in range(3):
        st = g.step()
        assert st["converged"] == 1
        for r in range(len(reps)):
            assert fp64_residual(g, r) <= cfgs[r].conResTol * 1.0001


def test_restart_step_count_continues_noise(gpu_lib):
    """A context restarted from the rods after step 3 with the step count set
    to 3 reproduces steps 3 and 4 of an uninterrupted run bit for bit (the
    step keys the Brownian noise), whether the count is set before the
    device state exists or after a step."""
    w = workloads.small_periodic(n=1000, box=5.0, seed=0)
    cfg = workloads.config_with(w.cfg, warmStart=capi.WARM_ZERO)
    a = capi.GpuSystem(cfg)
    a.set_rods(w.rods)
    for _ in range(3):
        a.step()
    p3, q3 = a.get_rods()
    for _ in range(2):
        a.step()
    p5, q5 = a.get_rods()
    r3 = w.rods.copy()
    r3.pos, r3.quat = p3.copy(), q3.copy()
    b = capi.GpuSystem(cfg)
    b.set_rods(r3)
    b.set_step_count(3)
    c = capi.GpuSystem(cfg)
    c.set_rods(w.rods)
    c.step()
    c.update_rods(p3, q3)
    c.set_step_count(3)
    for s in (b, c):
        s.step()
        s.step()
        assert s.step_count() == 5
        pb, qb = s.get_rods()
        assert np.array_equal(pb, p5) and np.array_equal(qb, q5)
    d = capi.GpuSystem(cfg)
    d.set_rods(r3)
    d.step()
    d.step()
    assert not np.array_equal(d.get_rods()[0], p5)
    with pytest.raises(capi.AlensError):
        b.set_step_count(-1)
    b.detect()
    with pytest.raises(capi.AlensError):
        b.set_step_count(7)  # a staged step is pending
