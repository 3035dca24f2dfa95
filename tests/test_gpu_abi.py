"""C ABI entry points named by the drop-in boundary (alens_get_pairs,
alens_get_gamma, alens_step_batched) and the bounded-wait path of the
solver (alens_set_wait_limit), on the GPU.

The timeout test makes the solver's grid barriers wait for one block more
than the launch holds, so the real bounded wait runs out inside its limit:
the step must return ALENS_TIMEOUT with the rods unmoved and the step count
unchanged, and the next step on the same context, with the hook removed,
must match the oracle bit for bit (FP64) or converge (mixed precision).
Nothing faults; every wait ends by its own limit.
"""
import ctypes as C

import numpy as np
import pytest

from alens_gb300 import capi, workloads
from alens_gb300.oracle_api import OracleSystem

pytestmark = pytest.mark.gpu


def _pairs(g):
    n = C.c_int()
    rc = g.lib.alens_get_pairs(g.h, 0, 0, C.byref(n), None, None, None)
    assert rc == capi.ALENS_CAPACITY or (rc == capi.ALENS_OK and n.value == 0)
    ii = np.empty(n.value, np.int32)
    jj = np.empty(n.value, np.int32)
    im = np.empty(n.value, np.int32)
    rc = g.lib.alens_get_pairs(g.h, 0, n.value, C.byref(n), ii.ctypes.data_as(C.POINTER(C.c_int32)),
                               jj.ctypes.data_as(C.POINTER(C.c_int32)), im.ctypes.data_as(C.POINTER(C.c_int32)))
    assert rc == capi.ALENS_OK
    return ii, jj, im


def _gamma(g):
    n = C.c_int()
    g.lib.alens_get_gamma(g.h, 0, 0, C.byref(n), None, None)
    pairs = np.empty(2 * n.value, np.int32)
    gam = np.empty(n.value)
    rc = g.lib.alens_get_gamma(g.h, 0, n.value, C.byref(n), pairs.ctypes.data_as(C.POINTER(C.c_int32)),
                               gam.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == capi.ALENS_OK
    return pairs.reshape(-1, 2), gam


def test_pairs_and_gamma_getters_match_constraints(gpu_lib):
    w = workloads.small_periodic(n=1000, box=5.0, seed=3)
    pairs_ = workloads.pair_list(capi.GpuSystem, w.cfg, w.rods, 0.05)
    links = workloads.make_links(w.cfg, w.rods, pairs_, 100, seed=3)
    g = capi.GpuSystem(w.cfg)
    g.set_rods(w.rods)
    g.set_links(links)
    o = OracleSystem(w.cfg)
    o.set_rods(w.rods)
    o.set_links(links)
    g.detect()
    o.detect()
    ii, jj, im = _pairs(g)
    co = o.constraints()
    nc = co["ncoll"]
    assert np.array_equal(ii, co["i"][:nc]) and np.array_equal(jj, co["j"][:nc])
    assert np.array_equal(im, co["image"][:nc])
    g.solve()
    o.solve()
    pairs, gam = _gamma(g)
    co = o.constraints()
    assert gam.shape[0] == nc + 100
    assert np.array_equal(pairs[:, 0], co["i"]) and np.array_equal(pairs[:, 1], co["j"])
    assert np.array_equal(gam, co["gamma"])
    n = C.c_int()
    assert g.lib.alens_get_gamma(g.h, 0, 3, C.byref(n), None, None) == capi.ALENS_CAPACITY
    assert n.value == nc + 100
    g.close()
    o.close()


def test_step_batched_matches_separate_contexts(gpu_lib):
    """Three independent systems stepped together equal the same systems
    stepped one by one (FP64: bit for bit), and the oracle."""
    ws = [workloads.small_periodic(n=n, box=b, seed=s) for n, b, s in ((600, 4.0, 1), (900, 4.5, 2), (300, 3.0, 3))]
    batch = [capi.GpuSystem(w.cfg) for w in ws]
    single = [capi.GpuSystem(w.cfg) for w in ws]
    orc = [OracleSystem(w.cfg) for w in ws]
    for w, a, b_, o in zip(ws, batch, single, orc):
        a.set_rods(w.rods)
        b_.set_rods(w.rods)
        o.set_rods(w.rods)
    arr = (C.c_void_p * 3)(*[g.h.value for g in batch])
    stats = (capi.AlensStepStats * 3)()
    lib = batch[0].lib
    for _ in range(3):
        rc = lib.alens_step_batched(arr, 3, stats)
        assert rc in (capi.ALENS_OK, capi.ALENS_NOT_CONVERGED)
        for k in range(3):
            sb = single[k].step()
            so = orc[k].step()
            assert stats[k].iterations == sb["iterations"] == so["iterations"]
            assert stats[k].nCollision == sb["nCollision"] == so["nCollision"]
    for a, b_, o in zip(batch, single, orc):
        pa, qa = a.get_rods()
        pb, qb = b_.get_rods()
        po, qo = o.get_rods()
        assert np.array_equal(pa, pb) and np.array_equal(qa, qb)
        assert np.array_equal(pa, po) and np.array_equal(qa, qo)
        assert a.step_count() == 3
    for g in batch + single:
        g.close()
    for o in orc:
        o.close()
    assert lib.alens_step_batched(None, 2, None) == capi.ALENS_INVALID_ARG
    assert lib.alens_step_batched(None, 0, None) == capi.ALENS_OK


@pytest.mark.parametrize("precision", [capi.PREC_FP64, capi.PREC_MIXED])
def test_solver_wait_runs_out_then_recovers(gpu_lib, precision):
    w = workloads.small_periodic(n=1000, box=5.0, seed=0)
    cfg = workloads.config_with(w.cfg, precision=precision)
    g = capi.GpuSystem(cfg)
    g.set_rods(w.rods)
    o = OracleSystem(w.cfg)
    o.set_rods(w.rods)
    p0, q0 = g.get_rods()
    lib = g.lib
    # every grid-barrier wait gives up after 2 ms: the step ends with a timeout
    assert lib.alens_set_wait_limit(g.h, 2_000_000, 1) == capi.ALENS_OK
    st = capi.AlensStepStats()
    assert lib.alens_step(g.h, C.byref(st)) == capi.ALENS_TIMEOUT
    p1, q1 = g.get_rods()
    assert np.array_equal(p0, p1) and np.array_equal(q0, q1)
    assert g.step_count() == 0
    assert lib.alens_set_wait_limit(g.h, 0, 2) == capi.ALENS_INVALID_ARG
    # hook removed: the same context steps normally
    assert lib.alens_set_wait_limit(g.h, 0, 0) == capi.ALENS_OK
    for _ in range(2):
        sg = g.step()
        so = o.step()
        assert sg["converged"] == 1
        assert sg["nCollision"] == so["nCollision"]
    pg, qg = g.get_rods()
    po, qo = o.get_rods()
    if precision == capi.PREC_FP64:
        assert np.array_equal(pg, po) and np.array_equal(qg, qo)
    else:
        assert float(np.max(np.abs(pg - po))) <= 1e-6
    assert g.step_count() == 2
    g.close()
    o.close()


def test_conblock_snapshot_carries_the_solve(gpu_lib, tmp_path):
    """write_snapshot(blocks=...) writes ConBlock_<id>.pvtp whose arrays are
    the step's constraints: multipliers, separations, crosslink stiffness, and
    per-block stresses that sum to the replica's pair virial."""
    import re
    from alens_gb300 import io
    w = workloads.small_periodic(n=1000, box=5.0, seed=3)
    pairs_ = workloads.pair_list(capi.GpuSystem, w.cfg, w.rods, 0.05)
    links = workloads.make_links(w.cfg, w.rods, pairs_, 100, seed=3)
    g = capi.GpuSystem(w.cfg)
    g.set_rods(w.rods)
    g.set_links(links)
    g.step()
    blocks = g.constraint_blocks()
    c = g.constraints()
    pos, quat = g.get_rods()
    rods = capi.RodState(w.rods.gid, pos, quat, w.rods.length, w.rods.radius)
    folder = io.write_snapshot(0, rods, step=1, time=1e-4, root=str(tmp_path / "result"), blocks=blocks,
                               info_path=str(tmp_path / "TimeStepInfo.txt"))
    text = open(folder + "ConBlock_r0_0.vtp").read()

    def arr(name, dtype):
        m = re.search(rf'Name="{name}" NumberOfComponents="\d+" format="binary">([^<]*)<', text)
        return io.read_vtk_binary_array(m.group(1), dtype)

    n = c["gamma"].shape[0]
    assert f'NumberOfLines="{n}"' in text
    assert np.array_equal(arr("gamma", "<f8"), c["gamma"])
    assert np.array_equal(arr("delta0", "<f8"), c["delta0"])
    assert np.array_equal(arr("globalIndexI", "<i4"), c["i"])
    kap = arr("kappa", "<f8")
    assert np.allclose(kap[c["ncoll"]:], 100.0) and np.all(kap[:c["ncoll"]] == 0.0)
    assert int(arr("bilateral", "<i4").sum()) == 100
    stress = arr("Stress", "<f8").reshape(-1, 3, 3).sum(axis=0)
    assert np.allclose(stress, g.con_stress(), rtol=1e-12, atol=1e-15)
    pts = arr("position", "<f8").reshape(-1, 3)
    assert np.array_equal(pts[0::2], blocks["labI"]) and np.array_equal(pts[1::2], blocks["labJ"])
    g.close()
