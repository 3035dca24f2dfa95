"""The allocation-free BBPGD entry point (alens_bbpgd_solve_noalloc).

It serves callers that cannot call cudaMalloc where they solve: a host code
whose GPU memory belongs to another allocator (a caching pool that has
reserved the device, or a fixed budget), or a time loop that must not stall
the device with an allocation.  Each test builds a step's operator with the
regular context API, then solves the same problem through the C ABI entry
point from device buffers owned by the test, twice in a row.  Each call must
return the gamma, status and iteration count of the regular solve
(alens_solve), within the 1e-9 relative bar of the other parity tests.

This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from alens_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _device_problem(op):
    torch = pytest.importorskip("torch")

    def dev(a, dt):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")

    return dict(rowPtr=dev(op["rowPtr"], torch.int32), cols=dev(op["cols"], torch.int32),
                vals=dev(op["vals"], torch.float64), q=dev(op["q"], torch.float64),
                cinv=dev(op["cinv"], torch.float64), lb=dev(op["lb"], torch.float64),
                g0=dev(op["gamma0"], torch.float64))


def _noalloc(lib, n, d, tol, max_ite):
    torch = pytest.importorskip("torch")
    out = torch.full((max(n, 1),), float("nan"), dtype=torch.float64, device="cuda")
    it = C.c_int(-1)
    res = C.c_double(-1.0)
    status = C.c_int(-1)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.alens_bbpgd_solve_noalloc(
        n, d["rowPtr"].data_ptr(), d["cols"].data_ptr(), d["vals"].data_ptr(), d["q"].data_ptr(),
        d["cinv"].data_ptr(), d["lb"].data_ptr(), d["g0"].data_ptr(), out.data_ptr(), tol, max_ite,
        C.c_void_p(stream), C.byref(it), C.byref(res), C.byref(status))
    return rc, out.cpu().numpy()[:n], it.value, res.value, status.value


def _check_against_context(cfg, rods, links=None, expect=capi.ALENS_OK):
    g = capi.GpuSystem(cfg)
    g.set_rods(rods)
    if links is not None:
        g.set_links(links)
    g.detect()
    op = g.operator()                    # operator and initial gamma
    st = g.solve(allow_not_converged=True)
    ref = g.constraints()["gamma"]
    g.close()
    assert st["rc"] == expect, st
    n = op["q"].shape[0]
    assert n > 100
    d = _device_problem(op)
    lib = capi.load_library()
    for call in range(2):
        rc, got, it, res, status = _noalloc(lib, n, d, cfg.conResTol, cfg.conMaxIte)
        assert rc == expect, (call, rc)
        assert status == expect, (call, status)
        err = float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)))
        assert err <= 1e-9, (call, err)
        assert it == st["iterations"], (call, it, st["iterations"])
        if expect == capi.ALENS_OK:
            assert res <= cfg.conResTol
    return op


def test_noalloc_solve_matches_context_solve(gpu_lib):
    w = workloads.small_periodic(n=1500, box=5.0, seed=4)
    _check_against_context(w.cfg, w.rods)


def test_noalloc_bilateral_rows_match_context_solve(gpu_lib):
    """Crosslinker rows: no lower bound (lb = -inf) and compliance 1/kappa."""
    w = workloads.small_periodic(n=1500, box=5.0, seed=5)
    pairs = workloads.pair_list(capi.GpuSystem, w.cfg, w.rods, 0.05)
    links = workloads.make_links(w.cfg, w.rods, pairs, 400, seed=5)
    op = _check_against_context(w.cfg, w.rods, links=links)
    assert np.isneginf(op["lb"]).sum() == 400
    assert np.count_nonzero(op["cinv"]) == 400


def test_noalloc_iteration_cap_matches_context_solve(gpu_lib):
    """With a cap of 3 iterations both solves stop unconverged after 3 and
    return the same last iterate."""
    w = workloads.small_periodic(n=1500, box=5.0, seed=4)
    cfg = workloads.config_with(w.cfg, conMaxIte=3, conResTol=1e-12)
    _check_against_context(cfg, w.rods, expect=capi.ALENS_NOT_CONVERGED)


def test_noalloc_empty_problem(gpu_lib):
    lib = capi.load_library()
    it = C.c_int(-1)
    res = C.c_double(-1.0)
    status = C.c_int(-1)
    rc = lib.alens_bbpgd_solve_noalloc(0, None, None, None, None, None, None, None, None, 1e-5, 10,
                                       None, C.byref(it), C.byref(res), C.byref(status))
    assert rc == capi.ALENS_OK
    assert (it.value, res.value, status.value) == (0, 0.0, capi.ALENS_OK)


def test_noalloc_rejects_column_out_of_range(gpu_lib):
    """A column index >= n is skipped by the kernel's bounds check and
    reported; the next call with a valid operator still converges."""
    w = workloads.small_periodic(n=1500, box=5.0, seed=4)
    g = capi.GpuSystem(w.cfg)
    g.set_rods(w.rods)
    g.detect()
    op = g.operator()
    g.close()
    n = op["q"].shape[0]
    bad = dict(op)
    bad["cols"] = op["cols"].copy()
    bad["cols"][len(bad["cols"]) // 2] = n + 7
    lib = capi.load_library()
    rc, _, _, _, _ = _noalloc(lib, n, _device_problem(bad), w.cfg.conResTol, w.cfg.conMaxIte)
    assert rc == capi.ALENS_INVALID_ARG
    rc, got, _, res, status = _noalloc(lib, n, _device_problem(op), w.cfg.conResTol, w.cfg.conMaxIte)
    assert rc == capi.ALENS_OK and status == capi.ALENS_OK and res <= w.cfg.conResTol
    assert np.all(np.isfinite(got))


def test_noalloc_rejects_oversize(gpu_lib):
    lib = capi.load_library()
    it = C.c_int(0)
    rc = lib.alens_bbpgd_solve_noalloc(65537, None, None, None, None, None, None, None, None, 1e-5, 10,
                                       None, C.byref(it), None, None)
    assert rc == capi.ALENS_INVALID_ARG
