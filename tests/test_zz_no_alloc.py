"""The allocation-free BBPGD entry point (alens_bbpgd_solve_noalloc).

It serves callers that cannot call cudaMalloc where they solve, such as a
time step recorded into a CUDA graph, or a GPU whose memory belongs to a
pool the caller must not disturb.  The test builds a step's operator with
the regular context API, then solves the same problem through the C ABI
entry point twice in a row from device buffers owned by the test.  Each
call must return the gamma and iteration count of the regular solve
(alens_solve), within the 1e-9 relative bar of the other parity tests.

This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from alens_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def test_noalloc_solve_matches_context_solve(gpu_lib):
    torch = pytest.importorskip("torch")
    w = workloads.small_periodic(n=1500, box=5.0, seed=4)
    g = capi.GpuSystem(w.cfg)
    g.set_rods(w.rods)
    g.detect()
    op = g.operator()                    # operator and initial gamma
    st = g.solve()
    ref = g.constraints()["gamma"]
    n = op["q"].shape[0]
    assert n > 100

    def dev(a, dt):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")

    rowPtr = dev(op["rowPtr"], torch.int32)
    cols = dev(op["cols"], torch.int32)
    vals = dev(op["vals"], torch.float64)
    q = dev(op["q"], torch.float64)
    cinv = dev(op["cinv"], torch.float64)
    lb = dev(op["lb"], torch.float64)
    g0 = dev(op["gamma0"], torch.float64)
    stream = torch.cuda.current_stream().cuda_stream
    lib = capi.load_library()
    for call in range(2):
        out = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        it = C.c_int(-1)
        res = C.c_double(-1.0)
        status = C.c_int(-1)
        rc = lib.alens_bbpgd_solve_noalloc(
            n, rowPtr.data_ptr(), cols.data_ptr(), vals.data_ptr(), q.data_ptr(), cinv.data_ptr(),
            lb.data_ptr(), g0.data_ptr(), out.data_ptr(), w.cfg.conResTol, w.cfg.conMaxIte,
            C.c_void_p(stream), C.byref(it), C.byref(res), C.byref(status))
        assert rc == capi.ALENS_OK, (call, rc)
        assert status.value == capi.ALENS_OK
        got = out.cpu().numpy()
        err = float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)))
        assert err <= 1e-9, (call, err)
        assert it.value == st["iterations"], (call, it.value, st["iterations"])
        assert res.value <= w.cfg.conResTol


def test_noalloc_rejects_oversize(gpu_lib):
    lib = capi.load_library()
    it = C.c_int(0)
    rc = lib.alens_bbpgd_solve_noalloc(65537, None, None, None, None, None, None, None, None, 1e-5, 10,
                                       None, C.byref(it), None, None)
    assert rc == capi.ALENS_INVALID_ARG
