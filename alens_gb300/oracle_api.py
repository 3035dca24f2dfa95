"""ctypes wrapper of the CPU oracle (``oracle/liboracle.so``).

Test infrastructure: imported only by ``tests/``, the smoke check and the
CPU-baseline leg of ``bench.py``.  It mirrors :class:`alens_gb300.capi.GpuSystem`
for a single system so that parity tests read the same on both sides.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build
from .capi import (ALENS_CAPACITY, ALENS_NOT_CONVERGED, ALENS_OK, PROTEIN_DTYPE, AlensBlock, AlensBoundary,
                   AlensConfig, AlensError, AlensKmcStats, AlensProteinType, AlensStepStats, RodState, _p)

_PD = C.POINTER(C.c_double)
_PI32 = C.POINTER(C.c_int32)
_PI64 = C.POINTER(C.c_int64)
_PU32 = C.POINTER(C.c_uint32)

_OLIB = None


def load_oracle(rebuild: bool = True) -> C.CDLL:
    global _OLIB
    if _OLIB is not None:
        return _OLIB
    path = _build.build_oracle() if rebuild else _build.oracle_path()
    lib = C.CDLL(str(path))
    vp = C.c_void_p
    sigs = {
        "orc_create": (C.c_int, [C.POINTER(AlensConfig), C.POINTER(vp)]),
        "orc_destroy": (C.c_int, [vp]),
        "orc_set_rods": (C.c_int, [vp, C.c_int, _PI64, _PD, _PD, _PD, _PD, _PI32]),
        "orc_update_rods": (C.c_int, [vp, C.c_int, _PD, _PD]),
        "orc_get_rods": (C.c_int, [vp, C.c_int, _PD, _PD]),
        "orc_get_velocity": (C.c_int, [vp, C.c_int, _PD, _PD]),
        "orc_get_known_velocity": (C.c_int, [vp, C.c_int, _PD]),
        "orc_add_bilateral": (C.c_int, [vp, C.c_int, C.POINTER(AlensBlock)]),
        "orc_set_initial_gamma": (C.c_int, [vp, C.c_int, _PD]),
        "orc_set_boundaries": (C.c_int, [vp, C.c_int, C.POINTER(AlensBoundary)]),
        "orc_set_links": (C.c_int, [vp, C.c_int, _PI32, _PI32, _PD, _PD, _PD, _PD]),
        "orc_step": (C.c_int, [vp, C.POINTER(AlensStepStats)]),
        "orc_detect": (C.c_int, [vp, C.POINTER(AlensStepStats)]),
        "orc_solve": (C.c_int, [vp, C.POINTER(AlensStepStats)]),
        "orc_advance": (C.c_int, [vp, C.POINTER(AlensStepStats)]),
        "orc_get_num_constraints": (C.c_int, [vp, _PI32, _PI32]),
        "orc_get_constraints": (C.c_int, [vp, C.c_int, _PI32, _PI32, _PI32, _PD, _PD, _PD]),
        "orc_get_con_stress": (C.c_int, [vp, _PD]),
        "orc_get_step_count": (C.c_int, [vp, _PI64]),
        "orc_get_solver_data": (C.c_int, [vp, C.c_int, _PD, _PD]),
        "orc_get_operator": (C.c_int, [vp, C.c_int, _PI32, _PI32, _PI32, _PD]),
        "orc_set_threads": (C.c_int, [C.c_int]),
        "orc_dcp": (None, [_PD, _PD, C.c_double, _PD, _PD, C.c_double, _PD, _PD, _PD, _PD, _PD]),
        "orc_log": (C.c_double, [C.c_double]),
        "orc_sincos": (None, [C.c_double, _PD, _PD]),
        "orc_philox4x32": (None, [_PU32, _PU32, _PU32]),
        "orc_normals6": (None, [C.c_uint64, C.c_int64, C.c_int64, _PD]),
        "orc_canon_sum": (C.c_double, [_PD, C.c_int64]),
        "orc_mobility": (None, [C.c_double, C.c_double, C.c_double, _PD]),
        "orc_set_protein_types": (C.c_int, [vp, C.c_int, C.POINTER(AlensProteinType), C.c_double, C.c_double]),
        "orc_set_proteins": (C.c_int, [vp, C.c_int, vp]),
        "orc_get_proteins": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int), vp]),
        "orc_protein_bind_step": (C.c_int, [vp, C.POINTER(AlensKmcStats)]),
        "orc_protein_motion_step": (C.c_int, [vp, C.POINTER(AlensKmcStats)]),
        "orc_kmc_exp": (C.c_double, [C.c_double]),
        "orc_kmc_expf": (C.c_float, [C.c_float]),
        "orc_kmc_sd_integral": (C.c_double, [C.POINTER(AlensProteinType), C.c_double, C.c_double, C.c_double,
                                             C.c_double, C.c_double, C.c_double]),
        "orc_kmc_sd_invert": (C.c_double, [C.POINTER(AlensProteinType), C.c_double, C.c_double, C.c_double,
                                           C.c_double, C.c_double, C.c_double, C.c_double]),
        "orc_kmc_bind_volume": (C.c_double, [C.POINTER(AlensProteinType), C.c_double, C.c_double]),
        "orc_kmc_binding_factor_sd": (C.c_double, [C.POINTER(AlensProteinType), C.c_int, _PD, _PD]),
        "orc_kmc_type_constants": (None, [C.POINTER(AlensProteinType), C.c_double, C.c_double, C.c_double, _PD]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _OLIB = lib
    return lib


def set_threads(n: int) -> int:
    return load_oracle().orc_set_threads(int(n))


def dcp(c1, u1, h1, c2, u2, h2):
    lib = load_oracle()
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (c1, u1, c2, u2)]
    s = C.c_double()
    t = C.c_double()
    P = np.empty(3)
    Q = np.empty(3)
    dist = C.c_double()
    lib.orc_dcp(_p(a[0], C.c_double), _p(a[1], C.c_double), float(h1), _p(a[2], C.c_double),
                _p(a[3], C.c_double), float(h2), C.byref(s), C.byref(t), _p(P, C.c_double),
                _p(Q, C.c_double), C.byref(dist))
    return s.value, t.value, P, Q, dist.value


def det_log(x: float) -> float:
    return load_oracle().orc_log(float(x))


def det_sincos(x: float):
    s = C.c_double()
    c = C.c_double()
    load_oracle().orc_sincos(float(x), C.byref(s), C.byref(c))
    return s.value, c.value


def philox4x32(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.empty(4, np.uint32)
    load_oracle().orc_philox4x32(_p(c, C.c_uint32), _p(k, C.c_uint32), _p(out, C.c_uint32))
    return out


def normals6(seed: int, gid: int, step: int):
    z = np.empty(6)
    load_oracle().orc_normals6(int(seed), int(gid), int(step), _p(z, C.c_double))
    return z


def canon_sum(v) -> float:
    v = np.ascontiguousarray(v, dtype=np.float64)
    return load_oracle().orc_canon_sum(_p(v, C.c_double), int(v.shape[0]))


def mobility(length: float, radius: float, viscosity: float):
    out = np.empty(3)
    load_oracle().orc_mobility(float(length), float(radius), float(viscosity), _p(out, C.c_double))
    return out


def kmc_exp(x: float) -> float:
    return load_oracle().orc_kmc_exp(float(x))


def kmc_expf(x: float) -> float:
    return load_oracle().orc_kmc_expf(float(x))


def kmc_sd_integral(ptype: AlensProteinType, kbt: float, d: float, dt: float, d2: float, sA: float,
                    sB: float) -> float:
    return load_oracle().orc_kmc_sd_integral(C.byref(ptype), kbt, d, dt, d2, sA, sB)


def kmc_sd_invert(ptype: AlensProteinType, kbt: float, d: float, dt: float, d2: float, sA: float, sB: float,
                  target: float) -> float:
    return load_oracle().orc_kmc_sd_invert(C.byref(ptype), kbt, d, dt, d2, sA, sB, target)


def kmc_bind_volume(ptype: AlensProteinType, kbt: float, d: float) -> float:
    return load_oracle().orc_kmc_bind_volume(C.byref(ptype), kbt, d)


def kmc_binding_factor_sd(ptype: AlensProteinType, end: int, dir_bound, dir_rod) -> float:
    a = np.ascontiguousarray(dir_bound, dtype=np.float64)
    b = np.ascontiguousarray(dir_rod, dtype=np.float64)
    return load_oracle().orc_kmc_binding_factor_sd(C.byref(ptype), int(end), _p(a, C.c_double), _p(b, C.c_double))


def kmc_type_constants(ptype: AlensProteinType, kbt: float, d: float, dt: float) -> dict:
    out = np.zeros(12)
    load_oracle().orc_kmc_type_constants(C.byref(ptype), kbt, d, dt, _p(out, C.c_double))
    keys = ("rcap", "rOuter", "A", "w", "usCoef0", "usCoef1", "suProb0", "suProb1", "sdCoef0", "sdCoef1",
            "koD0", "koD1")
    return dict(zip(keys, out.tolist()))


def _ck(rc, where, ok=(ALENS_OK,)):
    if rc not in ok:
        raise AlensError(rc, where)
    return rc


class OracleSystem:
    """One oracle context (single system)."""

    def __init__(self, cfg: AlensConfig):
        self.lib = load_oracle()
        self.h = C.c_void_p()
        _ck(self.lib.orc_create(C.byref(cfg), C.byref(self.h)), "orc_create")
        self.n = 0

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_rods(self, rods: RodState):
        _ck(self.lib.orc_set_rods(self.h, rods.n, _p(rods.gid, C.c_int64), _p(rods.pos, C.c_double),
                                  _p(rods.quat, C.c_double), _p(rods.length, C.c_double),
                                  _p(rods.radius, C.c_double), _p(rods.immovable, C.c_int32)),
            "orc_set_rods")
        self.n = rods.n

    def update_rods(self, pos, quat):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        quat = np.ascontiguousarray(quat, dtype=np.float64)
        _ck(self.lib.orc_update_rods(self.h, self.n, _p(pos, C.c_double), _p(quat, C.c_double)),
            "orc_update_rods")

    def get_rods(self):
        pos = np.empty((self.n, 3))
        quat = np.empty((self.n, 4))
        _ck(self.lib.orc_get_rods(self.h, self.n, _p(pos, C.c_double), _p(quat, C.c_double)),
            "orc_get_rods")
        return pos, quat

    def get_velocity(self):
        v = np.empty((self.n, 3))
        w = np.empty((self.n, 3))
        _ck(self.lib.orc_get_velocity(self.h, self.n, _p(v, C.c_double), _p(w, C.c_double)),
            "orc_get_velocity")
        return v, w

    def known_velocity(self):
        u = np.empty((self.n, 6))
        _ck(self.lib.orc_get_known_velocity(self.h, self.n, _p(u, C.c_double)), "orc_get_known_velocity")
        return u

    def add_bilateral(self, blocks):
        arr = (AlensBlock * len(blocks))(*blocks)
        _ck(self.lib.orc_add_bilateral(self.h, len(blocks), arr), "orc_add_bilateral")

    def set_links(self, links):
        a = [np.ascontiguousarray(links[k], dtype=t) for k, t in
             (("i", np.int32), ("j", np.int32), ("si", np.float64), ("sj", np.float64), ("rest", np.float64),
              ("kappa", np.float64))]
        _ck(self.lib.orc_set_links(self.h, int(a[0].shape[0]), _p(a[0], C.c_int32), _p(a[1], C.c_int32),
                                   _p(a[2], C.c_double), _p(a[3], C.c_double), _p(a[4], C.c_double),
                                   _p(a[5], C.c_double)), "orc_set_links")

    def set_protein_types(self, types, kbt: float = 0.00411, rod_diameter: float = 0.025):
        arr = (AlensProteinType * max(len(types), 1))(*types)
        _ck(self.lib.orc_set_protein_types(self.h, len(types), arr, float(kbt), float(rod_diameter)),
            "orc_set_protein_types")

    def set_proteins(self, proteins: np.ndarray):
        a = np.ascontiguousarray(proteins, dtype=PROTEIN_DTYPE)
        _ck(self.lib.orc_set_proteins(self.h, int(a.shape[0]), a.ctypes.data if a.size else None),
            "orc_set_proteins")

    def get_proteins(self) -> np.ndarray:
        n = C.c_int()
        _ck(self.lib.orc_get_proteins(self.h, 0, C.byref(n), None), "orc_get_proteins", ok=(ALENS_OK, ALENS_CAPACITY))
        a = np.zeros(n.value, dtype=PROTEIN_DTYPE)
        _ck(self.lib.orc_get_proteins(self.h, n.value, C.byref(n), a.ctypes.data if a.size else None),
            "orc_get_proteins")
        return a

    def protein_bind_step(self) -> dict:
        st = AlensKmcStats()
        _ck(self.lib.orc_protein_bind_step(self.h, C.byref(st)), "orc_protein_bind_step")
        return st.as_dict()

    def protein_motion_step(self) -> dict:
        st = AlensKmcStats()
        _ck(self.lib.orc_protein_motion_step(self.h, C.byref(st)), "orc_protein_motion_step")
        return st.as_dict()

    def set_boundaries(self, boundaries):
        arr = (AlensBoundary * max(len(boundaries), 1))(*boundaries)
        _ck(self.lib.orc_set_boundaries(self.h, len(boundaries), arr), "orc_set_boundaries")

    def set_initial_gamma(self, gamma):
        g = np.ascontiguousarray(gamma, dtype=np.float64)
        _ck(self.lib.orc_set_initial_gamma(self.h, int(g.shape[0]), _p(g, C.c_double)),
            "orc_set_initial_gamma")

    def _stage(self, fn, name, ok=(ALENS_OK,)):
        st = AlensStepStats()
        rc = fn(self.h, C.byref(st))
        _ck(rc, name, ok)
        d = st.as_dict()
        d["rc"] = rc
        return d

    def step(self, allow_not_converged=True):
        ok = (ALENS_OK, ALENS_NOT_CONVERGED) if allow_not_converged else (ALENS_OK,)
        return self._stage(self.lib.orc_step, "orc_step", ok)

    def detect(self):
        return self._stage(self.lib.orc_detect, "orc_detect")

    def solve(self, allow_not_converged=True):
        ok = (ALENS_OK, ALENS_NOT_CONVERGED) if allow_not_converged else (ALENS_OK,)
        return self._stage(self.lib.orc_solve, "orc_solve", ok)

    def advance(self):
        return self._stage(self.lib.orc_advance, "orc_advance")

    def num_constraints(self):
        a = C.c_int32()
        b = C.c_int32()
        _ck(self.lib.orc_get_num_constraints(self.h, C.byref(a), C.byref(b)), "orc_get_num_constraints")
        return a.value, b.value

    def constraints(self):
        nc, nb = self.num_constraints()
        n = nc + nb
        ii = np.empty(n, np.int32)
        jj = np.empty(n, np.int32)
        im = np.empty(n, np.int32)
        d0 = np.empty(n)
        g = np.empty(n)
        jac = np.empty((n, 12))
        _ck(self.lib.orc_get_constraints(self.h, n, _p(ii, C.c_int32), _p(jj, C.c_int32),
                                         _p(im, C.c_int32), _p(d0, C.c_double), _p(g, C.c_double),
                                         _p(jac, C.c_double)), "orc_get_constraints")
        return dict(i=ii, j=jj, image=im, delta0=d0, gamma=g, jac=jac, ncoll=nc, nbil=nb)

    def con_stress(self):
        s = np.empty(9)
        _ck(self.lib.orc_get_con_stress(self.h, _p(s, C.c_double)), "orc_get_con_stress")
        return s.reshape(3, 3)

    def step_count(self) -> int:
        c = C.c_int64()
        _ck(self.lib.orc_get_step_count(self.h, C.byref(c)), "orc_get_step_count")
        return c.value

    def operator(self):
        """Delassus operator (CSR) of the current constraints."""
        nc, nb = self.num_constraints()
        nnz = C.c_int()
        _ck(self.lib.orc_get_operator(self.h, 0, C.byref(nnz), None, None, None), "orc_get_operator")
        ptr = np.empty(nc + nb + 1, np.int32)
        cols = np.empty(max(nnz.value, 1), np.int32)
        vals = np.empty(max(nnz.value, 1))
        _ck(self.lib.orc_get_operator(self.h, cols.shape[0], C.byref(nnz), _p(ptr, C.c_int32), _p(cols, C.c_int32),
                                      _p(vals, C.c_double)), "orc_get_operator")
        m = nnz.value
        return dict(rowPtr=ptr, cols=cols[:m], vals=vals[:m])

    def solver_data(self):
        """q and diag(A) of the current constraints (after detect)."""
        nc, nb = self.num_constraints()
        q = np.empty(nc + nb)
        d = np.empty(nc + nb)
        _ck(self.lib.orc_get_solver_data(self.h, nc + nb, _p(q, C.c_double), _p(d, C.c_double)),
            "orc_get_solver_data")
        return q, d
