"""ctypes mirror of ``include/alens_gpu.h`` and thin Python wrappers.

``GpuSystem`` drives the CUDA library ``libalens_gpu.so`` through its C ABI;
this is the Python face of the drop-in boundary and what the tests and the
benchmark call.  Loading fails loudly if the library has not been built:
there is no CPU fallback.

``OracleSystem`` (in :mod:`alens_gb300.oracle_api`) wraps the CPU oracle with
the same methods for the tests.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

ALENS_OK = 0
ALENS_INVALID_ARG = 1
ALENS_CUDA_ERROR = 2
ALENS_NOT_CONVERGED = 3
ALENS_CAPACITY = 4
ALENS_TIMEOUT = 5
ALENS_NAN_DETECTED = 6
ALENS_NO_DEVICE = 7
ALENS_NOT_READY = 8

PREC_FP64 = 0
PREC_MIXED = 1
WARM_ZERO = 0
WARM_PREV = 1
WARM_MLP = 2

STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARG", 2: "CUDA_ERROR", 3: "NOT_CONVERGED", 4: "CAPACITY",
    5: "TIMEOUT", 6: "NAN_DETECTED", 7: "NO_DEVICE", 8: "NOT_READY",
}


class AlensConfig(C.Structure):
    _fields_ = [
        ("simBoxLow", C.c_double * 3),
        ("simBoxHigh", C.c_double * 3),
        ("simBoxPBC", C.c_int32 * 3),
        ("monolayer", C.c_int32),
        ("viscosity", C.c_double),
        ("KBT", C.c_double),
        ("dt", C.c_double),
        ("sylinderDiameterColRatio", C.c_double),
        ("sylinderLengthColRatio", C.c_double),
        ("sylinderColBuf", C.c_double),
        ("conResTol", C.c_double),
        ("conMaxIte", C.c_int32),
        ("conSolverChoice", C.c_int32),
        ("rngSeed", C.c_uint64),
        ("precision", C.c_int32),
        ("warmStart", C.c_int32),
        ("maxConstraints", C.c_int32),
        ("useGraph", C.c_int32),
        ("stageTiming", C.c_int32),
        ("stream", C.c_void_p),
    ]


class AlensBlock(C.Structure):
    _fields_ = [
        ("delta0", C.c_double),
        ("gamma", C.c_double),
        ("gidI", C.c_int64),
        ("gidJ", C.c_int64),
        ("globalIndexI", C.c_int32),
        ("globalIndexJ", C.c_int32),
        ("normI", C.c_double * 3),
        ("normJ", C.c_double * 3),
        ("posI", C.c_double * 3),
        ("posJ", C.c_double * 3),
        ("labI", C.c_double * 3),
        ("labJ", C.c_double * 3),
        ("oneSide", C.c_int32),
        ("bilateral", C.c_int32),
        ("kappa", C.c_double),
        ("gammaLB", C.c_double),
        ("stress", C.c_double * 9),
    ]


BOUNDARY_WALL = 0
BOUNDARY_SPHERE = 1
BOUNDARY_TUBE = 2


class AlensBoundary(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("inside", C.c_int32),
        ("center", C.c_double * 3),
        ("axis", C.c_double * 3),
        ("radius", C.c_double),
    ]


def make_boundary(kind: int, center=(0.0, 0.0, 0.0), axis=(0.0, 0.0, 1.0), radius: float = 1.0,
                  inside: bool = True) -> AlensBoundary:
    b = AlensBoundary()
    b.type = int(kind)
    b.inside = int(bool(inside))
    for d in range(3):
        b.center[d] = float(center[d])
        b.axis[d] = float(axis[d])
    b.radius = float(radius)
    return b


class AlensStepStats(C.Structure):
    _fields_ = [
        ("step", C.c_int64),
        ("nRods", C.c_int32),
        ("nCollision", C.c_int32),
        ("nBilateral", C.c_int32),
        ("iterations", C.c_int32),
        ("refineIterations", C.c_int32),
        ("converged", C.c_int32),
        ("status", C.c_int32),
        ("residual", C.c_double),
        ("constraintsNeeded", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class AlensProteinType(C.Structure):
    """One protein species (ProteinType of Protein/ProteinType.hpp:24-76),
    in ProteinConfig.yaml units."""
    _fields_ = [
        ("tag", C.c_int32),
        ("fixedEnd0", C.c_int32),
        ("useBindVol", C.c_int32),
        ("lookupType", C.c_int32),
        ("freeLength", C.c_double),
        ("kappa", C.c_double),
        ("lambda_", C.c_double),
        ("PtoAPratio", C.c_double),
        ("diffUnbound", C.c_double),
        ("rc", C.c_double),
        ("eps", C.c_double),
        ("ko_s", C.c_double * 2),
        ("ko_d", C.c_double * 2),
        ("Ka", C.c_double * 2),
        ("Ke", C.c_double * 2),
        ("walkOff", C.c_int32),
        ("vdrag", C.c_int32 * 2),
        ("pad2", C.c_int32),
        ("fstall", C.c_double),
        ("vmax", C.c_double * 2),
        ("vmaxAP", C.c_double * 2),
        ("diffBoundS", C.c_double * 2),
        ("diffBoundD", C.c_double * 2),
    ]


def make_protein_type(tag=0, freeLength=0.025, rc=0.025, kappa=200.0, lambda_=0.5, diffUnbound=1.0,
                      useBindVol=False, eps=400.0, Ka=(100.0, 100.0), ko_s=(28.1, 28.1), Ke=(100.0, 100.0),
                      ko_d=(28.1, 28.1), PtoAPratio=1.0, fixedEnd0=False, lookupType=0, walkOff=True,
                      vdrag=(False, False), fstall=5.0, vmax=(0.5, 0.5), vmaxAP=None, diffBoundS=(0.0, 0.0),
                      diffBoundD=(0.0, 0.0)) -> AlensProteinType:
    """A species; the defaults are the symmetric crosslinker of the dense
    monolayer example (Examples/DenseMonoLayer/ProteinConfig.yaml); vmaxAP
    defaults to vmax as in ProteinType::readFromYaml."""
    t = AlensProteinType()
    vmaxAP = vmax if vmaxAP is None else vmaxAP
    t.walkOff, t.fstall = int(walkOff), float(fstall)
    for e in range(2):
        t.vdrag[e], t.vmax[e], t.vmaxAP[e] = int(vdrag[e]), float(vmax[e]), float(vmaxAP[e])
        t.diffBoundS[e], t.diffBoundD[e] = float(diffBoundS[e]), float(diffBoundD[e])
    t.tag, t.fixedEnd0, t.useBindVol, t.lookupType = int(tag), int(fixedEnd0), int(useBindVol), int(lookupType)
    t.freeLength, t.kappa, t.lambda_, t.PtoAPratio = float(freeLength), float(kappa), float(lambda_), float(PtoAPratio)
    t.diffUnbound, t.rc, t.eps = float(diffUnbound), float(rc), float(eps)
    for e in range(2):
        t.ko_s[e], t.ko_d[e], t.Ka[e], t.Ke[e] = float(ko_s[e]), float(ko_d[e]), float(Ka[e]), float(Ke[e])
    return t


class AlensKmcStats(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("nU", "nS", "nD", "nUS", "nSU", "nSD", "nDS", "maxCandidates")]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


# AlensProtein (112 bytes) as a numpy record
PROTEIN_DTYPE = np.dtype([("gid", "<i8"), ("type", "<i4"), ("idBind", "<i4", (2,)), ("pad", "<i4"),
                          ("distBind", "<f8", (2,)), ("pos", "<f8", (3,)), ("posEnd", "<f8", (2, 3))])
assert PROTEIN_DTYPE.itemsize == 112


def protein_array(n: int) -> np.ndarray:
    """n unbound proteins (idBind = -1, NaN geometry) to fill in."""
    a = np.zeros(n, dtype=PROTEIN_DTYPE)
    a["idBind"] = -1
    a["distBind"] = np.nan
    a["posEnd"] = np.nan
    return a


def make_config(box_low=(0.0, 0.0, 0.0), box_high=(5.0, 5.0, 5.0), pbc=(1, 1, 1),
                monolayer=False, viscosity=0.01, kbt=0.00411, dt=1e-4,
                col_ratio_d=1.0, col_ratio_l=1.0, col_buf=0.025, tol=1e-5,
                max_ite=2000, seed=0, precision=PREC_FP64, warm=WARM_ZERO,
                max_constraints=0, use_graph=1, stage_timing=0, stream=None) -> AlensConfig:
    c = AlensConfig()
    for d in range(3):
        c.simBoxLow[d] = float(box_low[d])
        c.simBoxHigh[d] = float(box_high[d])
        c.simBoxPBC[d] = int(bool(pbc[d]))
    c.monolayer = int(bool(monolayer))
    c.viscosity = viscosity
    c.KBT = kbt
    c.dt = dt
    c.sylinderDiameterColRatio = col_ratio_d
    c.sylinderLengthColRatio = col_ratio_l
    c.sylinderColBuf = col_buf
    c.conResTol = tol
    c.conMaxIte = int(max_ite)
    c.conSolverChoice = 0
    c.rngSeed = int(seed) & 0xFFFFFFFFFFFFFFFF
    c.precision = int(precision)
    c.warmStart = int(warm)
    c.maxConstraints = int(max_constraints)
    c.useGraph = int(use_graph)
    c.stageTiming = int(stage_timing)
    c.stream = stream
    return c


class AlensError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        msg = f"{where}: {STATUS_NAMES.get(status, status)} ({status})"
        if detail:
            msg += f" [{detail}]"
        super().__init__(msg)
        self.status = status


def _p(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


_PD = C.POINTER(C.c_double)
_PI32 = C.POINTER(C.c_int32)
_PI64 = C.POINTER(C.c_int64)
_PF = C.POINTER(C.c_float)

MLP_NUM_FEATURES = 12
MLP_NUM_PARAMS = 5057

_LIB = None


def load_library(path: str | Path | None = None) -> C.CDLL:
    """Load libalens_gpu.so; raises if it is missing (no fallback)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else _build.lib_path()
    if not p.exists():
        raise RuntimeError(f"CUDA library not built: {p} (run __graft_entry__.build())")
    lib = C.CDLL(str(p))
    vp = C.c_void_p
    sigs = {
        "alens_config_default": (None, [C.POINTER(AlensConfig)]),
        "alens_status_str": (C.c_char_p, [C.c_int]),
        "alens_create": (C.c_int, [C.POINTER(AlensConfig), C.POINTER(vp)]),
        "alens_create_ensemble": (C.c_int, [C.POINTER(AlensConfig), C.c_int, C.POINTER(vp)]),
        "alens_destroy": (C.c_int, [vp]),
        "alens_set_rods": (C.c_int, [vp, C.c_int, C.c_int, _PI64, _PD, _PD, _PD, _PD, _PI32]),
        "alens_update_rods": (C.c_int, [vp, C.c_int, C.c_int, _PD, _PD]),
        "alens_get_rods": (C.c_int, [vp, C.c_int, C.c_int, _PD, _PD]),
        "alens_get_velocity": (C.c_int, [vp, C.c_int, C.c_int, _PD, _PD]),
        "alens_add_bilateral": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(AlensBlock)]),
        "alens_set_links": (C.c_int, [vp, C.c_int, C.c_int, _PI32, _PI32, _PD, _PD, _PD, _PD]),
        "alens_set_boundaries": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(AlensBoundary)]),
        "alens_step": (C.c_int, [vp, C.POINTER(AlensStepStats)]),
        "alens_detect": (C.c_int, [vp, C.POINTER(AlensStepStats)]),
        "alens_solve": (C.c_int, [vp, C.POINTER(AlensStepStats)]),
        "alens_advance": (C.c_int, [vp, C.POINTER(AlensStepStats)]),
        "alens_get_replica_stats": (C.c_int, [vp, C.c_int, C.POINTER(AlensStepStats)]),
        "alens_get_num_constraints": (C.c_int, [vp, C.c_int, _PI32, _PI32]),
        "alens_get_constraints": (C.c_int, [vp, C.c_int, C.c_int, _PI32, _PI32, _PI32, _PD, _PD, _PD]),
        "alens_get_con_stress": (C.c_int, [vp, C.c_int, _PD]),
        "alens_get_operator": (C.c_int, [vp, C.c_int, C.c_int, _PI32, _PI32, _PI32, _PD, _PD, _PD, _PD, _PD]),
        "alens_bbpgd_solve_noalloc": (C.c_int, [C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, C.c_double, C.c_int, vp,
                                                C.POINTER(C.c_int), _PD, C.POINTER(C.c_int)]),
        "alens_get_step_count": (C.c_int, [vp, _PI64]),
        "alens_set_step_count": (C.c_int, [vp, C.c_int64]),
        "alens_get_stream": (C.c_int, [vp, C.POINTER(vp)]),
        "alens_get_launch_count": (C.c_int, [vp, _PI64]),
        "alens_get_last_error": (C.c_char_p, [vp]),
        "alens_get_stage_times": (C.c_int, [vp, _PD]),
        "alens_step_batched": (C.c_int, [C.POINTER(vp), C.c_int, C.POINTER(AlensStepStats)]),
        "alens_get_gamma": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(C.c_int), _PI32, _PD]),
        "alens_get_pairs": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(C.c_int), _PI32, _PI32, _PI32]),
        "alens_set_wait_limit": (C.c_int, [vp, C.c_uint64, C.c_int]),
        "alens_get_constraint_points": (C.c_int, [vp, C.c_int, C.c_int, _PD]),
        "alens_set_protein_types": (C.c_int, [vp, C.c_int, C.POINTER(AlensProteinType), C.c_double, C.c_double]),
        "alens_set_proteins": (C.c_int, [vp, C.c_int, C.c_int, vp]),
        "alens_get_proteins": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(C.c_int), vp]),
        "alens_protein_bind_step": (C.c_int, [vp, C.POINTER(AlensKmcStats)]),
        "alens_protein_motion_step": (C.c_int, [vp, C.POINTER(AlensKmcStats)]),
        "alens_mlp_create": (C.c_int, [C.c_uint64, C.c_int64, C.POINTER(vp)]),
        "alens_mlp_destroy": (C.c_int, [vp]),
        "alens_mlp_get_params": (C.c_int, [vp, _PF]),
        "alens_mlp_set_params": (C.c_int, [vp, _PF]),
        "alens_mlp_add_samples": (C.c_int, [vp, C.c_int, _PF, _PF]),
        "alens_mlp_dataset_size": (C.c_int, [vp, _PI64]),
        "alens_mlp_clear_dataset": (C.c_int, [vp]),
        "alens_mlp_train": (C.c_int, [vp, C.c_int, C.c_int, C.c_float, C.c_uint64, _PF]),
        "alens_mlp_predict": (C.c_int, [vp, C.c_int, _PF, _PF]),
        "alens_mlp_gradient": (C.c_int, [vp, C.c_int, _PF, _PF, _PF, _PF]),
        "alens_attach_mlp": (C.c_int, [vp, vp]),
        "alens_set_feature_capture": (C.c_int, [vp, C.c_int]),
        "alens_mlp_collect": (C.c_int, [vp, vp, _PI64]),
        "alens_get_features": (C.c_int, [vp, C.c_int, C.c_int, _PF, _PF, _PI32]),
        "alens_autotune": (C.c_int, [vp, C.c_int, C.c_char_p, C.c_int]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def exported_symbols_from_header(header: Path | None = None) -> list[str]:
    """Names of the functions declared in include/*.h."""
    import re
    names = []
    hdrs = [header] if header else sorted((_build.ROOT / "include").glob("*.h"))
    for h in hdrs:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(alens_[a-z0-9_]+)\s*\(", text):
            if m.group(1) not in names:
                names.append(m.group(1))
    return names


def _ck(rc: int, where: str, ok=(ALENS_OK,)) -> int:
    if rc not in ok:
        raise AlensError(rc, where)
    return rc


class RodState:
    """Host-side rod arrays in the C ABI layout (orientation stored x,y,z,w)."""

    def __init__(self, gid, pos, quat, length, radius, immovable=None):
        self.gid = np.ascontiguousarray(gid, dtype=np.int64)
        self.pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self.quat = np.ascontiguousarray(quat, dtype=np.float64).reshape(-1, 4)
        self.length = np.ascontiguousarray(length, dtype=np.float64)
        self.radius = np.ascontiguousarray(radius, dtype=np.float64)
        self.immovable = (np.ascontiguousarray(immovable, dtype=np.int32)
                          if immovable is not None else None)

    @property
    def n(self) -> int:
        return int(self.gid.shape[0])

    def copy(self) -> "RodState":
        return RodState(self.gid.copy(), self.pos.copy(), self.quat.copy(), self.length.copy(),
                        self.radius.copy(), None if self.immovable is None else self.immovable.copy())


class GpuSystem:
    """One context of the CUDA library (``nrep`` replicas, default 1)."""

    def _ck(self, rc, where, ok=(ALENS_OK,)):
        if rc not in ok:
            detail = ""
            if self.h:
                d = self.lib.alens_get_last_error(self.h)
                detail = d.decode() if d else ""
            raise AlensError(rc, where, detail)
        return rc

    def __init__(self, cfg: AlensConfig | list[AlensConfig], lib: C.CDLL | None = None):
        self.lib = lib or load_library()
        self.h = C.c_void_p()
        if isinstance(cfg, (list, tuple)):
            arr = (AlensConfig * len(cfg))(*cfg)
            _ck(self.lib.alens_create_ensemble(arr, len(cfg), C.byref(self.h)), "alens_create_ensemble")
            self.nrep = len(cfg)
        else:
            _ck(self.lib.alens_create(C.byref(cfg), C.byref(self.h)), "alens_create")
            self.nrep = 1
        self.n = [0] * self.nrep

    def close(self):
        if self.h:
            self.lib.alens_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_rods(self, rods: RodState, replica: int = 0):
        self._ck(self.lib.alens_set_rods(self.h, replica, rods.n, _p(rods.gid, C.c_int64), _p(rods.pos, C.c_double),
                                    _p(rods.quat, C.c_double), _p(rods.length, C.c_double),
                                    _p(rods.radius, C.c_double), _p(rods.immovable, C.c_int32)),
            "alens_set_rods")
        self.n[replica] = rods.n

    def update_rods(self, pos, quat, replica: int = 0):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        quat = np.ascontiguousarray(quat, dtype=np.float64)
        self._ck(self.lib.alens_update_rods(self.h, replica, self.n[replica], _p(pos, C.c_double),
                                       _p(quat, C.c_double)), "alens_update_rods")

    def get_rods(self, replica: int = 0, out=None):
        n = self.n[replica]
        pos, quat = out if out is not None else (np.empty((n, 3)), np.empty((n, 4)))
        self._ck(self.lib.alens_get_rods(self.h, replica, n, _p(pos, C.c_double), _p(quat, C.c_double)),
            "alens_get_rods")
        return pos, quat

    def get_velocity(self, replica: int = 0):
        n = self.n[replica]
        v = np.empty((n, 3))
        w = np.empty((n, 3))
        self._ck(self.lib.alens_get_velocity(self.h, replica, n, _p(v, C.c_double), _p(w, C.c_double)),
            "alens_get_velocity")
        return v, w

    def add_bilateral(self, blocks, replica: int = 0):
        arr = (AlensBlock * len(blocks))(*blocks)
        self._ck(self.lib.alens_add_bilateral(self.h, replica, len(blocks), arr), "alens_add_bilateral")

    def set_links(self, links, replica: int = 0):
        """links: dict of arrays i, j (rod indices), si, sj (arc positions),
        rest, kappa."""
        a = [np.ascontiguousarray(links[k], dtype=t) for k, t in
             (("i", np.int32), ("j", np.int32), ("si", np.float64), ("sj", np.float64), ("rest", np.float64),
              ("kappa", np.float64))]
        self._ck(self.lib.alens_set_links(self.h, replica, int(a[0].shape[0]), _p(a[0], C.c_int32),
                                          _p(a[1], C.c_int32), _p(a[2], C.c_double), _p(a[3], C.c_double),
                                          _p(a[4], C.c_double), _p(a[5], C.c_double)), "alens_set_links")

    def set_protein_types(self, types, kbt: float = 0.00411, rod_diameter: float = 0.025):
        arr = (AlensProteinType * max(len(types), 1))(*types)
        self._ck(self.lib.alens_set_protein_types(self.h, len(types), arr, float(kbt), float(rod_diameter)),
                 "alens_set_protein_types")

    def set_proteins(self, proteins: np.ndarray, replica: int = 0):
        a = np.ascontiguousarray(proteins, dtype=PROTEIN_DTYPE)
        self._ck(self.lib.alens_set_proteins(self.h, replica, int(a.shape[0]), a.ctypes.data if a.size else None),
                 "alens_set_proteins")

    def get_proteins(self, replica: int = 0) -> np.ndarray:
        n = C.c_int()
        self._ck(self.lib.alens_get_proteins(self.h, replica, 0, C.byref(n), None), "alens_get_proteins",
                 ok=(ALENS_OK, ALENS_CAPACITY))
        a = np.zeros(n.value, dtype=PROTEIN_DTYPE)
        self._ck(self.lib.alens_get_proteins(self.h, replica, n.value, C.byref(n), a.ctypes.data if a.size else None),
                 "alens_get_proteins")
        return a

    def protein_bind_step(self) -> list[dict]:
        st = (AlensKmcStats * self.nrep)()
        self._ck(self.lib.alens_protein_bind_step(self.h, st), "alens_protein_bind_step")
        return [st[r].as_dict() for r in range(self.nrep)]

    def protein_motion_step(self) -> list[dict]:
        st = (AlensKmcStats * self.nrep)()
        self._ck(self.lib.alens_protein_motion_step(self.h, st), "alens_protein_motion_step")
        return [st[r].as_dict() for r in range(self.nrep)]

    def set_boundaries(self, boundaries, replica: int = 0):
        arr = (AlensBoundary * max(len(boundaries), 1))(*boundaries)
        self._ck(self.lib.alens_set_boundaries(self.h, replica, len(boundaries), arr), "alens_set_boundaries")

    def _stage(self, fn, name, ok=(ALENS_OK,)):
        st = AlensStepStats()
        rc = fn(self.h, C.byref(st))
        self._ck(rc, name, ok)
        d = st.as_dict()
        d["rc"] = rc
        return d

    def step(self, allow_not_converged=True):
        ok = (ALENS_OK, ALENS_NOT_CONVERGED) if allow_not_converged else (ALENS_OK,)
        return self._stage(self.lib.alens_step, "alens_step", ok)

    def detect(self):
        return self._stage(self.lib.alens_detect, "alens_detect")

    def solve(self, allow_not_converged=True):
        ok = (ALENS_OK, ALENS_NOT_CONVERGED) if allow_not_converged else (ALENS_OK,)
        return self._stage(self.lib.alens_solve, "alens_solve", ok)

    def advance(self):
        return self._stage(self.lib.alens_advance, "alens_advance")

    def replica_stats(self, replica: int):
        st = AlensStepStats()
        self._ck(self.lib.alens_get_replica_stats(self.h, replica, C.byref(st)), "alens_get_replica_stats")
        return st.as_dict()

    def num_constraints(self, replica: int = 0):
        a = C.c_int32()
        b = C.c_int32()
        self._ck(self.lib.alens_get_num_constraints(self.h, replica, C.byref(a), C.byref(b)),
            "alens_get_num_constraints")
        return a.value, b.value

    def constraints(self, replica: int = 0):
        nc, nb = self.num_constraints(replica)
        n = nc + nb
        ii = np.empty(n, np.int32)
        jj = np.empty(n, np.int32)
        im = np.empty(n, np.int32)
        d0 = np.empty(n)
        g = np.empty(n)
        jac = np.empty((n, 12))
        self._ck(self.lib.alens_get_constraints(self.h, replica, n, _p(ii, C.c_int32), _p(jj, C.c_int32),
                                           _p(im, C.c_int32), _p(d0, C.c_double), _p(g, C.c_double),
                                           _p(jac, C.c_double)), "alens_get_constraints")
        return dict(i=ii, j=jj, image=im, delta0=d0, gamma=g, jac=jac, ncoll=nc, nbil=nb)

    def operator(self, replica: int = 0):
        """Delassus operator of one replica (CSR, local columns) and the QP
        vectors; gamma0 is the current gamma."""
        nc, nb = self.num_constraints(replica)
        n = nc + nb
        nnz = C.c_int()
        self._ck(self.lib.alens_get_operator(self.h, replica, 0, C.byref(nnz), None, None, None, None, None,
                                             None, None), "alens_get_operator")
        ptr = np.empty(n + 1, np.int32)
        cols = np.empty(max(nnz.value, 1), np.int32)
        vals = np.empty(max(nnz.value, 1))
        q = np.empty(n)
        cinv = np.empty(n)
        lb = np.empty(n)
        g0 = np.empty(n)
        self._ck(self.lib.alens_get_operator(self.h, replica, cols.shape[0], C.byref(nnz), _p(ptr, C.c_int32),
                                             _p(cols, C.c_int32), _p(vals, C.c_double), _p(q, C.c_double),
                                             _p(cinv, C.c_double), _p(lb, C.c_double), _p(g0, C.c_double)),
                 "alens_get_operator")
        m = nnz.value
        return dict(rowPtr=ptr, cols=cols[:m], vals=vals[:m], q=q, cinv=cinv, lb=lb, gamma0=g0)

    def constraint_blocks(self, replica: int = 0) -> dict:
        """The last step's constraint blocks of one replica, canonical order:
        rod indices, periodic image, separation, multiplier, normal on rod I,
        lab-frame points, compliance-derived stiffness kappa (0 for
        collisions), bilateral and one-sided flags."""
        c = self.constraints(replica)
        op = self.operator(replica)
        n = c["i"].shape[0]
        lab = np.empty((n, 6))
        self._ck(self.lib.alens_get_constraint_points(self.h, replica, n, _p(lab, C.c_double)),
                 "alens_get_constraint_points")
        cinv = op["cinv"]
        kappa = np.where(cinv > 0.0, 1.0 / np.where(cinv > 0.0, cinv, 1.0), 0.0)
        return {"i": c["i"], "j": c["j"], "image": c["image"], "delta0": c["delta0"], "gamma": c["gamma"],
                "normI": c["jac"][:, 0:3].copy(), "labI": lab[:, 0:3].copy(), "labJ": lab[:, 3:6].copy(),
                "kappa": kappa, "bilateral": np.isneginf(op["lb"]).astype(np.int32),
                "oneSide": (c["j"] < 0).astype(np.int32)}

    def con_stress(self, replica: int = 0):
        s = np.empty(9)
        self._ck(self.lib.alens_get_con_stress(self.h, replica, _p(s, C.c_double)), "alens_get_con_stress")
        return s.reshape(3, 3)

    def step_count(self) -> int:
        c = C.c_int64()
        self._ck(self.lib.alens_get_step_count(self.h, C.byref(c)), "alens_get_step_count")
        return c.value

    def set_step_count(self, count: int):
        self._ck(self.lib.alens_set_step_count(self.h, int(count)), "alens_set_step_count")

    def launch_count(self) -> int:
        c = C.c_int64()
        self._ck(self.lib.alens_get_launch_count(self.h, C.byref(c)), "alens_get_launch_count")
        return c.value

    def stage_times(self):
        t = np.zeros(5)
        self._ck(self.lib.alens_get_stage_times(self.h, _p(t, C.c_double)), "alens_get_stage_times")
        return t

    def autotune(self, reps: int = 5) -> dict:
        """Time the solver configurations on the next step's problem and keep
        the fastest (the rods do not move); returns the report."""
        import json
        buf = C.create_string_buffer(16384)
        self._ck(self.lib.alens_autotune(self.h, int(reps), buf, len(buf)), "alens_autotune")
        return json.loads(buf.value.decode())

    # ---- learned warm start
    def attach_mlp(self, mlp: "Mlp | None"):
        self._ck(self.lib.alens_attach_mlp(self.h, mlp.h if mlp is not None else None), "alens_attach_mlp")
        self._mlp = mlp  # keep the model alive while attached

    def set_feature_capture(self, on: bool = True):
        self._ck(self.lib.alens_set_feature_capture(self.h, int(bool(on))), "alens_set_feature_capture")

    def collect(self, mlp: "Mlp") -> int:
        """Append the last step's (features, converged multiplier) rows to
        the model's dataset; returns the rows added."""
        added = C.c_int64()
        self._ck(self.lib.alens_mlp_collect(self.h, mlp.h, C.byref(added)), "alens_mlp_collect")
        return added.value

    def features(self, replica: int = 0):
        """Features (n x 12) and overlap-unit scales A_kk/d (n) of the last
        step's collision constraints, canonical order."""
        nc, _ = self.num_constraints(replica)
        f = np.empty((max(nc, 1), MLP_NUM_FEATURES), np.float32)
        sc = np.empty(max(nc, 1), np.float32)
        n = C.c_int32()
        self._ck(self.lib.alens_get_features(self.h, replica, nc, _p(f, C.c_float), _p(sc, C.c_float),
                                             C.byref(n)), "alens_get_features")
        return f[: n.value], sc[: n.value]

    def stream_handle(self) -> int:
        s = C.c_void_p()
        self._ck(self.lib.alens_get_stream(self.h, C.byref(s)), "alens_get_stream")
        return s.value or 0


class Mlp:
    """The learned warm-start model (``AlensMlp``): BF16 12-64-64-1 SiLU
    network trained with the library's tensor-core kernels and Adam."""

    def __init__(self, seed: int = 0, capacity: int = 0, lib: C.CDLL | None = None):
        self.lib = lib or load_library()
        self.h = C.c_void_p()
        _ck(self.lib.alens_mlp_create(int(seed) & 0xFFFFFFFFFFFFFFFF, int(capacity), C.byref(self.h)),
            "alens_mlp_create")

    def close(self):
        if self.h:
            self.lib.alens_mlp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.empty(MLP_NUM_PARAMS, np.float32)
        _ck(self.lib.alens_mlp_get_params(self.h, _p(p, C.c_float)), "alens_mlp_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (MLP_NUM_PARAMS,)
        _ck(self.lib.alens_mlp_set_params(self.h, _p(p, C.c_float)), "alens_mlp_set_params")

    def add_samples(self, feat, target):
        feat = np.ascontiguousarray(feat, dtype=np.float32).reshape(-1, MLP_NUM_FEATURES)
        target = np.ascontiguousarray(target, dtype=np.float32).reshape(-1)
        _ck(self.lib.alens_mlp_add_samples(self.h, feat.shape[0], _p(feat, C.c_float), _p(target, C.c_float)),
            "alens_mlp_add_samples")

    def dataset_size(self) -> int:
        n = C.c_int64()
        _ck(self.lib.alens_mlp_dataset_size(self.h, C.byref(n)), "alens_mlp_dataset_size")
        return n.value

    def clear_dataset(self):
        _ck(self.lib.alens_mlp_clear_dataset(self.h), "alens_mlp_clear_dataset")

    def train(self, epochs: int, batch: int = 65536, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        loss = np.zeros(max(epochs, 1), np.float32)
        _ck(self.lib.alens_mlp_train(self.h, int(epochs), int(batch), float(lr), int(seed), _p(loss, C.c_float)),
            "alens_mlp_train")
        return loss[:epochs]

    def predict(self, feat) -> np.ndarray:
        feat = np.ascontiguousarray(feat, dtype=np.float32).reshape(-1, MLP_NUM_FEATURES)
        out = np.empty(feat.shape[0], np.float32)
        _ck(self.lib.alens_mlp_predict(self.h, feat.shape[0], _p(feat, C.c_float), _p(out, C.c_float)),
            "alens_mlp_predict")
        return out

    def gradient(self, feat, target):
        feat = np.ascontiguousarray(feat, dtype=np.float32).reshape(-1, MLP_NUM_FEATURES)
        target = np.ascontiguousarray(target, dtype=np.float32).reshape(-1)
        g = np.empty(MLP_NUM_PARAMS, np.float32)
        loss = C.c_float()
        _ck(self.lib.alens_mlp_gradient(self.h, feat.shape[0], _p(feat, C.c_float), _p(target, C.c_float),
                                        _p(g, C.c_float), C.byref(loss)), "alens_mlp_gradient")
        return g, loss.value
