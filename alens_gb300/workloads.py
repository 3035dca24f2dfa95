"""Seeded synthetic rod systems with the shapes of the five benchmark
workloads, plus helpers shared by tests and the benchmark.

No public dataset is involved: every system is generated from a seed.
Rods are rigid spherocylinders in aLENS units (um, pN, s).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .capi import PREC_FP64, WARM_ZERO, AlensConfig, RodState, make_config

DIAMETER = 0.025
RADIUS = DIAMETER / 2


def axis_to_quat(axis: np.ndarray) -> np.ndarray:
    """Unit quaternions (x,y,z,w) rotating +z onto each axis."""
    a = np.asarray(axis, dtype=np.float64).reshape(-1, 3)
    a = a / np.linalg.norm(a, axis=1, keepdims=True)
    q = np.empty((a.shape[0], 4))
    q[:, 0] = -a[:, 1]
    q[:, 1] = a[:, 0]
    q[:, 2] = 0.0
    q[:, 3] = 1.0 + a[:, 2]
    bad = q[:, 3] < 1e-8
    q[bad] = np.array([1.0, 0.0, 0.0, 0.0])
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q


def quat_to_axis(q: np.ndarray) -> np.ndarray:
    q = np.asarray(q).reshape(-1, 4)
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([2 * (x * z + w * y), 2 * (y * z - w * x), 1 - 2 * (x * x + y * y)], axis=1)


def isotropic_axes(rng: np.random.Generator, n: int) -> np.ndarray:
    v = rng.standard_normal((n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


@dataclass
class Workload:
    name: str
    cfg: AlensConfig
    rods: RodState
    steps: int
    notes: dict = field(default_factory=dict)


def _cfg(box_high, pbc, seed, monolayer=False, **kw) -> AlensConfig:
    base = dict(viscosity=0.01, kbt=0.00411, dt=1e-4, col_buf=DIAMETER, tol=1e-5, max_ite=2000)
    base.update(kw)
    return make_config(box_low=(0.0, 0.0, 0.0), box_high=box_high, pbc=pbc, monolayer=monolayer,
                       seed=seed, **base)


def small_periodic(n: int = 1000, box: float = 5.0, seed: int = 0, lmin=0.5, lmax=1.0,
                   **kw) -> Workload:
    """Plain method, small: rods with lengths U[lmin,lmax], diameter 0.025,
    centres uniform in a periodic cube, isotropic axes (1,000 rods in 5^3 by
    default)."""
    rng = np.random.default_rng(seed)
    length = rng.uniform(lmin, lmax, n)
    pos = rng.uniform(0.0, box, (n, 3))
    quat = axis_to_quat(isotropic_axes(rng, n))
    rods = RodState(np.arange(n, dtype=np.int64), pos, quat, length, np.full(n, RADIUS))
    cfg = _cfg((box, box, box), (1, 1, 1), seed, **kw)
    return Workload(f"periodic_{n}_rods_{box:g}um_cube", cfg, rods, 100)


def dense_monolayer(n: int = 20000, side: float = 40.0, thickness: float = 0.1,
                    kappa_vm: float = 5.0, seed: int = 0, **kw) -> Workload:
    """Dense quasi-2D monolayer: rods of length 1.0 um, centres uniform in a
    side x side periodic slab of the given thickness, in-plane axes with
    von Mises angle (concentration kappa_vm) about x and random polarity.
    Rods move in 3D (the layer is free in z)."""
    rng = np.random.default_rng(seed)
    pos = np.empty((n, 3))
    pos[:, 0] = rng.uniform(0.0, side, n)
    pos[:, 1] = rng.uniform(0.0, side, n)
    pos[:, 2] = rng.uniform(0.0, thickness, n)
    phi = rng.vonmises(0.0, kappa_vm, n) + np.pi * (rng.random(n) < 0.5)
    axis = np.stack([np.cos(phi), np.sin(phi), np.zeros(n)], axis=1)
    quat = axis_to_quat(axis)
    rods = RodState(np.arange(n, dtype=np.int64), pos, quat, np.full(n, 1.0), np.full(n, RADIUS))
    # Motion is full 3D: with in-plane-only motion, rods that cross within a
    # diameter at different heights have a contact normal along z that no
    # in-plane velocity can relieve, and the complementarity problem has no
    # solution.  z is non-periodic without walls (a free quasi-2D layer).
    cfg = _cfg((side, side, thickness), (1, 1, 0), seed, monolayer=False, **kw)
    s2d = float(np.mean(np.cos(2 * phi)))
    s3d = float(np.mean(1.5 * np.cos(phi) ** 2 - 0.5))
    return Workload(f"monolayer_{n}_rods_{side:g}x{side:g}um", cfg, rods, 1000,
                    notes={"nematic_S2d": s2d, "nematic_S3d": s3d})


def crosslinked_bundle_rods(n: int = 50000, box: float = 20.0, seed: int = 0, **kw) -> Workload:
    """3D bundle rods: lengths U[0.5,2.0], 20^3 periodic, isotropic (the
    crosslinkers are added by :func:`make_links`)."""
    rng = np.random.default_rng(seed)
    length = rng.uniform(0.5, 2.0, n)
    pos = rng.uniform(0.0, box, (n, 3))
    quat = axis_to_quat(isotropic_axes(rng, n))
    rods = RodState(np.arange(n, dtype=np.int64), pos, quat, length, np.full(n, RADIUS))
    cfg = _cfg((box, box, box), (1, 1, 1), seed, **kw)
    return Workload(f"bundle_{n}_rods_{box:g}um_cube", cfg, rods, 500)


def large_eval(n: int = 200000, box: float = 40.0, seed: int = 0, **kw) -> Workload:
    """Evaluation system of the learned warm start: lengths U[0.5,1.5], 40^3
    periodic, isotropic."""
    rng = np.random.default_rng(seed)
    length = rng.uniform(0.5, 1.5, n)
    pos = rng.uniform(0.0, box, (n, 3))
    quat = axis_to_quat(isotropic_axes(rng, n))
    rods = RodState(np.arange(n, dtype=np.int64), pos, quat, length, np.full(n, RADIUS))
    cfg = _cfg((box, box, box), (1, 1, 1), seed, **kw)
    return Workload(f"eval_{n}_rods_{box:g}um_cube", cfg, rods, 100)


def ensemble(nrep: int = 64, nmin: int = 500, nmax: int = 8000, phi: float = 0.03,
             seed: int = 0, **kw) -> list[Workload]:
    """Independent replicas with rod counts log-uniform in [nmin, nmax], each
    in a periodic cube sized for volume fraction phi (cube side
    (N pi r^2 Lmean / phi)^(1/3)), lengths U[0.5,1.0]."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(math.log(nmin), math.log(nmax), nrep)).astype(int)
    out = []
    for r, n in enumerate(counts):
        side = (n * math.pi * RADIUS ** 2 * 0.75 / phi) ** (1.0 / 3.0)
        w = small_periodic(int(n), side, seed=seed * 1000 + r + 1, **kw)
        w.name = f"replica{r}_{n}_rods"
        out.append(w)
    return out


def segment_closest_params(c1, u1, h1, c2, u2, h2):
    """Closest-point parameters (s, t) of segment pairs c1 + s u1, c2 + t u2
    (|s| <= h1, |t| <= h2), vectorised over pairs; used to place crosslinker
    anchors."""
    w = c1 - c2
    b = np.einsum("ij,ij->i", u1, u2)
    d = np.einsum("ij,ij->i", u1, w)
    e = np.einsum("ij,ij->i", u2, w)
    det = 1.0 - b * b
    par = det <= 1e-12
    s = np.where(par, 0.0, (b * e - d) / np.where(par, 1.0, det))
    lo = np.maximum(-h1, -d - np.abs(b) * h2)
    hi = np.minimum(h1, -d + np.abs(b) * h2)
    s = np.where(par, np.where(lo <= hi, 0.5 * (lo + hi), np.clip(-d, -h1, h1)), np.clip(s, -h1, h1))
    t = b * s + e
    tc = np.clip(t, -h2, h2)
    s = np.where(t != tc, np.clip(b * tc - d, -h1, h1), s)
    return s, tc


def pair_list(system, cfg, rods, sep):
    """(i, j, image) of rod pairs with separation < sep, found with a detect
    pass of `system` (a GpuSystem or OracleSystem class) whose collision
    buffer is sep."""
    c = config_with(cfg, sylinderColBuf=float(sep), KBT=-1.0)
    s = system(c)
    s.set_rods(rods)
    s.detect()
    con = s.constraints()
    s.close() if hasattr(s, "close") else None
    return con["i"].copy(), con["j"].copy(), con["image"].copy()


def make_links(cfg, rods, pairs, nlinks: int, seed: int = 0, kappa: float = 100.0, rest: float = 0.05,
               jitter: float = 0.05) -> dict:
    """Pre-bound crosslinkers on random near pairs: anchors at the pair's
    closest points, moved along each rod by U(-jitter, jitter) and kept on
    the rod."""
    rng = np.random.default_rng(seed)
    pi, pj, pimg = pairs
    pick = rng.integers(0, pi.shape[0], nlinks)
    i, j, img = pi[pick], pj[pick], pimg[pick]
    box = np.array([cfg.simBoxHigh[d] - cfg.simBoxLow[d] for d in range(3)])
    shift = np.stack([img // 9 - 1, (img // 3) % 3 - 1, img % 3 - 1], axis=1) * box
    a = quat_to_axis(rods.quat)
    hI, hJ = 0.5 * rods.length[i], 0.5 * rods.length[j]
    s, t = segment_closest_params(rods.pos[i], a[i], hI, rods.pos[j] + shift, a[j], hJ)
    s = np.clip(s + rng.uniform(-jitter, jitter, nlinks), -hI, hI)
    t = np.clip(t + rng.uniform(-jitter, jitter, nlinks), -hJ, hJ)
    return {"i": i.astype(np.int32), "j": j.astype(np.int32), "si": s, "sj": t,
            "rest": np.full(nlinks, rest), "kappa": np.full(nlinks, kappa)}


def nematic_order_2d(quat: np.ndarray) -> float:
    a = quat_to_axis(quat)
    phi = np.arctan2(a[:, 1], a[:, 0])
    return float(np.mean(np.cos(2 * phi)))


def config_with(cfg: AlensConfig, **changes) -> AlensConfig:
    """Copy of a config with some fields replaced (names as in the C struct)."""
    c = AlensConfig()
    for name, _ in AlensConfig._fields_:
        v = getattr(cfg, name)
        if hasattr(v, "__len__") and not isinstance(v, (bytes, str)):
            arr = getattr(c, name)
            for i in range(len(v)):
                arr[i] = v[i]
        else:
            setattr(c, name, v)
    for k, v in changes.items():
        setattr(c, k, v)
    return c


__all__ = ["Workload", "small_periodic", "dense_monolayer", "crosslinked_bundle_rods", "large_eval",
           "ensemble", "axis_to_quat", "quat_to_axis", "nematic_order_2d", "config_with", "pair_list",
           "make_links", "segment_closest_params", "PREC_FP64", "WARM_ZERO"]


def protein_population(cfg, rods, n: int, frac_single: float = 0.3, frac_double: float = 0.2, seed: int = 0,
                       pairs=None, ntypes: int = 1, near: float = 0.02) -> np.ndarray:
    """n proteins over a rod configuration: a fraction singly bound (one head
    at a random arc position of a random rod), a fraction doubly bound (heads
    at the closest points of random near pairs, moved along each rod by up
    to ``near``; needs ``pairs`` from pair_list) and the rest unbound, half
    of them within ``near`` of a random rod point (so that they can bind)
    and half uniform in the box.  Types cycle over ``ntypes`` species; gids
    are 10^6 + index."""
    from .capi import protein_array
    rng = np.random.default_rng(seed)
    a = quat_to_axis(rods.quat)
    lo = np.array([cfg.simBoxLow[d] for d in range(3)])
    hi = np.array([cfg.simBoxHigh[d] for d in range(3)])
    p = protein_array(n)
    p["gid"] = 1_000_000 + np.arange(n)
    p["type"] = np.arange(n) % max(ntypes, 1)
    nd = int(n * frac_double) if pairs is not None and pairs[0].shape[0] > 0 else 0
    ns = int(n * frac_single)
    nu = n - nd - ns
    # unbound
    half = nu // 2
    r = rng.integers(0, rods.n, half)
    s = rng.uniform(-0.5, 0.5, half) * rods.length[r]
    off = rng.normal(size=(half, 3))
    off *= (near * rng.uniform(0, 1, half) / np.linalg.norm(off, axis=1))[:, None]
    p["pos"][:half] = rods.pos[r] + s[:, None] * a[r] + off
    p["pos"][half:nu] = lo + rng.uniform(0, 1, (nu - half, 3)) * (hi - lo)
    if cfg.monolayer:
        p["pos"][:nu, 2] = rods.pos[0, 2] + rng.uniform(-near, near, nu)
    # singly bound
    r = rng.integers(0, rods.n, ns)
    p["idBind"][nu:nu + ns, 0] = r
    p["distBind"][nu:nu + ns, 0] = rng.uniform(-0.5, 0.5, ns) * rods.length[r]
    # doubly bound
    if nd:
        pi, pj, pimg = pairs
        pick = rng.integers(0, pi.shape[0], nd)
        i, j, img = pi[pick], pj[pick], pimg[pick]
        box = hi - lo
        shift = np.stack([img // 9 - 1, (img // 3) % 3 - 1, img % 3 - 1], axis=1) * box
        hI, hJ = 0.5 * rods.length[i], 0.5 * rods.length[j]
        s, t = segment_closest_params(rods.pos[i], a[i], hI, rods.pos[j] + shift, a[j], hJ)
        o = nu + ns
        p["idBind"][o:, 0] = i
        p["idBind"][o:, 1] = j
        p["distBind"][o:, 0] = np.clip(s + rng.uniform(-near, near, nd), -hI, hI)
        p["distBind"][o:, 1] = np.clip(t + rng.uniform(-near, near, nd), -hJ, hJ)
    return p
