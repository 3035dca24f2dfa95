"""CPU tests of the oracle: known answers, the canonical reduction tree, the
BBPGD optimality conditions checked independently in numpy, invariances and
host-side failure handling.  No GPU needed."""
import math

import numpy as np
import pytest

from alens_gb300 import capi, workloads
from alens_gb300 import oracle_api as O


# ------------------------------------------------------------ Philox KAT
# Known-answer vectors published with the Random123 library for
# Philox4x32-10 (counter, key -> output).
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,out", PHILOX_KAT)
def test_philox_known_answers(ctr, key, out):
    assert list(O.philox4x32(ctr, key)) == out


def test_det_log_accuracy():
    rng = np.random.default_rng(1)
    xs = np.concatenate([10.0 ** rng.uniform(-300, 300, 2000), rng.uniform(0.5, 2.0, 2000),
                         [5e-324, 1e-310, 0.025, 0.0125 / 1.5, 1.0, 2.0, 0.5]])
    for x in xs:
        ref = math.log(x)
        got = O.det_log(x)
        assert abs(got - ref) <= 4e-16 * max(1.0, abs(ref)), (x, got, ref)


def test_det_sincos_accuracy():
    for x in np.concatenate([np.linspace(-math.pi, math.pi, 2001), [0.0, 1e-300, 1e-8, 0.0625, 0.07]]):
        s, c = O.det_sincos(float(x))
        assert abs(s - math.sin(x)) <= 2e-15 and abs(c - math.cos(x)) <= 2e-15, x


def test_normals_distribution_and_mapping():
    z = np.array([O.normals6(12345, g, 7) for g in range(20000)]).ravel()
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1.0) < 0.02
    # Box-Muller mapping re-derived here from the Philox words: 24-bit
    # uniforms, FP32 arithmetic in the library (within 2e-6 of FP64 here)
    w = np.concatenate([O.philox4x32([3, 0, 9, b], [5, 0]) for b in range(2)])
    u = [((int(w[i]) >> 8) + 0.5) / 16777216.0 for i in range(6)]
    ref = []
    for p in range(3):
        r = math.sqrt(-2.0 * math.log(u[2 * p]))
        th = 2 * math.pi * u[2 * p + 1]
        ref += [r * math.cos(th), r * math.sin(th)]
    got = O.normals6(5, 3, 9)
    assert np.allclose(got, ref, rtol=0, atol=2e-6)
    # the FP32 values are exactly representable: z is a float widened to double
    assert np.array_equal(np.asarray(got, np.float32).astype(np.float64), got)


# --------------------------------------------------------------- DCP KAT
def _dcp(c1, u1, h1, c2, u2, h2):
    return O.dcp(np.array(c1, float), np.array(u1, float), h1, np.array(c2, float),
                 np.array(u2, float), h2)


def test_dcp_crossing():
    s, t, P, Q, d = _dcp([0, 0, 0], [1, 0, 0], 1.0, [0, 0, 0.5], [0, 1, 0], 1.0)
    assert (s, t, d) == (0.0, 0.0, 0.5)
    assert np.array_equal(P, [0, 0, 0]) and np.array_equal(Q, [0, 0, 0.5])


def test_dcp_parallel_overlap_midpoint():
    s, t, P, Q, d = _dcp([0, 0, 0], [1, 0, 0], 1.0, [0.5, 0.3, 0], [1, 0, 0], 1.0)
    assert s == pytest.approx(0.25) and t == pytest.approx(-0.25) and d == pytest.approx(0.3)
    s, t, P, Q, d = _dcp([0, 0, 0], [1, 0, 0], 1.0, [0.5, 0.3, 0], [-1, 0, 0], 1.0)
    assert s == pytest.approx(0.25) and t == pytest.approx(0.25) and d == pytest.approx(0.3)
    assert np.allclose(Q, [0.25, 0.3, 0])


def test_dcp_collinear_disjoint():
    s, t, P, Q, d = _dcp([0, 0, 0], [1, 0, 0], 1.0, [3, 0, 0], [1, 0, 0], 1.0)
    assert (s, t, d) == (1.0, -1.0, 1.0)


def test_dcp_endpoint_endpoint():
    s, t, P, Q, d = _dcp([0, 0, 0], [1, 0, 0], 1.0, [2, 1, 0], [0, 1, 0], 0.5)
    assert s == 1.0 and t == -0.5 and d == pytest.approx(math.sqrt(1.25))


def test_dcp_t_shape():
    # segment J's end touches the middle of I at distance 0.2
    s, t, P, Q, d = _dcp([0, 0, 0], [1, 0, 0], 1.0, [0.3, 0.7, 0], [0, 1, 0], 0.5)
    assert s == pytest.approx(0.3) and t == -0.5 and d == pytest.approx(0.2)


def test_dcp_point_segment_and_point_point():
    s, t, P, Q, d = _dcp([0.3, 0.4, 0], [0, 0, 1], 0.0, [0, 0, 0], [1, 0, 0], 1.0)
    assert s == 0.0 and t == pytest.approx(0.3) and d == pytest.approx(0.4)
    s, t, P, Q, d = _dcp([0, 0, 0], [0, 0, 1], 0.0, [0.3, 0.4, 0], [0, 1, 0], 0.0)
    assert d == pytest.approx(0.5)


def test_dcp_random_against_brute_force():
    rng = np.random.default_rng(3)
    for _ in range(300):
        c1, c2 = rng.normal(size=3), rng.normal(size=3) * 0.5
        u1, u2 = rng.normal(size=3), rng.normal(size=3)
        u1 /= np.linalg.norm(u1)
        u2 /= np.linalg.norm(u2)
        h1, h2 = rng.uniform(0, 1, 2)
        s, t, P, Q, d = _dcp(c1, u1, h1, c2, u2, h2)
        ss = np.linspace(-h1, h1, 201)
        tt = np.linspace(-h2, h2, 201)
        X = c1[None, None, :] + ss[:, None, None] * u1 - (c2[None, None, :] + tt[None, :, None] * u2)
        dmin = np.sqrt((X ** 2).sum(-1)).min()
        assert d <= dmin + 1e-12
        assert d >= dmin - 2e-2 * (h1 + h2 + 1e-3)


# ------------------------------------------------- canonical reduction
def _warp(v):
    v = list(v)
    off = 16
    while off >= 1:
        for l in range(off):
            v[l] = v[l] + v[l + off]
        off //= 2
    return v[0]


def _canon_py(v):
    v = [float(x) for x in v]
    n = len(v)
    if n == 0:
        return 0.0
    def tile64(b):
        lanes = [v[b + l] if b + l < n else 0.0 for l in range(64)]
        return _warp(lanes[:32]) + _warp(lanes[32:])
    T = [tile64(b) for b in range(0, n, 64)]
    while True:
        m = len(T)
        R = []
        for c in range(0, m, 1024):
            lanes = []
            for l in range(32):
                acc = 0.0
                for j in range(32):
                    i = c + l + 32 * j
                    if i < m:
                        acc = acc + T[i]
                lanes.append(acc)
            R.append(_warp(lanes))
        if len(R) == 1:
            return R[0]
        T = R


@pytest.mark.parametrize("n", [0, 1, 63, 64, 65, 5000, 140000])
def test_canonical_sum_tree(n):
    rng = np.random.default_rng(n)
    v = rng.normal(size=n) * 10.0 ** rng.uniform(-8, 8, size=n)
    got = O.canon_sum(v)
    assert got == _canon_py(v)
    assert got == pytest.approx(math.fsum(v), rel=1e-9, abs=1e-300)


def test_canonical_sum_multilevel():
    v = np.random.default_rng(5).normal(size=600000)
    assert O.canon_sum(v) == pytest.approx(math.fsum(v), rel=1e-10, abs=1e-9)


def test_mobility_slender_body_and_sphere():
    mu = 0.01
    for L, r in [(1.0, 0.0125), (0.5, 0.0125), (2.0, 0.0125)]:
        b = -(1 + 2 * math.log(r / L))
        ref = [b / (4 * math.pi * mu * L), (b + 2) / (8 * math.pi * mu * L),
               3 * (b + 2) / (2 * math.pi * mu * L ** 3)]
        assert np.allclose(O.mobility(L, r, mu), ref, rtol=1e-14)
    ref = [1 / (6 * math.pi * mu * 0.1), 1 / (6 * math.pi * mu * 0.1), 1 / (8 * math.pi * mu * 0.1 ** 3)]
    assert np.allclose(O.mobility(0.15, 0.1, mu), ref, rtol=1e-14)


def test_brownian_velocity_fluctuation_dissipation():
    """Known velocity U_B = sqrt(2 kT/dt) M^1/2 xi has covariance (2 kT/dt) M:
    along the axis the parallel mobility, across it the perpendicular one,
    rotation only about axes normal to the rod (20,000 unit rods)."""
    w = workloads.small_periodic(n=20000, box=30.0, seed=3, lmin=1.0, lmax=1.0)
    s = O.OracleSystem(w.cfg)
    s.set_rods(w.rods)
    s.detect()
    u = s.known_velocity()
    a = workloads.quat_to_axis(w.rods.quat)
    m = O.mobility(1.0, float(w.rods.radius[0]), w.cfg.viscosity)
    c = 2.0 * w.cfg.KBT / w.cfg.dt
    ut, om = u[:, :3], u[:, 3:]
    upar = np.einsum("ij,ij->i", ut, a)
    uperp = ut - upar[:, None] * a
    opar = np.einsum("ij,ij->i", om, a)
    operp = om - opar[:, None] * a
    z = upar / math.sqrt(c * m[0])
    assert abs(z.mean()) < 0.03 and abs(z.var() - 1.0) < 0.05
    assert abs((uperp ** 2).sum(1).mean() / (c * m[1]) - 2.0) < 0.1
    assert abs((operp ** 2).sum(1).mean() / (c * m[2]) - 2.0) < 0.1
    assert np.abs(opar).max() <= 1e-12 * math.sqrt(c * m[2])
    assert abs(np.corrcoef(upar, uperp[:, 0])[0, 1]) < 0.05
    # a fresh context at the same step draws the same noise (keyed by seed, gid, step)
    s2 = O.OracleSystem(w.cfg)
    s2.set_rods(w.rods)
    s2.detect()
    assert np.array_equal(s2.known_velocity(), u)


# ---------------------------------------------- solve: independent KKT
def _assemble(sysO, rods, cfg):
    """D (6N x Nc), block mobility M and U_nc rebuilt in numpy."""
    con = sysO.constraints()
    n = rods.n
    nc = len(con["gamma"])
    D = np.zeros((6 * n, nc))
    for k in range(nc):
        i, j = con["i"][k], con["j"][k]
        D[6 * i:6 * i + 6, k] += con["jac"][k, :6]
        if j >= 0:
            D[6 * j:6 * j + 6, k] += con["jac"][k, 6:]
    pos, quat = sysO.get_rods()
    return con, D


def _mobility_matrix(quat_before, rods, mu, mono=False):
    a = workloads.quat_to_axis(quat_before)
    n = rods.n
    M = np.zeros((6 * n, 6 * n))
    for i in range(n):
        m = O.mobility(rods.length[i], rods.radius[i], mu)
        sphere = rods.length[i] < 2 * rods.radius[i]
        if sphere:
            Mt = m[0] * np.eye(3)
            Mr = m[2] * np.eye(3)
        else:
            aa = np.outer(a[i], a[i])
            Mt = m[0] * aa + m[1] * (np.eye(3) - aa)
            Mr = m[2] * (np.eye(3) - aa)
        M[6 * i:6 * i + 3, 6 * i:6 * i + 3] = Mt
        M[6 * i + 3:6 * i + 6, 6 * i + 3:6 * i + 6] = Mr
    return M


def test_bbpgd_kkt_independent():
    w = workloads.small_periodic(n=400, box=2.6, seed=11)
    sysO = O.OracleSystem(w.cfg)
    sysO.set_rods(w.rods)
    sysO.detect()
    unc = sysO.known_velocity().ravel()
    st = sysO.solve(allow_not_converged=False)
    con, D = _assemble(sysO, w.rods, w.cfg)
    M = _mobility_matrix(w.rods.quat, w.rods, w.cfg.viscosity)
    dt = w.cfg.dt
    gam = con["gamma"]
    q = con["delta0"] + dt * (D.T @ unc)
    g = dt * (D.T @ (M @ (D @ gam))) + q
    tol = w.cfg.conResTol
    assert st["nCollision"] > 20
    assert np.all(gam >= 0)
    assert np.all(g >= -tol * 1.0001 - 1e-12)
    res = np.max(np.abs(gam - np.maximum(gam - g, 0.0)))
    assert res <= tol * 1.0001 + 1e-12
    assert abs(res - st["residual"]) <= 1e-9


def test_collision_stress_is_pair_virial():
    """Collision virial sum_k gamma_k (P_k - Q_k) n_k^T rebuilt in numpy: with
    n = (P - Q)/|P - Q| it is sum_k gamma_k d_k n_k n_k^T, d_k = phi0_k +
    rcol_I + rcol_J, symmetric and positive semidefinite (gamma >= 0)."""
    w = workloads.small_periodic(n=400, box=2.6, seed=11, col_ratio_d=0.8)
    s = O.OracleSystem(w.cfg)
    s.set_rods(w.rods)
    s.detect()
    s.solve(allow_not_converged=False)
    con = s.constraints()
    assert con["nbil"] == 0 and con["ncoll"] > 20
    rcol = 0.8 * w.rods.radius
    d = con["delta0"] + rcol[con["i"]] + rcol[con["j"]]
    n = con["jac"][:, :3]
    ref = np.einsum("k,ka,kb->ab", con["gamma"] * d, n, n)
    got = s.con_stress()
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    assert np.allclose(got, got.T, rtol=0, atol=1e-12 * np.abs(ref).max())
    assert np.linalg.eigvalsh(0.5 * (got + got.T)).min() >= -1e-12 * np.abs(ref).max()


def test_collision_geometry_independent():
    """Every collision row of the oracle recomputed in numpy with the
    package's own clamped closest-point routine (a different formulation of
    the segment distance): the separation phi0 = |P - Q| - rcol_I - rcol_J,
    the normal (P - Q)/|P - Q| and the pair's periodic image."""
    w = workloads.small_periodic(n=1000, box=5.0, seed=0)
    s = O.OracleSystem(w.cfg)
    s.set_rods(w.rods)
    s.detect()
    con = s.constraints()
    nc = con["ncoll"]
    assert nc > 100
    i, j, img = con["i"][:nc], con["j"][:nc], con["image"][:nc]
    box = np.array([w.cfg.simBoxHigh[d] - w.cfg.simBoxLow[d] for d in range(3)])
    shift = np.stack([img // 9 - 1, (img // 3) % 3 - 1, img % 3 - 1], axis=1) * box
    a = workloads.quat_to_axis(w.rods.quat)
    hI, hJ = 0.5 * w.rods.length[i], 0.5 * w.rods.length[j]
    cI, cJ = w.rods.pos[i], w.rods.pos[j] + shift
    sp, tp = workloads.segment_closest_params(cI, a[i], hI, cJ, a[j], hJ)
    P = cI + sp[:, None] * a[i]
    Q = cJ + tp[:, None] * a[j]
    dist = np.linalg.norm(P - Q, axis=1)
    sep = dist - w.rods.radius[i] - w.rods.radius[j]
    assert np.max(np.abs(sep - con["delta0"][:nc])) <= 1e-12
    assert np.all(sep < w.cfg.sylinderColBuf)
    n = (P - Q) / dist[:, None]
    assert np.max(np.abs(n - con["jac"][:nc, :3])) <= 1e-9
    assert np.array_equal(con["jac"][:nc, 6:9], -con["jac"][:nc, :3])


def test_pair_set_complete_brute_force():
    """The oracle's collision set equals a brute-force scan of all rod pairs
    (minimum image; the 5 um box is wider than twice the cutoff, so one image
    per pair) with the numpy closest-point routine: nothing missed, nothing
    extra, and no pair within rounding distance of the cutoff."""
    w = workloads.small_periodic(n=1000, box=5.0, seed=0)
    s = O.OracleSystem(w.cfg)
    s.set_rods(w.rods)
    s.detect()
    con = s.constraints()
    nc = con["ncoll"]
    rods = w.rods
    I, J = np.triu_indices(rods.n, 1)
    d = rods.pos[J] - rods.pos[I]
    shift = -np.round(d / 5.0) * 5.0
    reach = (0.5 * (rods.length[I] + rods.length[J]) + rods.radius[I] + rods.radius[J]
             + w.cfg.sylinderColBuf)
    keep = np.linalg.norm(d + shift, axis=1) < reach
    I, J, shift = I[keep], J[keep], shift[keep]
    a = workloads.quat_to_axis(rods.quat)
    cI, cJ = rods.pos[I], rods.pos[J] + shift
    sp, tp = workloads.segment_closest_params(cI, a[I], 0.5 * rods.length[I], cJ, a[J], 0.5 * rods.length[J])
    sep = (np.linalg.norm(cI + sp[:, None] * a[I] - cJ - tp[:, None] * a[J], axis=1)
           - rods.radius[I] - rods.radius[J])
    hit = sep < w.cfg.sylinderColBuf
    assert np.min(np.abs(sep - w.cfg.sylinderColBuf)) > 1e-9
    brute = set(zip(I[hit].tolist(), J[hit].tolist()))
    found = {(min(x, y), max(x, y)) for x, y in zip(con["i"][:nc].tolist(), con["j"][:nc].tolist())}
    assert len(found) == nc > 100
    assert found == brute


def test_velocity_and_euler_update_independent():
    """Write-back and Euler update recomputed in numpy: U = U_nc + M D gamma
    per rod, x <- x + dt U (periodic wrap), q <- normalize(exp(dt w / 2) q)
    with the Hamilton product."""
    w = workloads.small_periodic(n=400, box=2.6, seed=11)
    s = O.OracleSystem(w.cfg)
    s.set_rods(w.rods)
    s.detect()
    unc = s.known_velocity().ravel()
    s.solve(allow_not_converged=False)
    con, D = _assemble(s, w.rods, w.cfg)
    M = _mobility_matrix(w.rods.quat, w.rods, w.cfg.viscosity)
    s.advance()
    vel, omega = s.get_velocity()
    pos, quat = s.get_rods()
    U = (unc + M @ (D @ con["gamma"])).reshape(-1, 6)
    assert con["ncoll"] > 20 and np.abs(M @ (D @ con["gamma"])).max() > 0
    scale = np.abs(U).max()
    assert np.abs(np.hstack([vel, omega]) - U).max() <= 1e-12 * scale
    dt = w.cfg.dt
    dx = pos - (w.rods.pos + dt * U[:, :3])
    dx -= np.round(dx / 2.6) * 2.6
    assert np.abs(dx).max() <= 1e-13
    assert np.all((pos >= 0.0) & (pos < 2.6))
    om = U[:, 3:]
    wn = np.linalg.norm(om, axis=1)
    half = 0.5 * dt * wn
    pw = np.cos(half)
    pv = (np.sin(half) / wn)[:, None] * om
    q0 = w.rods.quat
    qv, qw = q0[:, :3], q0[:, 3]
    nv = pw[:, None] * qv + qw[:, None] * pv + np.cross(pv, qv)
    nw = pw * qw - np.einsum("ij,ij->i", pv, qv)
    ref = np.hstack([nv, nw[:, None]])
    ref /= np.linalg.norm(ref, axis=1, keepdims=True)
    assert np.abs(quat - ref).max() <= 1e-14


def test_delassus_operator_independent():
    """The oracle's explicit operator equals dt D^T M D rebuilt densely in
    numpy (collisions plus crosslinks), with CSR rows sorted by column; the
    solver's diagonal adds the compliance 1/kappa of the bilateral rows."""
    w = workloads.small_periodic(n=400, box=2.6, seed=11)
    links = workloads.make_links(w.cfg, w.rods, workloads.pair_list(O.OracleSystem, w.cfg, w.rods, 0.05), 60,
                                 seed=2, kappa=100.0)
    s = O.OracleSystem(w.cfg)
    s.set_rods(w.rods)
    s.set_links(links)
    s.detect()
    con, D = _assemble(s, w.rods, w.cfg)
    assert con["ncoll"] > 20 and con["nbil"] == 60
    M = _mobility_matrix(w.rods.quat, w.rods, w.cfg.viscosity)
    ref = w.cfg.dt * (D.T @ M @ D)
    op = s.operator()
    nc = ref.shape[0]
    A = np.zeros((nc, nc))
    for r in range(nc):
        lo, hi = op["rowPtr"][r], op["rowPtr"][r + 1]
        cols = op["cols"][lo:hi]
        assert np.all(np.diff(cols) > 0)
        A[r, cols] = op["vals"][lo:hi]
    assert np.abs(A - ref).max() <= 1e-12 * np.abs(ref).max()
    # no structural entry missing: every nonzero of the dense product is stored
    assert np.count_nonzero(np.abs(ref) > 1e-14 * np.abs(ref).max()) <= op["rowPtr"][-1]
    _, diag = s.solver_data()
    comp = np.concatenate([np.zeros(con["ncoll"]), 1.0 / links["kappa"]])
    assert np.abs(diag - (np.diag(ref) + comp)).max() <= 1e-12 * np.abs(ref).max()


def test_crosslink_blocks_independent():
    """Crosslinker blocks built from the rod state, recomputed in numpy:
    anchors c + s a on both rods, separation reduced to the minimum image,
    phi0 = |d| - rest, normal d/|d| at I and -d/|d| at J, torque arms
    (s a) x n; every link row follows the collision rows."""
    w = workloads.small_periodic(n=400, box=2.6, seed=11)
    links = workloads.make_links(w.cfg, w.rods, workloads.pair_list(O.OracleSystem, w.cfg, w.rods, 0.05), 60,
                                 seed=2, kappa=100.0)
    s = O.OracleSystem(w.cfg)
    s.set_rods(w.rods)
    s.set_links(links)
    s.detect()
    con = s.constraints()
    nc = con["ncoll"]
    a = workloads.quat_to_axis(w.rods.quat)
    i, j = links["i"], links["j"]
    rI = links["si"][:, None] * a[i]
    rJ = links["sj"][:, None] * a[j]
    d = (w.rods.pos[i] + rI) - (w.rods.pos[j] + rJ)
    d -= 2.6 * np.round(d / 2.6)
    ln = np.linalg.norm(d, axis=1)
    n = d / ln[:, None]
    rows = slice(nc, nc + len(i))
    assert np.array_equal(con["i"][rows], i) and np.array_equal(con["j"][rows], j)
    assert np.abs(con["delta0"][rows] - (ln - links["rest"])).max() <= 1e-12
    jac = con["jac"][rows]
    assert np.abs(jac[:, 0:3] - n).max() <= 1e-12 and np.abs(jac[:, 6:9] + n).max() <= 1e-12
    assert np.abs(jac[:, 3:6] - np.cross(rI, n)).max() <= 1e-12
    assert np.abs(jac[:, 9:12] - np.cross(rJ, -n)).max() <= 1e-12


def test_pair_set_complete_headline_layer():
    """The 20,000-rod quasi-2D layer (periodic in x and y, free in z): the
    oracle's ~59,000 collisions equal a KD-tree scan of all rod pairs within
    the largest reach, decided with the numpy closest-point routine."""
    spatial = pytest.importorskip("scipy.spatial")
    w = workloads.dense_monolayer()
    s = O.OracleSystem(w.cfg)
    s.set_rods(w.rods)
    s.detect()
    con = s.constraints()
    nc = con["ncoll"]
    rods = w.rods
    L = np.array([w.cfg.simBoxHigh[d] - w.cfg.simBoxLow[d] for d in range(3)])
    pbc = np.array([bool(w.cfg.simBoxPBC[d]) for d in range(3)])
    box = np.where(pbc, L, 1e6)
    pos = rods.pos + np.array([0.0, 0.0, 1000.0])  # free axis: far from the tree's wrap
    tree = spatial.cKDTree(np.mod(pos, box), boxsize=box)
    reach = rods.length.max() + 2 * rods.radius.max() + w.cfg.sylinderColBuf
    pairs = tree.query_pairs(reach, output_type="ndarray")
    I, J = pairs[:, 0], pairs[:, 1]
    d = rods.pos[J] - rods.pos[I]
    shift = np.where(pbc, -np.round(d / L) * L, 0.0)
    a = workloads.quat_to_axis(rods.quat)
    cI, cJ = rods.pos[I], rods.pos[J] + shift
    sp, tp = workloads.segment_closest_params(cI, a[I], 0.5 * rods.length[I], cJ, a[J], 0.5 * rods.length[J])
    sep = (np.linalg.norm(cI + sp[:, None] * a[I] - cJ - tp[:, None] * a[J], axis=1)
           - rods.radius[I] - rods.radius[J])
    hit = sep < w.cfg.sylinderColBuf
    assert np.min(np.abs(sep - w.cfg.sylinderColBuf)) > 1e-9
    brute = set(zip(np.minimum(I, J)[hit].tolist(), np.maximum(I, J)[hit].tolist()))
    found = {(min(x, y), max(x, y)) for x, y in zip(con["i"][:nc].tolist(), con["j"][:nc].tolist())}
    assert len(found) == nc > 50000
    assert found == brute


def test_step_translation_invariance():
    w = workloads.small_periodic(n=300, box=2.5, seed=4, kbt=-1.0)
    a = O.OracleSystem(w.cfg)
    a.set_rods(w.rods)
    r2 = w.rods.copy()
    r2.pos = (r2.pos + np.array([2.5, -2.5, 5.0])).copy()  # whole box periods
    b = O.OracleSystem(w.cfg)
    b.set_rods(r2)
    sa, sb = a.detect(), b.detect()
    ca, cb = a.constraints(), b.constraints()
    assert sa["nCollision"] == sb["nCollision"]
    assert np.array_equal(ca["i"], cb["i"]) and np.array_equal(ca["j"], cb["j"])
    assert np.allclose(ca["delta0"], cb["delta0"], atol=1e-12)


def test_pair_set_permutation_invariance():
    w = workloads.small_periodic(n=300, box=2.5, seed=5, kbt=-1.0)
    perm = np.random.default_rng(0).permutation(w.rods.n)
    r2 = capi.RodState(w.rods.gid[perm], w.rods.pos[perm], w.rods.quat[perm], w.rods.length[perm],
                       w.rods.radius[perm])
    a, b = O.OracleSystem(w.cfg), O.OracleSystem(w.cfg)
    a.set_rods(w.rods)
    b.set_rods(r2)
    a.detect()
    b.detect()
    ca, cb = a.constraints(), b.constraints()

    def gidpairs(c, rods):
        out = set()
        for i, j, m in zip(c["i"], c["j"], c["image"]):
            gi, gj = rods.gid[i], rods.gid[j]
            sx, sy, sz = m // 9 - 1, (m // 3) % 3 - 1, m % 3 - 1
            if gi > gj or (gi == gj and m < 13):
                gi, gj, sx, sy, sz = gj, gi, -sx, -sy, -sz
            out.add((int(gi), int(gj), sx, sy, sz))
        return out

    assert gidpairs(ca, w.rods) == gidpairs(cb, r2)


def test_oracle_fault_handling():
    w = workloads.small_periodic(n=100, box=2.0, seed=1)
    s = O.OracleSystem(w.cfg)
    bad = w.rods.copy()
    bad.pos[5, 1] = np.nan
    s.set_rods(bad)
    with pytest.raises(capi.AlensError) as e:
        s.step()
    assert e.value.status == capi.ALENS_NAN_DETECTED
    cfg = workloads.config_with(w.cfg, conMaxIte=1)
    s2 = O.OracleSystem(cfg)
    dense = workloads.small_periodic(n=200, box=1.2, seed=2)
    s2.set_rods(dense.rods)
    st = s2.step()
    assert st["rc"] == capi.ALENS_NOT_CONVERGED and st["iterations"] == 1
    tiny = workloads.config_with(w.cfg)
    tiny.simBoxHigh[0] = 0.5
    s3 = O.OracleSystem(tiny)
    with pytest.raises(capi.AlensError) as e:
        s3.set_rods(w.rods)
    assert e.value.status == capi.ALENS_INVALID_ARG


def test_bilateral_spring_oracle():
    """Two parallel rods tied by a stretched bilateral spring move toward
    each other by the amount the implicit spring predicts."""
    cfg = capi.make_config(box_high=(10, 10, 10), pbc=(0, 0, 0), kbt=-1.0, col_buf=0.0, tol=1e-10)
    rods = capi.RodState([0, 1], [[5, 5, 5], [5, 5.3, 5]], workloads.axis_to_quat([[1, 0, 0], [1, 0, 0]]),
                         [1.0, 1.0], [0.0125, 0.0125])
    s = O.OracleSystem(cfg)
    s.set_rods(rods)
    kappa, ell0 = 100.0, 0.1
    blk = capi.AlensBlock()
    blk.delta0 = 0.3 - ell0
    blk.gamma = -blk.delta0 * kappa
    blk.globalIndexI, blk.globalIndexJ = 0, 1
    for d, v in enumerate([0, -1, 0]):
        blk.normI[d] = v
        blk.normJ[d] = -v
    blk.bilateral = 1
    blk.kappa = kappa
    s.add_bilateral([blk])
    st = s.step(allow_not_converged=False)
    pos, _ = s.get_rods()
    m_perp = O.mobility(1.0, 0.0125, cfg.viscosity)[1]
    # implicit spring: gamma = -kappa (delta0 + dt * 2 m_perp gamma)
    gam = -kappa * blk.delta0 / (1 + kappa * cfg.dt * 2 * m_perp)
    dy = cfg.dt * m_perp * gam
    assert st["nBilateral"] == 1
    assert pos[0, 1] == pytest.approx(5 - dy, abs=1e-9)
    assert pos[1, 1] == pytest.approx(5.3 + dy, abs=1e-9)


def test_library_exports_header_symbols():
    """The C ABI library loads and exports every function of include/*.h
    (no CUDA call is made)."""
    import ctypes

    from alens_gb300 import build
    path = build.build_lib()
    lib = ctypes.CDLL(str(path))
    names = capi.exported_symbols_from_header()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    lib.alens_status_str.restype = ctypes.c_char_p
    assert lib.alens_status_str(4) == b"constraint capacity exceeded"


def test_monolayer_motion_stays_in_plane():
    """monolayer: true (Examples/DenseMonoLayer/RunConfig.yaml:8) on the
    window fixture: three steps with collisions move rods in x and y only,
    with no out-of-plane velocity and rotation about z only, so in-plane
    axes stay in plane."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_fixtures
    cfg, rods = make_fixtures.load_fixture()
    assert cfg.monolayer
    s = O.OracleSystem(cfg)
    s.set_rods(rods)
    for _ in range(3):
        st = s.step(allow_not_converged=False)
    assert st["nCollision"] > 1000
    pos, quat = s.get_rods()
    vel, omega = s.get_velocity()
    assert np.array_equal(pos[:, 2], rods.pos[:, 2])
    assert np.abs(pos[:, :2] - rods.pos[:, :2]).max() > 1e-4
    assert np.all(vel[:, 2] == 0.0) and np.all(omega[:, :2] == 0.0)
    assert np.abs(workloads.quat_to_axis(quat)[:, 2]).max() <= 1e-14
