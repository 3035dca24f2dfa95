"""The oracle's restatement of the protein binding step (oracle/oracle_kmc.cpp),
checked on the CPU.

* The one known answer the reference ships for this path,
  Protein/ProteinTest.hpp:33-71 ("Parallel to Anti-parallel binding
  affinity"): with PtoAPratio = 0.5 the S->D binding factor towards a rod
  parallel to the bound rod, over the factor towards an antiparallel one,
  is 0.5 within 1e-6 (mock protein of Protein/ProteinType.hpp:171-188).
* The S->D integral and its inverse against scipy's adaptive quadrature,
  the bind volume against a numerical integral, the exp against numpy.
* The event frequencies of whole steps against the rates of
  Protein/ProteinModel.md (binomial bounds), the binding-point
  distributions against the chord and the Boltzmann integrand, and the
  springs the doubly bound proteins become.
"""
import math

import numpy as np
import pytest

from alens_gb300 import capi, workloads
from alens_gb300 import oracle_api as oa

integrate = pytest.importorskip("scipy.integrate")

KBT = 0.00411
D = 0.025


def mock_type(**kw):
    """ProteinType::setMockProteinType (Protein/ProteinType.hpp:171-188)."""
    base = dict(Ka=(1.0, 1.0), Ke=(1.0, 1.0), ko_s=(1.0, 1.0), ko_d=(1.0, 1.0), kappa=1.0, eps=1.0, rc=0.5,
                freeLength=1.0, lambda_=0.0, PtoAPratio=1.0, diffUnbound=0.0)
    base.update(kw)
    return capi.make_protein_type(**base)


def test_ptoap_ratio_known_answer():
    """Protein/ProteinTest.hpp:33-71: bound rod along x (MockSylinder,
    :19-31), head 0 bound, free end 1; para / antipara factor = PtoAPratio."""
    t = mock_type(PtoAPratio=0.5)
    x = np.array([1.0, 0.0, 0.0])
    para = oa.kmc_binding_factor_sd(t, 1, x, x)
    anti = oa.kmc_binding_factor_sd(t, 1, x, -x)
    assert abs(0.5 - para / anti) < 1e-6
    # the other branch: PtoAPratio > 1 scales the antiparallel factor
    t2 = mock_type(PtoAPratio=2.0)
    assert abs(2.0 - oa.kmc_binding_factor_sd(t2, 1, x, x) / oa.kmc_binding_factor_sd(t2, 1, x, -x)) < 1e-6
    # the prefactor never exceeds 1 (Protein/ProteinData.hpp:123)
    assert oa.kmc_binding_factor_sd(t2, 1, x, x) == 1.0
    # fixedEnd0: the end-0 turnover rates are zero
    t3 = mock_type(fixedEnd0=True)
    assert oa.kmc_binding_factor_sd(t3, 0, x, x) == 0.0


def test_type_constants_follow_the_model():
    t = capi.make_protein_type(ko_s=(3.0, 4.0), Ka=(60.2, 120.4), Ke=(6.02, 2.0), ko_d=(5.0, 6.0), eps=400.0,
                               rc=0.03, diffUnbound=1.0, kappa=200.0, lambda_=0.25)
    dt = 1e-4
    c = oa.kmc_type_constants(t, KBT, D, dt)
    rcap = max(0.03, math.sqrt(6 * 1.0 * dt))
    assert c["rcap"] == pytest.approx(rcap, rel=1e-15)
    # (Lc / 2rc)(3 Ka / (4 pi rc^3))(2 rc eps) ko_s dt = Lc * usCoef
    assert c["usCoef0"] == pytest.approx(3.0 * (60.2 / 602) * 400 * 3 / (4 * math.pi * rcap ** 3) * dt, rel=1e-14)
    assert c["usCoef1"] == pytest.approx(4.0 * (120.4 / 602) * 400 * 3 / (4 * math.pi * rcap ** 3) * dt, rel=1e-14)
    assert c["suProb0"] == pytest.approx(3.0 * dt, rel=1e-15)
    # useBindVol false: Ke is a number per site
    assert c["sdCoef1"] == pytest.approx(6.0 * 2.0 * 400 * dt, rel=1e-14)
    assert c["A"] == pytest.approx(0.75 * 200.0 / (2 * KBT), rel=1e-15)
    assert c["rOuter"] == pytest.approx(0.025 + D + 6 / math.sqrt(c["A"]), rel=1e-15)


def _integrand(t, d2, s):
    A = (1 - t.lambda_) * t.kappa / (2 * KBT)
    return math.exp(-A * (math.sqrt(d2 + s * s) - t.freeLength - D) ** 2)


@pytest.mark.parametrize("d,sA,sB", [(0.0, -0.5, 0.5), (0.03, -0.5, 0.5), (0.049, -0.2, 0.7), (0.06, 0.01, 0.4),
                                     (0.08, -0.3, -0.02), (0.1, -1.0, 1.0), (0.02, 0.05, 0.06), (0.04, -0.02, 0.02)])
@pytest.mark.parametrize("kappa,lam", [(200.0, 0.5), (300.0, 0.25822), (50.0, 0.0)])
def test_sd_integral_and_inverse_against_adaptive_quadrature(d, sA, sB, kappa, lam):
    """The integrand in FP32: the integral within 2e-6 (relative) of scipy's."""
    t = capi.make_protein_type(kappa=kappa, lambda_=lam, freeLength=0.025)
    d2 = d * d
    got = oa.kmc_sd_integral(t, KBT, D, 1e-5, d2, sA, sB)
    pts = [p for p in (-math.sqrt(max((0.05) ** 2 - d2, 0.0)), 0.0, math.sqrt(max(0.05 ** 2 - d2, 0.0)))
           if sA < p < sB]
    ref, _ = integrate.quad(lambda s: _integrand(t, d2, s), sA, sB, points=pts or None, epsabs=0.0,
                            epsrel=1e-13, limit=500)
    # the integrand is evaluated in FP32
    assert abs(got - ref) <= 2e-6 * max(ref, 1e-300) + 1e-12, (got, ref)
    if ref > 1e-12:
        for u in (0.0, 0.1, 0.5, 0.9, 0.999):
            s = oa.kmc_sd_invert(t, KBT, D, 1e-5, d2, sA, sB, u * got)
            assert sA - 1e-7 <= s <= sB + 1e-7      # FP32 bounds
            part, _ = integrate.quad(lambda x: _integrand(t, d2, x), sA, s, epsabs=0.0, epsrel=1e-13, limit=500)
            assert abs(part - u * got) <= 5e-6 * got, (u, part, u * got)


@pytest.mark.parametrize("d,sA,sB", [(0.03, -0.5, 0.5), (0.049, -0.2, 0.7), (0.07, -0.3, 0.3), (0.026, -0.5, 0.5),
                                     (0.1, -1.0, 1.0), (0.02, -0.5, 0.5)])
def test_sd_integral_lookup_type_1(d, sA, sB):
    """lookupType 1: stretch (1 - D/d) sqrt(d^2 + s^2) (Protein/ProteinModel.md),
    head distances up to ell0 + D + w; no binding when d <= D."""
    t = capi.make_protein_type(kappa=100.0, lambda_=0.5, freeLength=0.05, lookupType=1)
    A = 0.5 * 100.0 / (2 * KBT)
    rcap = 0.05 + D + 6 / math.sqrt(A)
    got = oa.kmc_sd_integral(t, KBT, D, 1e-5, d * d, sA, sB)
    if d <= D:
        assert got == 0.0
        return
    k = 1 - D / d
    smax = math.sqrt(max(rcap * rcap - d * d, 0.0))
    lo, hi = max(sA, -smax), min(sB, smax)
    f = lambda s: math.exp(-A * (k * math.sqrt(d * d + s * s) - 0.05) ** 2)
    ref = integrate.quad(f, lo, hi, epsabs=0.0, epsrel=1e-13, limit=500)[0] if hi > lo else 0.0
    # FP32 integrand; the scale 1 - D/d adds a rounding of its own
    assert abs(got - ref) <= 5e-6 * max(ref, 1e-300) + 1e-12, (got, ref)


def test_bind_volume_closed_form():
    for kappa, lam, ell0 in ((200.0, 0.5, 0.025), (300.0, 0.25822, 0.053), (1.0, 0.0, 1.0)):
        t = capi.make_protein_type(kappa=kappa, lambda_=lam, freeLength=ell0)
        a = (1 - lam) * kappa / (2 * KBT)
        c = ell0 + D
        ref, _ = integrate.quad(lambda r: 4 * math.pi * r * r * math.exp(-a * (r - c) ** 2), 0, c + 40 / math.sqrt(a),
                                epsabs=0.0, epsrel=1e-13, limit=500)
        assert oa.kmc_bind_volume(t, KBT, D) == pytest.approx(ref, rel=1e-12)


def test_exp_accuracy():
    x = np.concatenate([np.linspace(-745.0, 709.0, 20001), np.linspace(-1, 1, 2001), [0.0, -0.0, 1e-300]])
    got = np.array([oa.kmc_exp(v) for v in x])
    ref = np.exp(x)
    normal = ref > 2.3e-308
    rel = np.abs(got[normal] - ref[normal]) / ref[normal]
    assert rel.max() <= 4e-16, rel.max()
    assert oa.kmc_exp(0.0) == 1.0
    assert oa.kmc_exp(-800.0) == 0.0 and math.isinf(oa.kmc_exp(800.0))
    # the FP32 exp of the S->D integrand, on its range [-87, 0]
    xf = np.linspace(-87.0, 0.0, 20001).astype(np.float32)
    gotf = np.array([oa.kmc_expf(float(v)) for v in xf])
    reff = np.exp(xf.astype(np.float64))
    assert float(np.max(np.abs(gotf - reff) / reff)) <= 6e-7
    assert oa.kmc_expf(-100.0) == 0.0


# ----------------------------------------------------------- whole steps
def _one_rod_system(dt=1e-4, length=1.0, extra=None):
    cfg = capi.make_config(box_high=(4.0, 4.0, 4.0), pbc=(1, 1, 1), dt=dt)
    pos = [[2.0, 2.0, 2.0]]
    ax = [[1.0, 0.0, 0.0]]
    if extra is not None:
        pos.append(extra[0])
        ax.append(extra[1])
    n = len(pos)
    rods = capi.RodState(np.arange(n, dtype=np.int64), np.array(pos), workloads.axis_to_quat(np.array(ax)),
                         np.full(n, length), np.full(n, 0.0125))
    o = oa.OracleSystem(cfg)
    o.set_rods(rods)
    return o, cfg


def _binom_ok(k, n, p, z=5.0):
    mu = n * p
    sd = math.sqrt(max(n * p * (1 - p), 1e-12))
    return abs(k - mu) <= z * sd + 1


def test_unbound_binding_frequency_and_chord():
    t = capi.make_protein_type(rc=0.05, diffUnbound=0.0, ko_s=(50.0, 30.0), Ka=(0.05, 0.05), eps=400.0)
    o, cfg = _one_rod_system()
    o.set_protein_types([t], KBT, D)
    n = 40000
    p = capi.protein_array(n)
    p["gid"] = np.arange(n)
    d = 0.03                      # distance of the protein from the axis
    p["pos"] = [2.1, 2.0 + d, 2.0]
    o.set_proteins(p)
    st = o.protein_bind_step()
    c = oa.kmc_type_constants(t, KBT, D, cfg.dt)
    Lc = 2 * math.sqrt(0.05 ** 2 - d * d)
    P0, P1 = Lc * c["usCoef0"], Lc * c["usCoef1"]
    assert P0 + P1 < 1
    q = o.get_proteins()
    b0 = int(np.sum(q["idBind"][:, 0] == 0))
    b1 = int(np.sum(q["idBind"][:, 1] == 0))
    assert st["nUS"] == b0 + b1 and st["nS"] == b0 + b1
    assert _binom_ok(b0, n, P0) and _binom_ok(b1, n, P1)
    # binding points uniform on the chord [0.1 - Lc/2, 0.1 + Lc/2]
    s = np.concatenate([q["distBind"][q["idBind"][:, 0] == 0, 0], q["distBind"][q["idBind"][:, 1] == 0, 1]])
    assert s.min() >= 0.1 - Lc / 2 - 1e-12 and s.max() <= 0.1 + Lc / 2 + 1e-12
    stats = pytest.importorskip("scipy.stats")
    assert stats.kstest((s - (0.1 - Lc / 2)) / Lc, "uniform").pvalue > 1e-4
    o.close()


def test_single_to_double_frequency_and_positions():
    """Rod 0 along x at the origin of the box centre; rod 1 parallel at
    distance 0.06 (the bound head at the centre of rod 0)."""
    t = capi.make_protein_type(ko_s=(0.0, 0.0), ko_d=(100.0, 100.0), Ke=(0.5, 0.5), eps=400.0, kappa=200.0,
                               lambda_=0.5, PtoAPratio=0.5)
    o, cfg = _one_rod_system(extra=([2.1, 2.06, 2.0], [1.0, 0.0, 0.0]))
    o.set_protein_types([t], KBT, D)
    n = 40000
    p = capi.protein_array(n)
    p["gid"] = np.arange(n)
    p["idBind"][:, 0] = 0
    p["distBind"][:, 0] = 0.0
    o.set_proteins(p)
    st = o.protein_bind_step()
    c = oa.kmc_type_constants(t, KBT, D, cfg.dt)
    # foot of the head on rod 1: t0 = -0.1 from its centre; rod half-length 0.5
    I = oa.kmc_sd_integral(t, KBT, D, cfg.dt, 0.06 ** 2, -0.5 + 0.1, 0.5 + 0.1)
    P = 0.5 * c["sdCoef1"] * I      # parallel rods: PtoAPratio prefactor
    q = o.get_proteins()
    k = int(np.sum(q["idBind"][:, 1] == 1))
    assert st["nSD"] == k and st["nSU"] == 0
    assert _binom_ok(k, n, P), (k, n * P)
    # the bound points follow the integrand: CDF from scipy
    s = q["distBind"][q["idBind"][:, 1] == 1, 1] + 0.1     # arc from the foot

    def cdf(x):
        v, _ = integrate.quad(lambda y: _integrand(t, 0.06 ** 2, y), -0.4, x, epsrel=1e-10, limit=200)
        return v / I

    stats = pytest.importorskip("scipy.stats")
    assert stats.kstest(s, np.vectorize(cdf)).pvalue > 1e-4
    o.close()


def test_unbinding_frequencies_and_release():
    t = capi.make_protein_type(ko_s=(300.0, 100.0), ko_d=(80.0, 40.0), Ka=(0.0, 0.0), Ke=(0.0, 0.0), rc=0.04,
                               lambda_=0.0, diffUnbound=0.0)
    o, cfg = _one_rod_system(extra=([2.0, 2.05, 2.0], [1.0, 0.0, 0.0]))
    o.set_protein_types([t], KBT, D)
    n = 30000
    p = capi.protein_array(n)
    p["gid"] = np.arange(n)
    p["idBind"][: n // 3, 0] = 0                      # S, head 0
    p["distBind"][: n // 3, 0] = 0.2
    p["idBind"][n // 3: 2 * n // 3, 1] = 0            # S, head 1
    p["distBind"][n // 3: 2 * n // 3, 1] = -0.2
    p["idBind"][2 * n // 3:, 0] = 0                   # D
    p["idBind"][2 * n // 3:, 1] = 1
    p["distBind"][2 * n // 3:, 0] = 0.0
    p["distBind"][2 * n // 3:, 1] = 0.0
    o.set_proteins(p)
    o.protein_bind_step()
    q = o.get_proteins()
    m = n // 3
    su0 = int(np.sum(q["idBind"][:m, 0] == -1))
    su1 = int(np.sum(q["idBind"][m:2 * m, 1] == -1))
    assert _binom_ok(su0, m, 300.0 * cfg.dt) and _binom_ok(su1, m, 100.0 * cfg.dt)
    # released within the capture radius of the head
    rel = q["pos"][:m][q["idBind"][:m, 0] == -1] - np.array([2.2, 2.0, 2.0])
    assert np.all(np.linalg.norm(rel, axis=1) <= 0.04 + 1e-12)
    dd = q[2 * m:]
    ds0 = int(np.sum((dd["idBind"][:, 0] == -1)))
    ds1 = int(np.sum((dd["idBind"][:, 1] == -1)))
    assert _binom_ok(ds0, m, 80.0 * cfg.dt) and _binom_ok(ds1, m, 40.0 * cfg.dt)
    assert not np.any((dd["idBind"][:, 0] == -1) & (dd["idBind"][:, 1] == -1))
    o.close()


def test_load_dependent_unbinding():
    """lambda > 0: ko_d exp(lambda kappa (l - D - ell0)^2 / (2 kT))
    (Protein/ProteinData.hpp:132-140)."""
    lam, kappa, ell0 = 0.4, 100.0, 0.02
    t = capi.make_protein_type(ko_s=(0.0, 0.0), ko_d=(5.0, 5.0), Ka=(0.0, 0.0), Ke=(0.0, 0.0), lambda_=lam,
                               kappa=kappa, freeLength=ell0)
    sep = 0.07
    o, cfg = _one_rod_system(extra=([2.0, 2.0 + sep, 2.0], [1.0, 0.0, 0.0]))
    o.set_protein_types([t], KBT, D)
    n = 40000
    p = capi.protein_array(n)
    p["gid"] = np.arange(n)
    p["idBind"][:, 0] = 0
    p["idBind"][:, 1] = 1
    p["distBind"][:] = 0.0
    o.set_proteins(p)
    st = o.protein_bind_step()
    rate = 5.0 * math.exp(lam * kappa * (sep - D - ell0) ** 2 / (2 * KBT))
    assert _binom_ok(st["nDS"], n, 2 * rate * cfg.dt)
    o.close()


def test_load_dependent_unbinding_lookup_type_1():
    """lookupType 1: the stretch is (1 - D/d) ell - ell0, d the distance of
    head 0 from the segment of head 1's rod (Protein/ProteinData.hpp:171-195)."""
    lam, kappa, ell0 = 0.4, 100.0, 0.02
    t = capi.make_protein_type(ko_s=(0.0, 0.0), ko_d=(5.0, 5.0), Ka=(0.0, 0.0), Ke=(0.0, 0.0), lambda_=lam,
                               kappa=kappa, freeLength=ell0, lookupType=1)
    sep = 0.07
    o, cfg = _one_rod_system(extra=([2.0, 2.0 + sep, 2.0], [1.0, 0.0, 0.0]))
    o.set_protein_types([t], KBT, D)
    n = 40000
    p = capi.protein_array(n)
    p["gid"] = np.arange(n)
    p["idBind"][:, 0] = 0
    p["idBind"][:, 1] = 1
    p["distBind"][:, 0] = 0.0
    p["distBind"][:, 1] = 0.03
    o.set_proteins(p)
    st = o.protein_bind_step()
    ell = math.hypot(sep, 0.03)
    stretch = (1 - D / sep) * ell - ell0
    rate = 5.0 * math.exp(lam * kappa * stretch ** 2 / (2 * KBT))
    assert _binom_ok(st["nDS"], n, 2 * rate * cfg.dt)
    o.close()


def test_springs_lookup_type_1():
    """The spring's separation is the lookupType 1 stretch at the geometry
    of the step that built it."""
    o, cfg = _one_rod_system(extra=([2.0, 2.07, 2.0], [1.0, 0.0, 0.0]))
    o.set_protein_types([capi.make_protein_type(freeLength=0.05, lookupType=1)], KBT, D)
    p = capi.protein_array(1)
    p["idBind"][0] = [0, 1]
    p["distBind"][0] = [0.0, 0.04]
    o.set_proteins(p)
    o.detect()
    c = o.constraints()
    ell = math.hypot(0.07, 0.04)
    assert c["gamma"].shape[0] - c["ncoll"] == 1
    assert abs(c["delta0"][-1] - ((1 - D / 0.07) * ell - 0.05)) < 1e-12
    o.close()


def test_mixmotor_example_fixture():
    """The MixMotorSliding example (two parallel 20 um rods, 100 doubly bound
    motors of two lookupType 1 species) read with the protein readers and
    stepped by the oracle: the stage counts against the committed golden."""
    import json
    import os
    sys_path = os.path.join(os.path.dirname(__file__), "golden")
    import sys
    sys.path.insert(0, sys_path)
    import make_fixtures as mf
    cfg, rods, kbt, species, prots = mf.load_mixmotor()
    # 97 doubly bound motors and 3 singly bound ones in the example file
    assert prots.shape[0] == 100 and np.all(prots["idBind"][:, 0] >= 0)
    assert int(np.sum(prots["idBind"][:, 1] >= 0)) == 97
    assert [t.lookupType for t in species] == [1, 1]
    g = json.load(open(os.path.join(sys_path, "mixmotor_golden.json")))
    assert mf.mixmotor_golden(g["steps"]) == g


def test_doubly_bound_proteins_become_springs():
    w = workloads.small_periodic(n=300, box=3.0, seed=2)
    pairs = workloads.pair_list(oa.OracleSystem, w.cfg, w.rods, 0.05)
    t = capi.make_protein_type(kappa=150.0, freeLength=0.03)
    prots = workloads.protein_population(w.cfg, w.rods, 500, pairs=pairs, seed=2)
    o = oa.OracleSystem(w.cfg)
    o.set_rods(w.rods)
    o.set_protein_types([t], KBT, D)
    o.set_proteins(prots)
    o.detect()
    c = o.constraints()
    nd = int(np.sum((prots["idBind"][:, 0] >= 0) & (prots["idBind"][:, 1] >= 0)))
    nb = c["gamma"].shape[0] - c["ncoll"]
    assert nd > 0 and nb == nd
    dd = prots[(prots["idBind"][:, 0] >= 0) & (prots["idBind"][:, 1] >= 0)]
    assert np.array_equal(c["i"][c["ncoll"]:], dd["idBind"][:, 0])
    assert np.array_equal(c["j"][c["ncoll"]:], dd["idBind"][:, 1])
    # delta0 = head distance - (freeLength + D), gamma0 = -kappa delta0
    a = workloads.quat_to_axis(w.rods.quat)
    box = np.array([w.cfg.simBoxHigh[k] - w.cfg.simBoxLow[k] for k in range(3)])
    P = w.rods.pos[dd["idBind"][:, 0]] + dd["distBind"][:, :1] * a[dd["idBind"][:, 0]]
    Q = w.rods.pos[dd["idBind"][:, 1]] + dd["distBind"][:, 1:] * a[dd["idBind"][:, 1]]
    dv = P - Q
    dv -= box * np.floor(dv / box + 0.5)
    assert np.allclose(c["delta0"][c["ncoll"]:], np.linalg.norm(dv, axis=1) - 0.055, atol=1e-12)
    o.close()


def test_invalid_protein_input_is_rejected():
    o, _ = _one_rod_system()
    p = capi.protein_array(1)
    with pytest.raises(capi.AlensError):
        o.set_proteins(p)                      # no species yet
    with pytest.raises(capi.AlensError):
        o.set_protein_types([capi.make_protein_type(lookupType=2)])
    with pytest.raises(capi.AlensError):
        o.set_protein_types([capi.make_protein_type(lambda_=1.0)])
    o.set_protein_types([capi.make_protein_type()])
    p["pos"] = [1.0, 1.0, 1.0]
    bad = p.copy()
    bad["type"] = 1
    with pytest.raises(capi.AlensError):
        o.set_proteins(bad)
    bad = p.copy()
    bad["idBind"][0, 0] = 5
    bad["distBind"][0, 0] = 0.0
    with pytest.raises(capi.AlensError):
        o.set_proteins(bad)
    o.set_proteins(p)
    assert o.protein_bind_step()["nU"] == 1
    o.close()


# ------------------------------------------------------------ motion step
def _motion_system(extra_axis=(1.0, 0.0, 0.0), sep=0.06, walk_type=None, boundaries=None):
    o, cfg = _one_rod_system(extra=([2.0, 2.0 + sep, 2.0], list(extra_axis)))
    if boundaries:
        o.set_boundaries(boundaries)
    o.set_protein_types([walk_type], KBT, D)
    return o, cfg


def test_unbound_diffusion():
    """Unbound proteins: pos += sqrt(2 diffUnbound dt) N(0, 1)^3
    (ProteinData::updatePosDiffuse, Protein/ProteinData.hpp:395-402)."""
    t = capi.make_protein_type(diffUnbound=2.0, Ka=(0.0, 0.0), Ke=(0.0, 0.0))
    o, cfg = _motion_system(walk_type=t)
    n = 40000
    p = capi.protein_array(n)
    p["gid"] = np.arange(n)
    p["pos"] = [1.0, 1.0, 1.0]
    o.set_proteins(p)
    st = o.protein_motion_step()
    assert st["nU"] == n
    d = o.get_proteins()["pos"] - 1.0
    msd = float(np.mean(np.sum(d * d, axis=1)))
    assert abs(msd / (6 * 2.0 * cfg.dt) - 1.0) < 0.03
    assert abs(float(np.mean(d))) < 5 * math.sqrt(2 * 2.0 * cfg.dt / (3 * n))
    o.close()


def test_singly_bound_walk_and_walk_off():
    """A singly bound head walks vmax dt (no load, Protein/ProteinData.hpp:328-331);
    past the rod end it unbinds (walkOff) or is clamped to the end."""
    for walk_off in (True, False):
        t = capi.make_protein_type(vmax=(0.8, -0.3), walkOff=walk_off, Ka=(0.0, 0.0), Ke=(0.0, 0.0),
                                   ko_s=(0.0, 0.0), ko_d=(0.0, 0.0))
        o, cfg = _motion_system(walk_type=t)
        p = capi.protein_array(3)
        p["gid"] = [0, 1, 2]
        p["idBind"][0, 0], p["distBind"][0, 0] = 0, 0.1           # end 0 walks +0.8 dt
        p["idBind"][1, 1], p["distBind"][1, 1] = 0, -0.2          # end 1 walks -0.3 dt
        p["idBind"][2, 0], p["distBind"][2, 0] = 0, 0.5 - 1e-6    # walks past the plus end
        p["pos"][2] = [2.0 + 0.5 - 1e-6, 2.0, 2.0]                 # its centre: the head
        o.set_proteins(p)
        st = o.protein_motion_step()
        q = o.get_proteins()
        assert q["distBind"][0, 0] == 0.1 + (0.8 * cfg.dt + 0.0)
        assert q["distBind"][1, 1] == -0.2 + (-0.3 * cfg.dt + 0.0)
        if walk_off:
            assert q["idBind"][2].tolist() == [-1, -1] and st["nSU"] == 1 and st["nU"] == 1
            # the centre stays at the last head position
            assert np.allclose(q["pos"][2], [2.0 + 0.5 - 1e-6, 2.0, 2.0], atol=1e-12)
        else:
            assert q["idBind"][2, 0] == 0 and q["distBind"][2, 0] == 0.5 and st["nSU"] == 0
        o.close()


def _expected_walk(t, sep, da, db, antiparallel):
    """Walk velocities of both heads of a doubly bound protein on rods along
    +x (head 0) and +x or -x (head 1) at distance sep in y, from
    ProteinData::calcEndWalkVelocity / calcEndDragVelocity and the spring
    load of updateForceTorqueBind (lookupType 0)."""
    a0 = np.array([1.0, 0.0, 0.0])
    a1 = -a0 if antiparallel else a0
    P0 = np.array([2.0, 2.0, 2.0]) + da * a0
    P1 = np.array([2.0, 2.0 + sep, 2.0]) + db * a1
    r = P0 - P1
    ell = np.linalg.norm(r)
    force = (ell - D - t.freeLength) * t.kappa
    f = [-force * r / ell, force * r / ell]
    out = []
    for e, a in enumerate((a0, a1)):
        fdir = float(f[e] @ a)
        sgn = np.sign(t.vmax[e])
        vfrac = min(1.0, max(0.0, 1.0 + sgn * fdir / abs(t.fstall)))
        vel = (t.vmaxAP[e] if antiparallel else t.vmax[e]) * vfrac
        drag = fdir * t.diffBoundD[e] / KBT if t.vdrag[e] else 0.0
        out.append(vel + drag)
    return out


@pytest.mark.parametrize("antiparallel", [False, True])
def test_doubly_bound_walk_under_load(antiparallel):
    """Each head walks vmax (vmaxAP on antiparallel rods) times
    clamp(1 + sign(vmax) f.dir / fstall, 0, 1), f the spring load
    (Protein/ProteinData.hpp:418-478)."""
    t = capi.make_protein_type(vmax=(0.6, -0.4), vmaxAP=(0.2, -0.1), fstall=3.0, kappa=200.0, freeLength=0.02,
                               Ka=(0.0, 0.0), Ke=(0.0, 0.0), ko_s=(0.0, 0.0), ko_d=(0.0, 0.0))
    ax = (-1.0, 0.0, 0.0) if antiparallel else (1.0, 0.0, 0.0)
    o, cfg = _motion_system(extra_axis=ax, sep=0.06, walk_type=t)
    da, db = np.array([0.0, 0.05, -0.1]), np.array([0.03, -0.02, 0.0])
    p = capi.protein_array(3)
    p["gid"] = [0, 1, 2]
    p["idBind"][:] = [0, 1]
    p["distBind"][:, 0], p["distBind"][:, 1] = da, db
    o.set_proteins(p)
    o.protein_motion_step()
    q = o.get_proteins()
    for k in range(3):
        v = _expected_walk(t, 0.06, da[k], db[k], antiparallel)
        assert abs(q["distBind"][k, 0] - (da[k] + v[0] * cfg.dt)) < 1e-15
        assert abs(q["distBind"][k, 1] - (db[k] + v[1] * cfg.dt)) < 1e-15
    o.close()


def test_drag_and_bound_diffusion():
    """vdrag adds load x diffBoundD / KBT to a doubly bound head's velocity;
    the head also diffuses with diffBoundD (mean over many proteins)."""
    t = capi.make_protein_type(vmax=(0.0, 0.0), vdrag=(True, True), diffBoundD=(0.05, 0.05), kappa=200.0,
                               freeLength=0.02, Ka=(0.0, 0.0), Ke=(0.0, 0.0), ko_s=(0.0, 0.0), ko_d=(0.0, 0.0))
    o, cfg = _motion_system(sep=0.06, walk_type=t)
    n = 20000
    p = capi.protein_array(n)
    p["gid"] = np.arange(n)
    p["idBind"][:] = [0, 1]
    p["distBind"][:] = [0.0, 0.04]
    o.set_proteins(p)
    o.protein_motion_step()
    q = o.get_proteins()
    v = _expected_walk(t, 0.06, 0.0, 0.04, False)
    sd = math.sqrt(2 * 0.05 * cfg.dt)
    for e, d0 in enumerate((0.0, 0.04)):
        mean = float(np.mean(q["distBind"][:, e] - d0))
        assert abs(mean - v[e] * cfg.dt) < 5 * sd / math.sqrt(n)
        assert abs(float(np.std(q["distBind"][:, e])) / sd - 1.0) < 0.05
    o.close()


def test_doubly_bound_both_ends_off():
    """Both heads past their rod ends: one head, chosen by the roll with
    probability 1/2, unbinds; the other is clamped (Protein/ProteinData.hpp:352-381)."""
    t = capi.make_protein_type(vmax=(1.0, -1.0), fstall=1e9, Ka=(0.0, 0.0), Ke=(0.0, 0.0), ko_s=(0.0, 0.0),
                               ko_d=(0.0, 0.0))
    o, cfg = _motion_system(sep=0.06, walk_type=t)
    n = 4000
    p = capi.protein_array(n)
    p["gid"] = np.arange(n)
    p["idBind"][:] = [0, 1]
    p["distBind"][:] = [0.5 - 1e-6, -0.5 + 1e-6]
    o.set_proteins(p)
    st = o.protein_motion_step()
    q = o.get_proteins()
    assert st["nDS"] == n and st["nS"] == n
    k0 = int(np.sum(q["idBind"][:, 0] == -1))
    assert _binom_ok(k0, n, 0.5)
    kept0 = q["idBind"][:, 0] == 0
    assert np.all(q["distBind"][kept0, 0] == 0.5) and np.all(q["distBind"][~kept0, 1] == -0.5)
    o.close()


def test_unbound_boundary_projection():
    """Unbound proteins outside a boundary after the motion are moved onto it
    (SRC/TubuleSystem.cpp:285-305): wall, and inside a sphere."""
    t = capi.make_protein_type(diffUnbound=0.0, Ka=(0.0, 0.0), Ke=(0.0, 0.0))
    wall = capi.make_boundary(capi.BOUNDARY_WALL, center=(0.0, 0.0, 1.5), axis=(0.0, 0.0, 1.0))
    sph = capi.make_boundary(capi.BOUNDARY_SPHERE, center=(2.0, 2.0, 2.0), radius=1.2, inside=True)
    o, cfg = _motion_system(walk_type=t, boundaries=[wall, sph])
    p = capi.protein_array(3)
    p["gid"] = [0, 1, 2]
    p["pos"] = [[2.0, 2.0, 1.2], [2.0, 3.5, 2.0], [2.1, 2.0, 2.0]]
    o.set_proteins(p)
    o.protein_motion_step()
    q = o.get_proteins()
    assert np.allclose(q["pos"][0], [2.0, 2.0, 1.5], atol=1e-12)      # onto the wall
    assert np.allclose(q["pos"][1], [2.0, 3.2, 2.0], atol=1e-12)      # onto the sphere
    assert np.allclose(q["pos"][2], [2.1, 2.0, 2.0], atol=1e-15)      # inside both: unchanged
    o.close()


def test_protein_snapshot_restart_round_trip(tmp_path):
    """write_snapshot(proteins=...) writes ProteinAscii_<id>.dat and
    Protein_<id>.pvtp; reading the .pvtp back and rebuilding the bindings
    (the restart of TubuleSystem::readProteinVTK) gives the same stages,
    rods and arc positions."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_fixtures as mf
    from alens_gb300 import io
    cfg, rods, kbt, species, prots = mf.load_mixmotor()
    o = oa.OracleSystem(cfg)
    o.set_rods(rods)
    o.set_protein_types(species, kbt, mf.cfg_diameter(cfg))
    o.set_proteins(prots)
    for _ in range(2):
        o.protein_motion_step()
        o.protein_bind_step()
        o.step()
    # the snapshot is taken where aLENS writes it: after the binding step,
    # before the rods move (SRC/TubuleSystem.cpp:205-224)
    o.protein_motion_step()
    o.protein_bind_step()
    q = o.get_proteins()
    pos, quat = o.get_rods()
    o.close()
    now = capi.RodState(rods.gid, pos, quat, rods.length, rods.radius, rods.immovable)
    folder = io.write_snapshot(3, now, step=2, time=2 * cfg.dt, root=str(tmp_path / "result"),
                               info_path=str(tmp_path / "TimeStepInfo.txt"), proteins=q, species=species)
    assert os.path.exists(folder + "ProteinAscii_3.dat") and os.path.exists(folder + "Protein_r0_3.vtp")
    back = io.proteins_from_ascii(io.read_protein_pvtp(folder + "Protein_3.pvtp"), now, species, cfg)
    assert np.array_equal(back["idBind"], q["idBind"]) and np.array_equal(back["gid"], q["gid"])
    bound = q["idBind"] >= 0
    assert np.allclose(back["distBind"][bound], q["distBind"][bound], rtol=0, atol=1e-12)
    txt = io.read_protein_ascii(folder + "ProteinAscii_3.dat")
    assert np.array_equal(txt["gid"], q["gid"])
