"""Confinement boundaries (walls, spheres, tubes).

CPU: the oracle's boundary constraints on hand-built cases (a rod poking
through a wall is pushed back along the wall normal; rods in a spherical
cavity stay inside; a rod against an outside sphere touches it at the point
nearest the centre).  GPU: the library's boundary constraints, pair set,
multipliers and trajectory equal the oracle's bit for bit.
"""
import numpy as np
import pytest

from alens_gb300 import capi, workloads
from alens_gb300.oracle_api import OracleSystem

R = 0.0125


def rods_of(pos, axes, length):
    n = len(pos)
    return capi.RodState(np.arange(n), np.asarray(pos, float), workloads.axis_to_quat(np.asarray(axes, float)),
                         np.asarray(length, float), np.full(n, R))


def test_wall_pushes_rod_back(oracle_lib):
    # rod along z whose lower end pokes 0.05 um through the wall z = 0
    cfg = capi.make_config(box_low=(-2, -2, -2), box_high=(2, 2, 2), pbc=(0, 0, 0), kbt=-1.0)
    rods = rods_of([[0.0, 0.0, 0.45]], [[0.0, 0.3, 1.0]], [1.0])
    o = OracleSystem(cfg)
    o.set_rods(rods)
    o.set_boundaries([capi.make_boundary(capi.BOUNDARY_WALL, center=(0, 0, 0), axis=(0, 0, 2))])
    o.detect()
    con = o.constraints()
    assert con["ncoll"] == 1 and con["j"][0] == -1 and con["image"][0] == 27
    assert con["jac"][0][:3].tolist() == [0.0, 0.0, 1.0]      # force along the wall normal
    a = workloads.quat_to_axis(rods.quat)[0]
    end = rods.pos[0] - 0.5 * a
    assert con["delta0"][0] == pytest.approx(end[2] - R)        # separation of the lower end
    o.solve()
    o.advance()
    pos, quat = o.get_rods()
    a2 = workloads.quat_to_axis(quat)[0]
    low = (pos[0] - 0.5 * a2)[2] - R
    assert low > -2e-5                                          # no longer through the wall


def test_spherical_cavity_keeps_rods_inside(oracle_lib):
    rng = np.random.default_rng(3)
    n = 300
    d = rng.standard_normal((n, 3))
    pos = 0.6 * rng.random((n, 1)) ** (1 / 3) * d / np.linalg.norm(d, axis=1, keepdims=True)
    rods = rods_of(pos, workloads.isotropic_axes(rng, n), rng.uniform(0.2, 0.6, n))
    cfg = capi.make_config(box_low=(-2, -2, -2), box_high=(2, 2, 2), pbc=(0, 0, 0), max_ite=20000)
    o = OracleSystem(cfg)
    o.set_rods(rods)
    o.set_boundaries([capi.make_boundary(capi.BOUNDARY_SPHERE, center=(0, 0, 0), radius=0.8, inside=True)])
    for _ in range(5):
        st = o.step()
        assert st["converged"] == 1
    p, q = o.get_rods()
    a = workloads.quat_to_axis(q)
    ends = np.concatenate([p - 0.5 * rods.length[:, None] * a, p + 0.5 * rods.length[:, None] * a])
    assert np.max(np.linalg.norm(ends, axis=1)) <= 0.8 - R + 1e-3


def test_outside_sphere_contact_point(oracle_lib):
    # rod tangent above a sphere obstacle: contact at the rod point nearest
    # the centre, normal pointing away from the centre
    cfg = capi.make_config(box_low=(-2, -2, -2), box_high=(2, 2, 2), pbc=(0, 0, 0), kbt=-1.0)
    rods = rods_of([[0.1, 0.0, 0.51]], [[1.0, 0.0, 0.0]], [1.0])
    o = OracleSystem(cfg)
    o.set_rods(rods)
    o.set_boundaries([capi.make_boundary(capi.BOUNDARY_SPHERE, center=(0, 0, 0), radius=0.5, inside=False)])
    o.detect()
    con = o.constraints()
    assert con["ncoll"] == 1 and con["image"][0] == 27
    assert np.allclose(con["jac"][0][:3], [0, 0, 1])
    assert con["delta0"][0] == pytest.approx(0.01 - R)


@pytest.mark.gpu
def test_boundaries_gpu_parity(gpu_lib):
    """Rods in a tube with an end wall and an outside-sphere obstacle
    (Examples/DenseStrainingMotion-like confinement): GPU = oracle."""
    rng = np.random.default_rng(11)
    n = 2500
    x = rng.uniform(0.1, 3.9, n)
    rr = 0.45 * np.sqrt(rng.random(n))
    th = rng.uniform(0, 2 * np.pi, n)
    pos = np.stack([x, 0.5 + rr * np.cos(th), 0.5 + rr * np.sin(th)], axis=1)
    ax = workloads.isotropic_axes(rng, n)
    ax[:, 0] += 2.0
    rods = rods_of(pos, ax, rng.uniform(0.2, 0.5, n))
    cfg = capi.make_config(box_low=(0, -1, -1), box_high=(4, 2, 2), pbc=(1, 0, 0), max_ite=20000)
    bnd = [capi.make_boundary(capi.BOUNDARY_TUBE, center=(1, 0.5, 0.5), axis=(1, 0, 0), radius=0.5),
           capi.make_boundary(capi.BOUNDARY_WALL, center=(0.05, 0, 0), axis=(1, 0, 0)),
           capi.make_boundary(capi.BOUNDARY_SPHERE, center=(2.0, 0.5, 0.5), radius=0.15, inside=False)]
    g = capi.GpuSystem(cfg)
    o = OracleSystem(cfg)
    for s in (g, o):
        s.set_rods(rods)
        s.set_boundaries(bnd)
    nb = 0
    for _ in range(5):
        sg, so = g.step(), o.step()
        assert sg["nCollision"] == so["nCollision"]
        assert sg["iterations"] == so["iterations"]
        cg, co = g.constraints(), o.constraints()
        assert np.array_equal(cg["i"], co["i"]) and np.array_equal(cg["j"], co["j"])
        assert np.array_equal(cg["image"], co["image"])
        assert np.array_equal(cg["gamma"], co["gamma"])
        nb = int(np.sum(cg["image"] >= 27))
    assert nb > 10
    pg, qg = g.get_rods()
    po, qo = o.get_rods()
    assert np.array_equal(pg, po) and np.array_equal(qg, qo)


BOUNDARY_YAML = """rngSeed: 99
simBoxLow: [0, -1, -1]
simBoxHigh: [4, 2, 2]
simBoxPBC: [true, false, false]
monolayer: false
viscosity: 0.01
KBT: 0.00411
linkKappa: 100
sylinderDiameter: 0.025
sylinderColBuf: 0.025
dt: 0.0001
conResTol: 1e-5
conMaxIte: 20000
conSolverChoice: 0
boundaries:
  - type: "tube"
    center: [1, 0.5, 0.5]
    radius: 0.5
    axis: [1, 0, 0]
    inside: true
  # an obstacle
  - type: 'sphere'
    center: [2.0, 0.5, 0.5]
    radius: 0.15
    inside: false
"""


def test_read_boundaries(tmp_path):
    from alens_gb300 import io
    p = tmp_path / "run.yaml"
    p.write_text(BOUNDARY_YAML)
    b = io.read_boundaries(str(p))
    assert [x.type for x in b] == [capi.BOUNDARY_TUBE, capi.BOUNDARY_SPHERE]
    assert list(b[0].center) == [1, 0.5, 0.5] and list(b[0].axis) == [1, 0, 0] and b[0].inside == 1
    assert b[1].radius == 0.15 and b[1].inside == 0


@pytest.mark.gpu
def test_facade_reads_boundaries(gpu_lib, tmp_path):
    """The C++ facade parses `boundaries:` and confines the rods exactly as
    the C ABI does with the Python reader's boundaries."""
    import json
    import subprocess
    import sys
    from alens_gb300 import build, io
    sys.path.insert(0, str(__import__("pathlib").Path(__file__).parent / "golden"))
    import make_fixtures
    rng = np.random.default_rng(5)
    n = 800
    pos = np.stack([rng.uniform(0.1, 3.9, n), 0.5 + 0.3 * rng.uniform(-1, 1, n),
                    0.5 + 0.3 * rng.uniform(-1, 1, n)], axis=1)
    rods = rods_of(pos, workloads.isotropic_axes(rng, n), rng.uniform(0.2, 0.5, n))
    yml = tmp_path / "run.yaml"
    yml.write_text(BOUNDARY_YAML)
    dat = tmp_path / "rods.dat"
    io.write_sylinder_ascii(str(dat), rods)
    steps = 4
    proc = subprocess.run([str(build.build_facade_driver()), str(yml), str(dat), str(steps)],
                          capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    res = json.loads(proc.stdout.strip().splitlines()[-1])
    cfg = io.read_run_config(str(yml))
    rods2, _ = io.read_sylinder_ascii(str(dat))
    g = capi.GpuSystem(cfg)
    g.set_rods(rods2)
    g.set_boundaries(io.read_boundaries(str(yml)))
    its = 0
    for _ in range(steps):
        p, _ = g.get_rods()
        g.add_bilateral([make_fixtures.spring_block(p, rods2.gid, 100.0)])
        its += g.step()["iterations"]
    pg, _ = g.get_rods()
    assert res["iterations"] == its
    assert res["rod0"] == pg[0].tolist()
