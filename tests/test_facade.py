"""GPU tests of the drop-in boundary on the monolayer window fixture:
the C ABI and the C++ SylinderSystem facade (run as a TubuleSystem-like
driver) reproduce the oracle's golden outputs."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from alens_gb300 import build, capi

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)
import make_fixtures  # noqa: E402

pytestmark = pytest.mark.gpu


def golden():
    with open(os.path.join(GOLDEN, "monolayer_window_golden.json")) as f:
        return json.load(f)


def test_c_abi_reproduces_golden(gpu_lib):
    gold = golden()
    cfg, rods = make_fixtures.load_fixture()
    g = capi.GpuSystem(cfg)
    g.set_rods(rods)
    its, coll = [], []
    for _ in range(gold["steps"]):
        pos, _ = g.get_rods()
        g.add_bilateral([make_fixtures.spring_block(pos, rods.gid, 1000.0)])
        st = g.step()
        its.append(st["iterations"])
        coll.append(st["nCollision"])
    pos, quat = g.get_rods()
    s9 = g.con_stress()
    assert its == gold["iterations"] and coll == gold["collisions"]
    assert pos[0].tolist() == gold["rod0"]
    assert pos[:8].tolist() == gold["pos_head"] and quat[:8].tolist() == gold["quat_head"]
    assert float(s9[0, 0] + s9[1, 1] + s9[2, 2]) == gold["stress_trace"]


def test_facade_driver_reproduces_golden(gpu_lib, tmp_path):
    gold = golden()
    exe = build.build_facade_driver()
    out = tmp_path / "result.dat"
    proc = subprocess.run([str(exe), os.path.join(GOLDEN, "monolayer_window.yaml"),
                           os.path.join(GOLDEN, "monolayer_window.dat"), str(gold["steps"]), str(out)],
                          capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    res = json.loads(proc.stdout.strip().splitlines()[-1])
    assert res["rods"] == gold["rods"] and res["steps"] == gold["steps"]
    assert res["iterations"] == sum(gold["iterations"])
    assert res["collisions"] == sum(gold["collisions"])
    assert res["rod0"] == gold["rod0"]
    assert np.allclose(res["sum_pos"], gold["sum_pos"], rtol=1e-12)
    assert res["stress_trace"] == gold["stress_trace"]
    from alens_gb300 import io
    back, _ = io.read_sylinder_ascii(str(out))
    assert back.n == gold["rods"]
    assert np.allclose(back.pos[0], gold["rod0"], atol=1e-12)


def _write_filament(tmp_path, n=100, radius=0.01, gap=0.0002):
    """A straight bead chain in the Examples/FlexibleFilament layout:
    zero-length rods (spheres) along x, 'L a b' lines joining neighbours."""
    lines = ["# flexible filament", "#"]
    x0 = -1.0
    for k in range(n):
        x = x0 + k * (2 * radius + gap)
        lines.append(f"C {k} {radius} {x:.6f} 0.010000 0.000000 {x + 1e-6:.6f} 0.010000 0.000000 0")
    for k in range(n - 1):
        lines.append(f"L {k} {k + 1}")
    dat = tmp_path / "filament.dat"
    dat.write_text("\n".join(lines) + "\n")
    yml = tmp_path / "filament.yaml"
    yml.write_text("""rngSeed: 1234
simBoxLow: [-5.0, -5.0, -5.0]
simBoxHigh: [5.0, 5.0, 5.0]
simBoxPBC: [false, false, false]
monolayer: false
viscosity: 1
KBT: 0.00411
linkKappa: 3650
linkGap: .0002
sylinderDiameter: 0.02
sylinderDiameterColRatio: 1.0
sylinderLengthColRatio: 1.0
sylinderColBuf: 0.02
dt: .0001
timeTotal: 1.
conResTol: 1e-5
conMaxIte: 100000
conSolverChoice: 0
""")
    return str(yml), str(dat)


def test_flexible_filament_links(gpu_lib, tmp_path):
    """'L' link lines become device-built springs (linkKappa, surfaces
    linkGap apart) in the C++ facade exactly as in the Python reader; the
    C ABI run equals the facade driver's and the oracle's bit for bit."""
    from alens_gb300 import io
    from alens_gb300.oracle_api import OracleSystem
    yml, dat = _write_filament(tmp_path)
    steps = 5
    exe = build.build_facade_driver()
    proc = subprocess.run([str(exe), yml, dat, str(steps)], capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    res = json.loads(proc.stdout.strip().splitlines()[-1])
    cfg = io.read_run_config(yml)
    rods, pairs = io.read_sylinder_ascii(dat)
    assert len(pairs) == rods.n - 1
    kappa, gap = io.read_link_params(yml)
    links = io.filament_links(rods, pairs, kappa, gap)
    g = capi.GpuSystem(cfg)
    o = OracleSystem(cfg)
    its = 0
    for s in (g, o):
        s.set_rods(rods)
        s.set_links(links)
    for _ in range(steps):
        pos, _ = g.get_rods()
        blk = make_fixtures.spring_block(pos, rods.gid, kappa)
        g.add_bilateral([blk])
        o.add_bilateral([blk])
        sg, so = g.step(), o.step()
        assert sg["nBilateral"] == so["nBilateral"] == rods.n
        assert sg["iterations"] == so["iterations"]
        its += sg["iterations"]
    pg, _ = g.get_rods()
    po, _ = o.get_rods()
    assert np.array_equal(pg, po)
    assert res["iterations"] == its
    assert res["rod0"] == pg[0].tolist()
    assert np.allclose(res["sum_pos"], pg.sum(axis=0), rtol=1e-12)
    # the chain holds together: neighbour spacing stays near 2r + gap
    d = np.linalg.norm(np.diff(pg, axis=0), axis=1)
    assert np.all(np.abs(d[1:] - (0.02 + gap)) < 0.01)


def test_facade_snapshot_and_restart(gpu_lib, tmp_path):
    """writeResult() before every runStep writes SylinderAscii_<snapID>.dat,
    Sylinder_<snapID>.pvtp (+ piece) and ConBlock_<snapID>.pvtp (+ piece)
    into ./result/result0-399/ every
    round(timeSnap/dt) steps plus
    ./TimeStepInfo.txt; reinitialize from TimeStepInfo.txt restores the last
    snapshot's rods, its snapID + 1 and its step."""
    exe = build.build_facade_driver()
    with open(os.path.join(GOLDEN, "monolayer_window.yaml")) as f:
        text = f.read()
    yml = tmp_path / "RunConfig.yaml"
    yml.write_text(text + "timeSnap: 0.00002\n")  # every 2 steps (dt = 1e-5)
    proc = subprocess.run([str(exe), "--restart-check", str(yml), os.path.join(GOLDEN, "monolayer_window.dat"), "5"],
                          capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert proc.returncode == 0, proc.stderr
    r = json.loads(proc.stdout.strip().splitlines()[-1])
    assert r["steps"] == 5 and r["snap_id_after"] == 3  # steps 0, 2, 4
    assert r["last_snap_id"] == 2 and r["last_snap_step"] == 4
    assert r["restart_snap_id"] == 3 and r["restart_step"] == 4
    assert r["same_count"] == 1 and r["max_dpos"] < 1e-12 and r["max_daxis"] < 1e-12
    folder = tmp_path / "result" / "result0-399"
    names = sorted(p.name for p in folder.iterdir())
    assert [x for x in names if x.startswith("SylinderAscii_")] == [f"SylinderAscii_{i}.dat" for i in range(3)]
    assert [x for x in names if x.startswith("Sylinder_") and x.endswith(".pvtp")] == \
        [f"Sylinder_{i}.pvtp" for i in range(3)]
    assert [x for x in names if x.startswith("Sylinder_r0_")] == [f"Sylinder_r0_{i}.vtp" for i in range(3)]
    # the constraint blocks of the last runStep beside every rod snapshot (none
    # before the first step)
    assert [x for x in names if x.startswith("ConBlock_") and x.endswith(".pvtp")] == \
        [f"ConBlock_{i}.pvtp" for i in range(3)]
    assert [x for x in names if x.startswith("ConBlock_r0_")] == [f"ConBlock_r0_{i}.vtp" for i in range(3)]
    assert 'NumberOfLines="0"' in (folder / "ConBlock_r0_0.vtp").read_text()
    assert 'NumberOfLines="0"' not in (folder / "ConBlock_r0_2.vtp").read_text()
    assert len(names) == 15
    assert (tmp_path / "TimeStepInfo.txt").read_text().split()[:2] == ["4", "2"]


def test_facade_protein_steps_match_oracle(gpu_lib, tmp_path):
    """TubuleSystem::step()'s order through the facade (updateProteinMotion,
    calcBindInteraction, then runStep) on the MixMotorSliding example: two
    parallel 20 um rods,
    100 motors of two lookupType 1 species read from its ProteinInitial.dat.
    After five steps the proteins and the per-step counts equal the oracle's
    and the committed golden."""
    cfg, rods, kbt, species, prots = make_fixtures.load_mixmotor()
    gold = json.load(open(os.path.join(GOLDEN, "mixmotor_golden.json")))
    setup = tmp_path / "setup.txt"
    with open(setup, "w") as f:
        for t in species:
            f.write("S %d %d %d %d %r %r %r %r %r %r %r %r %r %r %r %r %r %r %r" % (
                t.tag, t.fixedEnd0, t.useBindVol, t.lookupType, t.freeLength, t.kappa, t.lambda_, t.PtoAPratio,
                t.diffUnbound, t.rc, t.eps, t.ko_s[0], t.ko_s[1], t.ko_d[0], t.ko_d[1], t.Ka[0], t.Ka[1], t.Ke[0],
                t.Ke[1]))
            f.write(" %d %d %d %r %r %r %r %r %r %r %r %r\n" % (
                t.walkOff, t.vdrag[0], t.vdrag[1], t.fstall, t.vmax[0], t.vmax[1], t.vmaxAP[0], t.vmaxAP[1],
                t.diffBoundS[0], t.diffBoundS[1], t.diffBoundD[0], t.diffBoundD[1]))
        for p in prots:
            f.write("P %d %d %d %d %r %r %r %r %r\n" % (int(p["gid"]), int(p["type"]), int(p["idBind"][0]),
                                                      int(p["idBind"][1]), float(p["distBind"][0]),
                                                      float(p["distBind"][1]), *map(float, p["pos"])))
    out = tmp_path / "out.txt"
    exe = build.build_facade_driver()
    steps = gold["steps"]
    proc = subprocess.run([str(exe), "--proteins", os.path.join(GOLDEN, "mixmotor_run.yaml"),
                           os.path.join(GOLDEN, "mixmotor_tubules.dat"), str(setup), repr(kbt), str(steps), str(out)],
                          capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    res = json.loads(proc.stdout.strip().splitlines()[-1])
    assert res["counts"] == gold["counts"] and res["step_count"] == steps
    from alens_gb300.oracle_api import OracleSystem
    o = OracleSystem(cfg)
    o.set_rods(rods)
    o.set_protein_types(species, kbt, make_fixtures.cfg_diameter(cfg))
    o.set_proteins(prots)
    for _ in range(steps):
        o.protein_motion_step()
        o.protein_bind_step()
        o.step()
    q = o.get_proteins()
    o.close()
    rows = [ln.split() for ln in out.read_text().splitlines()]
    assert len(rows) == q.shape[0]
    for r, p in zip(rows, q):
        assert int(r[0]) == int(p["gid"]) and int(r[1]) == int(p["type"])
        assert [int(r[2]), int(r[3])] == p["idBind"].tolist()
        got = np.array([float(v) for v in r[4:]])
        want = np.concatenate([p["distBind"], p["pos"], p["posEnd"].ravel()])
        assert np.array_equal(got, want, equal_nan=True)
