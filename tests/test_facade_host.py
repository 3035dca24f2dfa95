"""CPU tests of the C++ SylinderSystem facade's single-rank getters: result
folders and snapshot schedule, domain, communicator and the per-thread
random pool (no device call)."""
import json
import subprocess

from alens_gb300 import build

YAML = """rngSeed: 99
simBoxLow: [0.0, -1.0, 2.0]
simBoxHigh: [40.0, 39.0, 2.5]
simBoxPBC: [true, true, false]
dt: 0.0001
timeSnap: 0.01
"""


def _host_checks(tmp_path, text=YAML):
    build.build_lib()
    exe = build.build_facade_driver()
    yml = tmp_path / "RunConfig.yaml"
    yml.write_text(text)
    proc = subprocess.run([str(exe), "--host-checks", str(yml)], capture_output=True, text=True, timeout=120)
    assert proc.returncode == 0, proc.stderr
    return json.loads(proc.stdout.strip().splitlines()[-1])


def test_result_folders_and_snapshot_schedule(tmp_path):
    r = _host_checks(tmp_path)
    # 400 snapshots per folder: result0-399, result400-799, ...
    assert r["folders"] == ["./result/result0-399/", "./result/result0-399/", "./result/result400-799/",
                            "./result/result1200-1599/"]
    assert r["snap_every"] == 100  # timeSnap / dt
    assert r["due"] == [1, 0, 1, 0]  # steps 0, 1, 100, 301


def test_domain_and_single_rank(tmp_path):
    r = _host_checks(tmp_path)
    assert r["low"] == [0.0, -1.0, 2.0] and r["high"] == [40.0, 39.0, 2.5]
    assert r["pbc"] == [1, 1, 0] and r["len0"] == 40.0
    assert r["rank"] == 0 and r["size"] == 1


def test_random_pool_streams(tmp_path):
    r = _host_checks(tmp_path)
    # 200,000 draws: U(0,1) mean 1/2, variance 1/12, open interval; N(0,1)
    assert abs(r["u_mean"] - 0.5) < 0.005 and abs(r["u_var"] - 1.0 / 12.0) < 0.002
    assert 0.0 < r["u_min"] and r["u_max"] < 1.0
    assert abs(r["n_mean"]) < 0.01 and abs(r["n_var"] - 1.0) < 0.02
    # same seed, same streams; streams of different threads differ
    assert r["again1_first"] == r["stream1_first"]
    assert r["again0_first"] != r["again1_first"]
    assert r["out_of_range"] == 1
    other = _host_checks(tmp_path, YAML.replace("rngSeed: 99", "rngSeed: 100"))
    assert other["again0_first"] != r["again0_first"]


def test_time_step_info_restart_files(tmp_path):
    from alens_gb300 import io
    info = tmp_path / "TimeStepInfo.txt"
    io.write_time_step_info(info, 1200, 12, 0.12)
    snap = tmp_path / "SylinderAscii_12.dat"
    snap.write_text("2\n0.12\nC 0 0.0125 0 0 0 1 0 0 0\nC 1 0.0125 0 1 0 1 1 0 0\n")
    short = tmp_path / "short.txt"
    short.write_text("1 2\n")
    build.build_lib()
    exe = build.build_facade_driver()
    yml = tmp_path / "RunConfig.yaml"
    yml.write_text(YAML)
    proc = subprocess.run([str(exe), "--host-checks", str(yml), str(info), str(snap), str(short),
                           str(tmp_path / "absent.txt")], capture_output=True, text=True, timeout=120)
    assert proc.returncode == 0, proc.stderr
    r = json.loads(proc.stdout.strip().splitlines()[-1])["restart"]
    # the Python writer and the facade reader agree; snapshots and anything
    # else are not taken for restart bookkeeping
    assert r[0] == [1, 1200, 12, 0.12]
    assert [x[0] for x in r[1:]] == [0, 0, 0]
    assert io.read_time_step_info(info) == (1200, 12, 0.12)


def test_facade_vtk_writer_matches_python(tmp_path):
    """The facade's Sylinder_<id>.pvtp / Sylinder_r0_<id>.vtp writer and the
    Python one produce the same bytes for the same rods (both read from the
    same TubuleInitial.dat by bit-identical readers)."""
    import os
    from alens_gb300 import io
    dat = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "monolayer_window.dat")
    build.build_lib()
    exe = build.build_facade_driver()
    cpp, py = tmp_path / "cpp", tmp_path / "py"
    cpp.mkdir()
    py.mkdir()
    proc = subprocess.run([str(exe), "--write-vtk", dat, str(cpp), "7"], capture_output=True, text=True, timeout=120)
    assert proc.returncode == 0, proc.stderr
    rods, _ = io.read_sylinder_ascii(dat)
    io.write_sylinder_pvtp(str(py), 7, rods)
    for name in ("Sylinder_7.pvtp", "Sylinder_r0_7.vtp"):
        assert (cpp / name).read_bytes() == (py / name).read_bytes(), name


def test_facade_conblock_writer_matches_python(tmp_path):
    """The facade's ConBlock_<id>.pvtp / ConBlock_r0_<id>.vtp writer and the
    Python one produce the same bytes for the same blocks: collisions, a
    boundary contact (no rod J), crosslinker springs, and an empty set."""
    import numpy as np
    from alens_gb300 import io
    rng = np.random.default_rng(3)
    n = 40
    gid = np.arange(100, 160, dtype=np.int64)
    j = rng.integers(0, 60, n).astype(np.int32)
    j[5] = -1
    blocks = {"i": rng.integers(0, 60, n).astype(np.int32), "j": j, "image": rng.integers(0, 27, n).astype(np.int32),
              "delta0": rng.normal(0, 0.01, n), "gamma": np.abs(rng.normal(0, 0.3, n)), "normI": rng.normal(0, 1, (n, 3)),
              "labI": rng.uniform(0, 5, (n, 3)), "labJ": rng.uniform(0, 5, (n, 3)),
              "kappa": np.where(np.arange(n) >= 30, 100.0, 0.0), "bilateral": (np.arange(n) >= 30).astype(np.int32),
              "oneSide": (j < 0).astype(np.int32)}
    build.build_lib()
    exe = build.build_facade_driver()
    for label, sel in (("some", np.arange(n)), ("none", np.arange(0))):
        b = {k: np.asarray(v)[sel] for k, v in blocks.items()}
        cells = io.conblock_cells(b, gid)
        rec = tmp_path / f"{label}.txt"
        with open(rec, "w") as f:
            for k in range(sel.shape[0]):
                vals = [cells["gamma"][k], cells["delta0"][k], cells["kappa"][k], cells["bilateral"][k],
                        cells["oneSide"][k], cells["gidI"][k], cells["gidJ"][k], cells["globalIndexI"][k],
                        cells["globalIndexJ"][k], cells["image"][k], *b["normI"][k], *b["labI"][k], *b["labJ"][k]]
                f.write(" ".join(repr(float(v)) if isinstance(v, (float, np.floating)) else str(int(v))
                                 for v in vals) + "\n")
        cpp, py = tmp_path / f"cpp_{label}", tmp_path / f"py_{label}"
        cpp.mkdir()
        py.mkdir()
        proc = subprocess.run([str(exe), "--write-conblock", str(rec), str(cpp), "4"], capture_output=True,
                              text=True, timeout=120)
        assert proc.returncode == 0, proc.stderr
        io.write_conblock_pvtp(str(py), 4, b, gid)
        for name in ("ConBlock_4.pvtp", "ConBlock_r0_4.vtp"):
            assert (cpp / name).read_bytes() == (py / name).read_bytes(), (label, name)


def test_facade_protein_ascii_writer_matches_python(tmp_path):
    """The facade's ProteinAscii and Protein_<id>.pvtp writers
    (SylinderSystem::writeProteinAscii / writeProteinVTK) and
    io.write_protein_ascii / write_protein_pvtp produce the same bytes:
    doubly bound (head positions), singly bound and unbound (the centre
    twice) proteins of two species, rod gids for the bound ends; both read
    back."""
    import numpy as np
    from alens_gb300 import capi, io
    rng = np.random.default_rng(5)
    n = 30
    species = [capi.make_protein_type(tag=7), capi.make_protein_type(tag=2)]
    rod_gid = np.arange(1000, 1040, dtype=np.int64)
    p = capi.protein_array(n)
    p["gid"] = rng.integers(0, 10**6, n)
    p["type"] = np.arange(n) % 2
    p["pos"] = rng.uniform(-3, 40, (n, 3))
    p["idBind"][:10] = rng.integers(0, 40, (10, 2))
    p["posEnd"][:10] = rng.uniform(0, 40, (10, 2, 3)) * 1.0000001
    p["idBind"][10:20, 0] = rng.integers(0, 40, 10)
    p["posEnd"][10:20, 0] = rng.uniform(0, 40, (10, 3))
    p["pos"][5] = [1e-7, -2.5e-5, 123456.789]
    build.build_lib()
    exe = build.build_facade_driver()
    rec = tmp_path / "prot.txt"
    with open(rec, "w") as f:
        f.write("T " + " ".join(str(t.tag) for t in species) + "\n")
        f.write("R " + " ".join(str(int(g)) for g in rod_gid) + "\n")
        for q in p:
            vals = [int(q["gid"]), int(q["type"]), int(q["idBind"][0]), int(q["idBind"][1])]
            vals += [repr(float(v)) for v in (*q["pos"], *q["posEnd"][0], *q["posEnd"][1])]
            f.write(" ".join(str(v) for v in vals) + "\n")
    cpp, py = tmp_path / "cpp.dat", tmp_path / "py.dat"
    proc = subprocess.run([str(exe), "--write-protein-ascii", str(rec), str(cpp), "0.0125"], capture_output=True,
                          text=True, timeout=120)
    assert proc.returncode == 0, proc.stderr
    io.write_protein_ascii(str(py), p, species, rod_gid, time=0.0125)
    assert cpp.read_bytes() == py.read_bytes()
    # the VTK snapshot pair, same bytes, and read back as the restart does
    vc, vp = tmp_path / "vtk_cpp", tmp_path / "vtk_py"
    vc.mkdir()
    vp.mkdir()
    proc = subprocess.run([str(exe), "--write-protein-vtk", str(rec), str(vc), "9"], capture_output=True,
                          text=True, timeout=120)
    assert proc.returncode == 0, proc.stderr
    io.write_protein_pvtp(str(vp), 9, p, species, rod_gid)
    for name in ("Protein_9.pvtp", "Protein_r0_9.vtp"):
        assert (vc / name).read_bytes() == (vp / name).read_bytes(), name
    rv = io.read_protein_pvtp(str(vp / "Protein_9.pvtp"))
    pts, ids = io.protein_points(p, rod_gid)
    assert np.array_equal(rv["gid"], p["gid"]) and np.array_equal(rv["idBind"], ids)
    assert np.array_equal(rv["end0"], pts[0::2]) and np.array_equal(rv["end1"], pts[1::2])
    # and it reads back
    back = io.read_protein_ascii(str(py))
    assert np.array_equal(back["gid"], p["gid"])
    assert np.array_equal(back["tag"], [species[t].tag for t in p["type"]])
