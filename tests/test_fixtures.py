"""CPU tests of the committed fixtures (derived from the reference's
Examples/DenseMonoLayer data by tests/golden/make_fixtures.py), the aLENS
text formats and the oracle's regression pin on them."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)

import make_fixtures  # noqa: E402

from alens_gb300 import io, workloads  # noqa: E402


def test_fixture_files_parse():
    cfg, rods = make_fixtures.load_fixture()
    assert rods.n == 1277
    assert cfg.monolayer == 1 and cfg.dt == 1e-5 and cfg.conMaxIte == 3000
    assert np.allclose(rods.pos[:, 2], 5.5)
    assert np.all(rods.radius == 0.0125)
    assert np.allclose(rods.length, 0.25, atol=1e-6)


def test_sylinder_ascii_round_trip(tmp_path):
    _, rods = make_fixtures.load_fixture()
    p = tmp_path / "out.dat"
    io.write_sylinder_ascii(str(p), rods, time=0.5)
    back, links = io.read_sylinder_ascii(str(p))
    assert links == []
    assert np.array_equal(back.gid, rods.gid)
    assert np.allclose(back.pos, rods.pos, atol=1e-14)
    assert np.allclose(back.length, rods.length, atol=1e-14)
    assert np.allclose(back.quat, rods.quat, atol=1e-12)


def test_links_and_stationary_lines(tmp_path):
    p = tmp_path / "in.dat"
    p.write_text("3\n0\nS 0 0.0125 0 0.5 0.5 20 0.5 0.5\nC 1 0.0125 0 0.5 0.57 20 0.5 0.57 3\nL 0 1\n")
    rods, links = io.read_sylinder_ascii(str(p))
    assert rods.n == 2 and links == [(0, 1)]
    assert list(rods.immovable) == [1, 0]
    assert np.allclose(rods.length, 20.0)
    assert np.allclose(rods.pos[1], [10.0, 0.5, 0.57])
    # links survive a write and a read
    q = tmp_path / "out.dat"
    io.write_sylinder_ascii(str(q), rods, links=links)
    back, back_links = io.read_sylinder_ascii(str(q))
    assert back_links == [(0, 1)] and list(back.immovable) == [1, 0]


def test_oracle_reproduces_golden():
    """Regression pin of the oracle on the monolayer window."""
    with open(os.path.join(GOLDEN, "monolayer_window_golden.json")) as f:
        gold = json.load(f)
    g = make_fixtures.golden(steps=gold["steps"])
    assert g["iterations"] == gold["iterations"]
    assert g["collisions"] == gold["collisions"]
    assert g["rod0"] == gold["rod0"]
    assert g["pos_head"] == gold["pos_head"] and g["quat_head"] == gold["quat_head"]
    assert g["stress_trace"] == gold["stress_trace"]


def test_vtp_and_restart_info(tmp_path):
    import xml.etree.ElementTree as ET
    _, rods = make_fixtures.load_fixture()
    p = tmp_path / "snap.vtp"
    io.write_vtp(str(p), rods, gamma_sum=np.arange(rods.n, dtype=float))
    root = ET.parse(str(p)).getroot()
    piece = root.find("PolyData/Piece")
    assert int(piece.get("NumberOfPoints")) == 2 * rods.n and int(piece.get("NumberOfLines")) == rods.n
    pts = np.array(piece.find("Points/DataArray").text.split(), float).reshape(-1, 3)
    mid = 0.5 * (pts[0::2] + pts[1::2])
    assert np.allclose(mid, rods.pos, atol=1e-12)
    assert np.allclose(np.linalg.norm(pts[1::2] - pts[0::2], axis=1), rods.length, atol=1e-12)
    names = [d.get("Name") for d in piece.find("CellData")]
    assert names == ["gid", "length", "radius", "force"]
    io.write_time_step_info(str(tmp_path / "TimeStepInfo.txt"), 1200, 12, 0.12)
    assert io.read_time_step_info(str(tmp_path / "TimeStepInfo.txt")) == (1200, 12, 0.12)


def test_sylinder_pvtp_snapshot(tmp_path):
    """aLENS snapshot layout: result/result0-399/ holds SylinderAscii_<id>.dat
    and Sylinder_<id>.pvtp indexing Sylinder_r0_<id>.vtp; the binary arrays
    decode to the rods' end points, gids and geometry."""
    import re
    import xml.etree.ElementTree as ET
    _, rods = make_fixtures.load_fixture()
    info = tmp_path / "TimeStepInfo.txt"
    folder = io.write_snapshot(12, rods, step=1200, time=0.012, root=str(tmp_path / "result"),
                               links=[(0, 1)], info_path=str(info))
    assert folder == str(tmp_path / "result") + "/result0-399/"
    assert io.result_folder(400) == "./result/result400-799/"
    assert io.read_time_step_info(info) == (1200, 12, 0.012)
    back, links = io.read_sylinder_ascii(folder + "SylinderAscii_12.dat")
    assert links == [(0, 1)] and back.n == rods.n
    index = ET.parse(folder + "Sylinder_12.pvtp").getroot()
    assert index.get("type") == "PPolyData"
    pieces = [p.get("Source") for p in index.iter("Piece")]
    assert pieces == ["Sylinder_r0_12.vtp"]
    # the frame number the aLENS .pvd collector takes from the index name
    assert int(re.search(r"_([^_.]+)(?:\.[^_]*)?$", "Sylinder_12.pvtp").group(1)) == 12
    declared = [(a.get("Name"), a.get("type")) for a in index.iter("PDataArray")]
    root = ET.parse(folder + pieces[0]).getroot()
    piece = root.find("PolyData/Piece")
    assert int(piece.get("NumberOfPoints")) == 2 * rods.n and int(piece.get("NumberOfLines")) == rods.n
    arrays = {a.get("Name"): a for a in root.iter("DataArray")}
    assert [(n, arrays[n].get("type")) for n, _ in declared] == declared
    types = {"Float64": "<f8", "Int64": "<i8", "Int32": "<i4"}

    def values(name):
        a = arrays[name]
        return io.read_vtk_binary_array(a.text, types[a.get("type")])

    pts = values("position").reshape(-1, 2, 3)
    axis = workloads.quat_to_axis(rods.quat)
    h = 0.5 * rods.length[:, None]
    assert np.array_equal(pts[:, 0], rods.pos - h * axis) and np.array_equal(pts[:, 1], rods.pos + h * axis)
    assert np.array_equal(values("connectivity"), np.arange(2 * rods.n))
    assert np.array_equal(values("offsets"), 2 * np.arange(1, rods.n + 1))
    assert np.array_equal(values("gid"), rods.gid)
    assert np.array_equal(values("length"), rods.length) and np.array_equal(values("radius"), rods.radius)
    assert np.array_equal(values("direction").reshape(-1, 3), axis)
    assert np.all(values("group") == -1)
