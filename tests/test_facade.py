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
