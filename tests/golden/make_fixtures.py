"""Generate the committed test fixtures from the reference's example data.

Reads Examples/DenseMonoLayer/TubuleInitial.dat of the aLENS checkout
(a relaxed monolayer of 9,700 rods, length 0.25 um, at z = 5.5 um) and keeps
the rods whose centres lie in a 4 x 4 um window, written in the same
TubuleInitial.dat line format.  The run configuration uses the example's
physical settings (Examples/DenseMonoLayer/RunConfig.yaml) on a closed
(non-periodic) 4 x 4 window.  Golden outputs: five oracle steps with one
bilateral spring between the first two rods (the facade driver's protocol).

usage: python tests/golden/make_fixtures.py /path/to/aLENS
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

WINDOW = 4.0


def write_fixture(ref):
    src = os.path.join(ref, "Examples", "DenseMonoLayer", "TubuleInitial.dat")
    lines = open(src).read().splitlines()
    keep = []
    for ln in lines[2:]:
        f = ln.split()
        if len(f) < 9 or f[0] not in ("C", "S"):
            continue
        m = np.array(f[3:6], float)
        p = np.array(f[6:9], float)
        c = 0.5 * (m + p)
        if 0.0 <= c[0] < WINDOW and 0.0 <= c[1] < WINDOW:
            keep.append(ln)
    with open(os.path.join(HERE, "monolayer_window.dat"), "w") as out:
        out.write(f"{len(keep)}\n0\n")
        out.write("\n".join(keep) + "\n")
    cfg = f"""# physical settings of Examples/DenseMonoLayer/RunConfig.yaml on a closed window
rngSeed: 1234
simBoxLow: [0.0, 0.0, 0.0]
simBoxHigh: [{WINDOW}, {WINDOW}, 11.0]
simBoxPBC: [false, false, false]
monolayer: true
viscosity: 1.0
KBT: 0.00411
linkKappa: 1000.0
sylinderDiameter: 0.025
sylinderColBuf: 0.025
sylinderDiameterColRatio: 1.0
sylinderLengthColRatio: 1.0
dt: 0.00001
timeTotal: 0.0001
conResTol: 1e-6
conMaxIte: 3000
conSolverChoice: 0
"""
    with open(os.path.join(HERE, "monolayer_window.yaml"), "w") as out:
        out.write(cfg)
    return len(keep)


def spring_block(pos, gid, kappa, rest=0.05):
    """The facade driver's bilateral block between rods 0 and 1."""
    from alens_gb300 import capi
    d = pos[0] - pos[1]
    L = float(np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]))
    b = capi.AlensBlock()
    b.delta0 = L - rest
    b.gamma = -(L - rest) * kappa
    b.gidI, b.gidJ = int(gid[0]), int(gid[1])
    b.globalIndexI, b.globalIndexJ = 0, 1
    for k in range(3):
        b.normI[k] = d[k] / L
        b.normJ[k] = -(d[k] / L)
        b.labI[k] = pos[0][k]
        b.labJ[k] = pos[1][k]
    b.bilateral = 1
    b.kappa = kappa
    return b


def load_fixture():
    from alens_gb300 import capi, io
    rods, _ = io.read_sylinder_ascii(os.path.join(HERE, "monolayer_window.dat"))
    cfg = io.read_run_config(os.path.join(HERE, "monolayer_window.yaml"))
    return cfg, rods


def golden(steps=5):
    from alens_gb300 import oracle_api as O
    cfg, rods = load_fixture()
    o = O.OracleSystem(cfg)
    o.set_rods(rods)
    its, coll = [], []
    for _ in range(steps):
        pos, _ = o.get_rods()
        o.add_bilateral([spring_block(pos, rods.gid, 1000.0)])
        st = o.step()
        its.append(st["iterations"])
        coll.append(st["nCollision"])
    pos, quat = o.get_rods()
    s9 = o.con_stress()
    return {"rods": int(rods.n), "steps": steps, "iterations": its, "collisions": coll,
            "sum_pos": pos.sum(axis=0).tolist(), "rod0": pos[0].tolist(),
            "stress_trace": float(s9[0, 0] + s9[1, 1] + s9[2, 2]),
            "pos_head": pos[:8].tolist(), "quat_head": quat[:8].tolist()}


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_fixtures.py /path/to/aLENS")
    ref = sys.argv[1]
    n = write_fixture(ref)
    g = golden()
    with open(os.path.join(HERE, "monolayer_window_golden.json"), "w") as f:
        json.dump(g, f, indent=1)
    print(n, "rods;", g["iterations"], g["collisions"])
