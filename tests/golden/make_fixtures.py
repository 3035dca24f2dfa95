"""Generate the committed test fixtures from the reference's example data.

Reads Examples/DenseMonoLayer/TubuleInitial.dat of the aLENS checkout
(a relaxed monolayer of 9,700 rods, length 0.25 um, at z = 5.5 um) and keeps
the rods whose centres lie in a 4 x 4 um window, written in the same
TubuleInitial.dat line format.  The run configuration uses the example's
physical settings (Examples/DenseMonoLayer/RunConfig.yaml) on a closed
(non-periodic) 4 x 4 window.  Golden outputs: five oracle steps with one
bilateral spring between the first two rods (the facade driver's protocol).

Second fixture, proteins: Examples/MixMotorSliding (two parallel 20 um
rods 0.07 um apart, the first immovable, 100 doubly bound motors of two
species): its rods (TubuleInitial.dat lines), its proteins (the 'P' lines of
ProteinInitial.dat), the species of its ProteinConfig.yaml re-emitted as flat
keys, and the run settings of its RunConfig.yaml.  Golden outputs: the
oracle's stage counts over five motion + binding + rod steps (a regression
pin of the oracle; the reference ships no outputs for this path).

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


MIX_KEYS = ("rngSeed", "dt", "timeSnap", "simBoxHigh", "simBoxLow", "simBoxPBC", "monolayer", "viscosity", "KBT",
            "conMaxIte", "conResTol", "conSolverChoice", "sylinderColBuf", "sylinderDiameterColRatio",
            "sylinderLengthColRatio", "sylinderDiameter")
SPECIES_KEYS = ("tag", "fixedEnd0", "useBindVol", "lookupType", "freeLength", "kappa", "lambda", "PtoAPratio",
                "diffUnbound", "rc", "eps", "ko_s", "ko_d", "Ka", "Ke", "walkOff", "fstall", "vmax", "vmaxAP",
                "vdrag", "diffBoundS", "diffBoundD")


def write_mixmotor_fixture(ref):
    from alens_gb300 import io
    src = os.path.join(ref, "Examples", "MixMotorSliding")
    with open(os.path.join(src, "TubuleInitial.dat")) as f:
        rods = [ln for ln in f.read().splitlines() if ln[:1] in ("C", "S")]
    with open(os.path.join(HERE, "mixmotor_tubules.dat"), "w") as out:
        out.write(f"{len(rods)}\n0\n" + "\n".join(rods) + "\n")
    with open(os.path.join(src, "ProteinInitial.dat")) as f:
        lines = f.read().splitlines()
    prots = [ln for ln in lines[2:] if ln[:1] == "P"]
    with open(os.path.join(HERE, "mixmotor_proteins.dat"), "w") as out:
        out.write(f"{len(prots)} \n 0.000000\n" + "\n".join(prots) + "\n")
    keep = []
    with open(os.path.join(src, "RunConfig.yaml")) as f:
        for ln in f:
            k = ln.split("#", 1)[0].split(":", 1)[0].strip()
            if k in MIX_KEYS and ln[:1] not in " \t-":
                keep.append(ln.split("#", 1)[0].rstrip())
    with open(os.path.join(HERE, "mixmotor_run.yaml"), "w") as out:
        out.write("# run settings of Examples/MixMotorSliding/RunConfig.yaml\n" + "\n".join(keep) + "\n")
    kbt, _, entries = io.read_protein_config(os.path.join(src, "ProteinConfig.yaml"))
    text = ["# species of Examples/MixMotorSliding/ProteinConfig.yaml", f"KBT: {kbt!r}", "proteins:"]
    for e in entries:
        first = True
        for k in SPECIES_KEYS:
            if k not in e:
                continue
            v = e[k]
            v = "[" + ", ".join(repr(float(x)) for x in v) + "]" if isinstance(v, list) else repr(v)
            text.append(("  - " if first else "    ") + f"{k}: {v}")
            first = False
    with open(os.path.join(HERE, "mixmotor_species.yaml"), "w") as out:
        out.write("\n".join(text) + "\n")
    return len(rods), len(prots)


def load_mixmotor():
    from alens_gb300 import io
    cfg = io.read_run_config(os.path.join(HERE, "mixmotor_run.yaml"))
    rods, _ = io.read_sylinder_ascii(os.path.join(HERE, "mixmotor_tubules.dat"))
    kbt, species, _ = io.read_protein_config(os.path.join(HERE, "mixmotor_species.yaml"))
    rec = io.read_protein_ascii(os.path.join(HERE, "mixmotor_proteins.dat"))
    prots = io.proteins_from_ascii(rec, rods, species, cfg)
    return cfg, rods, kbt, species, prots


def mixmotor_golden(steps=5):
    from alens_gb300 import oracle_api as O
    cfg, rods, kbt, species, prots = load_mixmotor()
    o = O.OracleSystem(cfg)
    o.set_rods(rods)
    o.set_protein_types(species, kbt, float(cfg_diameter(cfg)))
    o.set_proteins(prots)
    counts = []
    for _ in range(steps):
        o.protein_motion_step()
        st = o.protein_bind_step()
        r = o.step()
        counts.append([st[k] for k in ("nU", "nS", "nD", "nUS", "nSU", "nSD", "nDS")] + [r["nBilateral"]])
    q = o.get_proteins()
    o.close()
    return {"steps": steps, "counts": counts, "idBind": q["idBind"].tolist(),
            "distBind_sum": float(np.nansum(q["distBind"]))}


def cfg_diameter(cfg):
    """sylinderDiameter of the MixMotorSliding run (RunConfig key)."""
    with open(os.path.join(HERE, "mixmotor_run.yaml")) as f:
        for ln in f:
            if ln.split(":", 1)[0].strip() == "sylinderDiameter":
                return float(ln.split(":", 1)[1].split("#", 1)[0])
    return 0.025


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_fixtures.py /path/to/aLENS")
    ref = sys.argv[1]
    n = write_fixture(ref)
    g = golden()
    with open(os.path.join(HERE, "monolayer_window_golden.json"), "w") as f:
        json.dump(g, f, indent=1)
    print(n, "rods;", g["iterations"], g["collisions"])
    nr, npr = write_mixmotor_fixture(ref)
    gm = mixmotor_golden()
    with open(os.path.join(HERE, "mixmotor_golden.json"), "w") as f:
        json.dump(gm, f, indent=1)
    print(nr, "rods,", npr, "proteins;", gm["counts"])
