"""aLENS text formats: TubuleInitial.dat / SylinderAscii rod lines
("C|S gid radius mx my mz px py pz [group]", docs/source/quickstart.md:211-218;
'L a b' link lines as in Utils/gen_flexible_init.py) and the flat keys of
RunConfig.yaml (docs/source/quickstart.md:316-358)."""
from __future__ import annotations

import math

import numpy as np

from .capi import AlensConfig, RodState, make_config
from .workloads import quat_to_axis


def _quat_from_direction(d0, d1, d2):
    """Rotation of +z onto (d0, d1, d2) as (x, y, z, w), with the operation
    order of the C++ facade's reader (gpu::readSylinderAscii), so both
    readers produce bit-identical rods."""
    x, y, z, w = -d1, d0, 0.0, 1.0 + d2
    if w < 1e-8:
        x, y, z, w = 1.0, 0.0, 0.0, 0.0
    n = math.sqrt(x * x + y * y + z * z + w * w)
    return [x / n, y / n, z / n, w / n]


def read_sylinder_ascii(path):
    """Rods and links of a TubuleInitial.dat / SylinderAscii file."""
    gid, pos, quat, length, radius, imm, group, links = [], [], [], [], [], [], [], []
    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "L" and len(t) >= 3:
                links.append((int(t[1]), int(t[2])))
                continue
            if t[0] not in ("C", "S") or len(t) < 9:
                continue
            m = [float(v) for v in t[3:6]]
            p = [float(v) for v in t[6:9]]
            d = [p[k] - m[k] for k in range(3)]
            L = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
            if L > 0:
                d = [d[k] / L for k in range(3)]
            else:
                d = [0.0, 0.0, 1.0]
            gid.append(int(t[1]))
            radius.append(float(t[2]))
            pos.append([0.5 * (m[k] + p[k]) for k in range(3)])
            quat.append(_quat_from_direction(*d))
            length.append(L)
            imm.append(1 if t[0] == "S" else 0)
            group.append(int(t[9]) if len(t) > 9 else -1)
    n = len(gid)
    rods = RodState(np.array(gid, np.int64), np.array(pos).reshape(n, 3), np.array(quat).reshape(n, 4),
                    np.array(length), np.array(radius), np.array(imm, np.int32))
    return rods, links


def write_sylinder_ascii(path, rods: RodState, time: float = 0.0, group=None, links=()):
    """Rods as 'C|S gid radius minus-end plus-end group' lines, then the
    links as 'L a b' lines (gids), readable by read_sylinder_ascii."""
    a = quat_to_axis(rods.quat)
    h = 0.5 * rods.length[:, None]
    m = rods.pos - h * a
    p = rods.pos + h * a
    imm = rods.immovable if rods.immovable is not None else np.zeros(rods.n, np.int32)
    with open(path, "w") as f:
        f.write(f"{rods.n}\n{time:.17g}\n")
        for i in range(rods.n):
            g = -1 if group is None else int(group[i])
            f.write("%s %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %d\n" % (
                "S" if imm[i] else "C", rods.gid[i], rods.radius[i], *m[i], *p[i], g))
        for la, lb in links:
            f.write("L %d %d\n" % (int(la), int(lb)))


def read_run_config(path, **overrides) -> AlensConfig:
    vals = {}
    with open(path) as f:
        for line in f:
            line = line.split("#", 1)[0]
            if not line.strip() or line[0] in " \t-" or ":" not in line:
                continue
            k, v = line.split(":", 1)
            vals[k.strip()] = v.strip()

    def vec(v, conv=float):
        return [conv(x.strip()) for x in v.strip("[] ").split(",")]

    def b(x):
        return str(x).strip().lower() in ("true", "1", "yes")

    cfg = make_config(
        box_low=vec(vals.get("simBoxLow", "[0,0,0]")), box_high=vec(vals.get("simBoxHigh", "[1,1,1]")),
        pbc=[b(x) for x in vals.get("simBoxPBC", "[false,false,false]").strip("[] ").split(",")],
        monolayer=b(vals.get("monolayer", "false")), viscosity=float(vals.get("viscosity", 0.01)),
        kbt=float(vals.get("KBT", 0.00411)), dt=float(vals.get("dt", 1e-4)),
        col_ratio_d=float(vals.get("sylinderDiameterColRatio", 1.0)),
        col_ratio_l=float(vals.get("sylinderLengthColRatio", 1.0)),
        col_buf=float(vals.get("sylinderColBuf", 0.025)), tol=float(vals.get("conResTol", 1e-5)),
        max_ite=int(float(vals.get("conMaxIte", 2000))), seed=int(vals.get("rngSeed", 1234)), **overrides)
    return cfg


def read_link_params(path):
    """linkKappa and linkGap of a RunConfig.yaml (defaults 1000 pN/um, 0)."""
    kappa, gap = 1000.0, 0.0
    with open(path) as f:
        for line in f:
            line = line.split("#", 1)[0]
            if ":" not in line:
                continue
            k, v = (x.strip() for x in line.split(":", 1))
            if k == "linkKappa":
                kappa = float(v)
            elif k == "linkGap":
                gap = float(v)
    return kappa, gap


def filament_links(rods: RodState, pairs, kappa: float, gap: float) -> dict:
    """Spring links of 'L a b' lines (rod gids) for GpuSystem.set_links: plus
    end of a (centre + L/2 axis) to minus end of b, rest length gap plus both
    radii, stiffness kappa (the C++ facade builds the same set)."""
    index = {int(g): i for i, g in enumerate(rods.gid)}
    I = np.array([index[a] for a, _ in pairs], np.int32)
    J = np.array([index[b] for _, b in pairs], np.int32)
    return {"i": I, "j": J, "si": 0.5 * rods.length[I], "sj": -0.5 * rods.length[J],
            "rest": gap + rods.radius[I] + rods.radius[J], "kappa": np.full(len(pairs), float(kappa))}


def read_boundaries(path):
    """The `boundaries:` list of a RunConfig.yaml as AlensBoundary structs
    (type "wall" | "sphere" | "tube"; center, radius, axis or norm, inside),
    parsed as the C++ facade parses it."""
    from .capi import BOUNDARY_SPHERE, BOUNDARY_TUBE, BOUNDARY_WALL, make_boundary
    out, cur, inside = [], None, False
    with open(path) as f:
        for raw in f:
            line = raw.split("#", 1)[0]
            if not line.strip():
                continue
            nested = line[0] in " \t-"
            if inside and nested:
                t = line.strip()
                if t.startswith("-"):
                    cur = {"type": "wall", "center": (0, 0, 0), "axis": (0, 0, 1), "radius": 0.0, "inside": True}
                    out.append(cur)
                    t = t[1:].strip()
                if ":" not in t or cur is None:
                    continue
                k, v = (x.strip() for x in t.split(":", 1))
                if k == "type":
                    cur["type"] = v.strip("\"'")
                elif k in ("center", "axis", "norm"):
                    cur["axis" if k == "norm" else k] = [float(x) for x in v.strip("[] ").split(",")]
                elif k == "radius":
                    cur["radius"] = float(v)
                elif k == "inside":
                    cur["inside"] = v.lower() in ("true", "1", "yes")
                continue
            if nested:
                continue
            inside = line.split(":", 1)[0].strip() == "boundaries"
    kinds = {"wall": BOUNDARY_WALL, "sphere": BOUNDARY_SPHERE, "tube": BOUNDARY_TUBE}
    return [make_boundary(kinds.get(b["type"], BOUNDARY_WALL), b["center"], b["axis"], b["radius"], b["inside"])
            for b in out]


def write_vtp(path, rods: RodState, gamma_sum=None):
    """Rods as a VTK XML PolyData file (.vtp, ASCII): two points per rod (its
    segment ends) joined by one line cell, with per-rod cell data gid,
    length, radius and, when given, the summed constraint force magnitude.
    The role of the snapshot writer the reference's ParaView states read
    (Examples/*/ *.pvsm load SylinderAscii / VTK output)."""
    a = quat_to_axis(rods.quat)
    h = 0.5 * rods.length[:, None]
    pts = np.empty((2 * rods.n, 3))
    pts[0::2] = rods.pos - h * a
    pts[1::2] = rods.pos + h * a

    def arr(name, typ, vals, ncomp=1):
        body = " ".join(repr(float(v)) if typ.startswith("Float") else str(int(v)) for v in np.ravel(vals))
        return (f'<DataArray type="{typ}" Name="{name}" NumberOfComponents="{ncomp}" format="ascii">'
                f"{body}</DataArray>\n")

    with open(path, "w") as f:
        f.write('<?xml version="1.0"?>\n<VTKFile type="PolyData" version="0.1" byte_order="LittleEndian">\n')
        f.write(f'<PolyData>\n<Piece NumberOfPoints="{2 * rods.n}" NumberOfVerts="0" NumberOfLines="{rods.n}" '
                'NumberOfStrips="0" NumberOfPolys="0">\n')
        f.write("<Points>\n" + arr("Points", "Float64", pts, 3) + "</Points>\n")
        f.write("<Lines>\n" + arr("connectivity", "Int64", np.arange(2 * rods.n))
                + arr("offsets", "Int64", 2 * np.arange(1, rods.n + 1)) + "</Lines>\n")
        f.write("<CellData>\n" + arr("gid", "Int64", rods.gid) + arr("length", "Float64", rods.length)
                + arr("radius", "Float64", rods.radius))
        if gamma_sum is not None:
            f.write(arr("force", "Float64", gamma_sum))
        f.write("</CellData>\n</Piece>\n</PolyData>\n</VTKFile>\n")


# --------------------------------------------------------------- snapshots
# aLENS result layout (docs/source/visualization.md:13,32; README.md:135-148):
# snapshots grouped 400 to a folder (result/result0-399/, result400-799/, ...),
# each snapshot a SylinderAscii_<id>.dat text file and a parallel VTK index
# Sylinder_<id>.pvtp naming one serial piece per rank, Sylinder_r<rank>_<id>.vtp
# (here one rank).  Data arrays are inline binary: base64 of a UInt64 byte
# count followed by the little-endian values.  The C++ facade writes the same
# bytes (gpu::SylinderSystem::writeSylinderVTK).

SNAPSHOTS_PER_FOLDER = 400

# cell data of a rod piece: (name, VTK type, numpy dtype, components)
_ROD_CELL_FIELDS = [("gid", "Int64", "<i8", 1), ("radius", "Float64", "<f8", 1), ("length", "Float64", "<f8", 1),
                    ("group", "Int32", "<i4", 1), ("isImmovable", "Int32", "<i4", 1),
                    ("direction", "Float64", "<f8", 3)]


def result_folder(snap_id: int, root: str = "./result") -> str:
    lo = snap_id // SNAPSHOTS_PER_FOLDER * SNAPSHOTS_PER_FOLDER
    return f"{root}/result{lo}-{lo + SNAPSHOTS_PER_FOLDER - 1}/"


def _b64_array(name, vtk_type, values, ncomp):
    import base64
    import struct
    raw = np.ascontiguousarray(values).tobytes()
    body = base64.b64encode(struct.pack("<Q", len(raw)) + raw).decode("ascii")
    return (f'<DataArray type="{vtk_type}" Name="{name}" NumberOfComponents="{ncomp}" format="binary">'
            f"{body}</DataArray>\n")


def write_sylinder_pvtp(folder, snap_id: int, rods: RodState, group=None):
    """Sylinder_<id>.pvtp and its piece Sylinder_r0_<id>.vtp in `folder`: two
    points per rod (minus end, plus end) joined by a line cell; cell data gid,
    radius, length, group, isImmovable and the unit direction."""
    import os
    n = rods.n
    a = quat_to_axis(rods.quat)
    h = 0.5 * rods.length[:, None]
    pts = np.empty((2 * n, 3))
    pts[0::2] = rods.pos - h * a
    pts[1::2] = rods.pos + h * a
    imm = rods.immovable if rods.immovable is not None else np.zeros(n, np.int32)
    grp = np.full(n, -1, np.int32) if group is None else np.asarray(group)
    cells = {"gid": rods.gid, "radius": rods.radius, "length": rods.length, "group": grp, "isImmovable": imm,
             "direction": a}
    piece = f"Sylinder_r0_{snap_id}.vtp"
    head = '<?xml version="1.0"?>\n'
    with open(os.path.join(folder, piece), "w") as f:
        f.write(head + '<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n')
        f.write(f'<PolyData>\n<Piece NumberOfPoints="{2 * n}" NumberOfVerts="0" NumberOfLines="{n}" '
                'NumberOfStrips="0" NumberOfPolys="0">\n')
        f.write("<Points>\n" + _b64_array("position", "Float64", pts.astype("<f8"), 3) + "</Points>\n")
        f.write("<Lines>\n" + _b64_array("connectivity", "Int32", np.arange(2 * n, dtype="<i4"), 1)
                + _b64_array("offsets", "Int32", 2 * np.arange(1, n + 1, dtype="<i4"), 1) + "</Lines>\n")
        f.write('<CellData Scalars="scalars">\n')
        for name, vt, dt, nc in _ROD_CELL_FIELDS:
            f.write(_b64_array(name, vt, np.asarray(cells[name]).astype(dt), nc))
        f.write("</CellData>\n</Piece>\n</PolyData>\n</VTKFile>\n")
    with open(os.path.join(folder, f"Sylinder_{snap_id}.pvtp"), "w") as f:
        f.write(head + '<VTKFile type="PPolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n')
        f.write('<PPolyData GhostLevel="0">\n<PPoints>\n'
                '<PDataArray type="Float64" Name="position" NumberOfComponents="3"/>\n</PPoints>\n')
        f.write('<PCellData Scalars="scalars">\n')
        for name, vt, _, nc in _ROD_CELL_FIELDS:
            f.write(f'<PDataArray type="{vt}" Name="{name}" NumberOfComponents="{nc}"/>\n')
        f.write(f'</PCellData>\n<Piece Source="{piece}"/>\n</PPolyData>\n</VTKFile>\n')


# cell data of a constraint-block piece (ConBlock_<id>.pvtp): the fields of a
# ConstraintBlock (SRC/TubuleSystem.cpp:727-736) that describe the solved
# block, and its pair virial gamma (labI - labJ) (x) normI as "Stress"
_CON_CELL_FIELDS = [("gamma", "Float64", "<f8", 1), ("delta0", "Float64", "<f8", 1), ("kappa", "Float64", "<f8", 1),
                    ("bilateral", "Int32", "<i4", 1), ("oneSide", "Int32", "<i4", 1), ("gidI", "Int64", "<i8", 1),
                    ("gidJ", "Int64", "<i8", 1), ("globalIndexI", "Int32", "<i4", 1),
                    ("globalIndexJ", "Int32", "<i4", 1), ("image", "Int32", "<i4", 1),
                    ("normI", "Float64", "<f8", 3), ("Stress", "Float64", "<f8", 9)]


def conblock_cells(blocks: dict, gid) -> dict:
    """Cell arrays of a ConBlock piece from GpuSystem.constraint_blocks()
    and the rods' gids (gidJ = -1 for boundary contacts)."""
    gid = np.asarray(gid, dtype=np.int64)
    i = np.asarray(blocks["i"], dtype=np.int64)
    j = np.asarray(blocks["j"], dtype=np.int64)
    r = np.asarray(blocks["labI"]) - np.asarray(blocks["labJ"])
    n = np.asarray(blocks["normI"])
    g = np.asarray(blocks["gamma"])
    stress = (g[:, None, None] * r[:, :, None]) * n[:, None, :]
    return {"gamma": g, "delta0": blocks["delta0"], "kappa": blocks["kappa"], "bilateral": blocks["bilateral"],
            "oneSide": blocks["oneSide"], "gidI": gid[i] if i.size else i,
            "gidJ": np.where(j >= 0, gid[np.maximum(j, 0)] if j.size else j, -1),
            "globalIndexI": i, "globalIndexJ": j, "image": blocks["image"], "normI": n,
            "Stress": stress.reshape(-1, 9)}


def write_conblock_pvtp(folder, snap_id: int, blocks: dict, gid):
    """ConBlock_<id>.pvtp and its piece ConBlock_r0_<id>.vtp in `folder` (the
    constraint-block snapshot aLENS lists in README.md:142 and collects with
    Run/result/Result2PVD.py:26): one line cell per block from its contact
    point on rod I (labI) to the one on rod J or the boundary (labJ); cell
    data as _CON_CELL_FIELDS.  The C++ facade writes the same bytes
    (gpu::SylinderSystem::writeConBlockVTK)."""
    import os
    cells = conblock_cells(blocks, gid)
    n = int(np.asarray(blocks["gamma"]).shape[0])
    pts = np.empty((2 * n, 3))
    pts[0::2] = np.asarray(blocks["labI"]).reshape(-1, 3)
    pts[1::2] = np.asarray(blocks["labJ"]).reshape(-1, 3)
    piece = f"ConBlock_r0_{snap_id}.vtp"
    head = '<?xml version="1.0"?>\n'
    with open(os.path.join(folder, piece), "w") as f:
        f.write(head + '<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n')
        f.write(f'<PolyData>\n<Piece NumberOfPoints="{2 * n}" NumberOfVerts="0" NumberOfLines="{n}" '
                'NumberOfStrips="0" NumberOfPolys="0">\n')
        f.write("<Points>\n" + _b64_array("position", "Float64", pts.astype("<f8"), 3) + "</Points>\n")
        f.write("<Lines>\n" + _b64_array("connectivity", "Int32", np.arange(2 * n, dtype="<i4"), 1)
                + _b64_array("offsets", "Int32", 2 * np.arange(1, n + 1, dtype="<i4"), 1) + "</Lines>\n")
        f.write('<CellData Scalars="scalars">\n')
        for name, vt, dt, nc in _CON_CELL_FIELDS:
            f.write(_b64_array(name, vt, np.asarray(cells[name]).astype(dt), nc))
        f.write("</CellData>\n</Piece>\n</PolyData>\n</VTKFile>\n")
    with open(os.path.join(folder, f"ConBlock_{snap_id}.pvtp"), "w") as f:
        f.write(head + '<VTKFile type="PPolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n')
        f.write('<PPolyData GhostLevel="0">\n<PPoints>\n'
                '<PDataArray type="Float64" Name="position" NumberOfComponents="3"/>\n</PPoints>\n')
        f.write('<PCellData Scalars="scalars">\n')
        for name, vt, _, nc in _CON_CELL_FIELDS:
            f.write(f'<PDataArray type="{vt}" Name="{name}" NumberOfComponents="{nc}"/>\n')
        f.write(f'</PCellData>\n<Piece Source="{piece}"/>\n</PPolyData>\n</VTKFile>\n')


def protein_points(proteins, rod_gid):
    """The two points per protein of its snapshot lines (the heads when both
    are bound, the centre twice otherwise) and the bound rods as gids."""
    n = proteins.shape[0]
    both = (proteins["idBind"] >= 0).all(axis=1)
    pts = np.empty((2 * n, 3))
    pts[0::2] = np.where(both[:, None], proteins["posEnd"][:, 0], proteins["pos"])
    pts[1::2] = np.where(both[:, None], proteins["posEnd"][:, 1], proteins["pos"])
    rg = np.asarray(rod_gid, dtype=np.int64)
    ids = np.where(proteins["idBind"] >= 0, rg[np.maximum(proteins["idBind"], 0)] if rg.size else -1, -1)
    return pts, ids


def write_protein_pvtp(folder, snap_id: int, proteins, species, rod_gid):
    """Protein_<id>.pvtp and its piece Protein_r0_<id>.vtp in `folder`
    (ProteinData::writeVTP / writePVTP, Protein/ProteinData.hpp:583-700):
    two points per protein joined by a line cell, point data idBind (the
    bound rods' gids, -1 unbound), cell data gid and tag (Int32 as the
    reference writes them).  The C++ facade writes the same bytes."""
    import os
    n = proteins.shape[0]
    pts, ids = protein_points(proteins, rod_gid)
    tags = np.array([species[int(t)].tag for t in proteins["type"]], dtype="<i4")
    piece = f"Protein_r0_{snap_id}.vtp"
    head = '<?xml version="1.0"?>\n'
    with open(os.path.join(folder, piece), "w") as f:
        f.write(head + '<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n')
        f.write(f'<PolyData>\n<Piece NumberOfPoints="{2 * n}" NumberOfVerts="0" NumberOfLines="{n}" '
                'NumberOfStrips="0" NumberOfPolys="0">\n')
        f.write("<Points>\n" + _b64_array("position", "Float64", pts.astype("<f8"), 3) + "</Points>\n")
        f.write("<Lines>\n" + _b64_array("connectivity", "Int32", np.arange(2 * n, dtype="<i4"), 1)
                + _b64_array("offsets", "Int32", 2 * np.arange(1, n + 1, dtype="<i4"), 1) + "</Lines>\n")
        f.write('<PointData Scalars="scalars">\n' + _b64_array("idBind", "Int32", ids.reshape(-1).astype("<i4"), 1)
                + "</PointData>\n")
        f.write('<CellData Scalars="scalars">\n' + _b64_array("gid", "Int32", proteins["gid"].astype("<i4"), 1)
                + _b64_array("tag", "Int32", tags, 1) + "</CellData>\n</Piece>\n</PolyData>\n</VTKFile>\n")
    with open(os.path.join(folder, f"Protein_{snap_id}.pvtp"), "w") as f:
        f.write(head + '<VTKFile type="PPolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n')
        f.write('<PPolyData GhostLevel="0">\n<PPoints>\n'
                '<PDataArray type="Float64" Name="position" NumberOfComponents="3"/>\n</PPoints>\n')
        f.write('<PPointData Scalars="scalars">\n<PDataArray type="Int32" Name="idBind" NumberOfComponents="1"/>\n'
                '</PPointData>\n<PCellData Scalars="scalars">\n'
                '<PDataArray type="Int32" Name="gid" NumberOfComponents="1"/>\n'
                '<PDataArray type="Int32" Name="tag" NumberOfComponents="1"/>\n')
        f.write(f'</PCellData>\n<Piece Source="{piece}"/>\n</PPolyData>\n</VTKFile>\n')


def read_protein_pvtp(path):
    """The proteins of a Protein_<id>.pvtp snapshot (its pieces, in order),
    as read_protein_ascii returns them, for the restart of
    TubuleSystem::readProteinVTK (SRC/TubuleSystem.cpp:811-872): rebuild the
    bindings with proteins_from_ascii."""
    import os
    import re
    text = open(path).read()
    pieces = re.findall(r'<Piece Source="([^"]+)"', text)
    parts = []
    for pc in pieces:
        body = open(os.path.join(os.path.dirname(path), pc)).read()

        def arr(name, dtype):
            m = re.search(rf'Name="{name}" NumberOfComponents="\d+" format="binary">([^<]*)<', body)
            return read_vtk_binary_array(m.group(1), dtype)
        pts = arr("position", "<f8").reshape(-1, 3)
        ids = arr("idBind", "<i4").reshape(-1, 2)
        parts.append({"gid": arr("gid", "<i4").astype(np.int64), "tag": arr("tag", "<i4").astype(np.int32),
                      "end0": pts[0::2], "end1": pts[1::2], "idBind": ids.astype(np.int64)})
    return {k: np.concatenate([p[k] for p in parts]) for k in ("gid", "tag", "end0", "end1", "idBind")}


def write_snapshot(snap_id: int, rods: RodState, step: int, time: float, root: str = "./result", links=(),
                   group=None, info_path: str = "TimeStepInfo.txt", blocks: dict | None = None,
                   proteins=None, species=None) -> str:
    """One aLENS snapshot: SylinderAscii_<id>.dat, Sylinder_<id>.pvtp (+ piece),
    with `blocks` (GpuSystem.constraint_blocks() of the last step)
    ConBlock_<id>.pvtp (+ piece), with `proteins` and `species`
    ProteinAscii_<id>.dat and Protein_<id>.pvtp (+ piece), in
    result_folder(snap_id, root), then the restart bookkeeping file.
    Returns the folder."""
    import os
    folder = result_folder(snap_id, root)
    os.makedirs(folder, exist_ok=True)
    write_sylinder_ascii(os.path.join(folder, f"SylinderAscii_{snap_id}.dat"), rods, time=time, group=group,
                         links=links)
    write_sylinder_pvtp(folder, snap_id, rods, group=group)
    if blocks is not None:
        write_conblock_pvtp(folder, snap_id, blocks, rods.gid)
    if proteins is not None:
        write_protein_ascii(os.path.join(folder, f"ProteinAscii_{snap_id}.dat"), proteins, species, rods.gid,
                            time=time)
        write_protein_pvtp(folder, snap_id, proteins, species, rods.gid)
    write_time_step_info(info_path, step, snap_id, time)
    return folder


def read_vtk_binary_array(text: str, dtype):
    """Values of one inline binary DataArray body (UInt64 byte-count header)."""
    import base64
    import struct
    raw = base64.b64decode(text.strip())
    nbytes = struct.unpack("<Q", raw[:8])[0]
    return np.frombuffer(raw[8:8 + nbytes], dtype=dtype)


def write_time_step_info(path, step: int, snap_id: int, time: float):
    """Restart bookkeeping next to a snapshot (the role of TimeStepInfo.txt,
    whose presence makes aLENS restart, SRC/main.cpp:28-37)."""
    with open(path, "w") as f:
        f.write(f"{int(step)}\n{int(snap_id)}\n{time:.17g}\n")


def read_time_step_info(path):
    with open(path) as f:
        vals = f.read().split()
    return int(vals[0]), int(vals[1]), float(vals[2])


# ---------------------------------------------------------------- proteins
_PROTEIN_KEYS_SCALAR = ("tag", "fixedEnd0", "useBindVol", "lookupType", "freeLength", "kappa", "lambda",
                        "PtoAPratio", "diffUnbound", "rc", "eps", "freeNumber")
_PROTEIN_KEYS_PAIR = ("ko_s", "ko_d", "Ka", "Ke")


def read_protein_config(path):
    """ProteinConfig.yaml (Protein/ProteinConfig.cpp:6-45, keys of
    ProteinType::readFromYaml, Protein/ProteinType.hpp:81-129): KBT and the
    `proteins:` list, parsed as flat YAML.  Returns (KBT, species) with one
    AlensProteinType per list entry, in file order, and the entries' raw
    dicts (freeNumber, fixedLocationPerMT, ...) beside them."""
    from .capi import make_protein_type
    kbt, entries, cur, inside = 0.00411, [], None, False

    def val(v):
        v = v.strip().strip("\"'")
        if v.startswith("["):
            return [val(x) for x in v.strip("[] ").split(",") if x.strip()]
        low = v.lower()
        if low in ("true", "yes"):
            return 1
        if low in ("false", "no"):
            return 0
        try:
            return float(v)
        except ValueError:
            return v

    with open(path) as f:
        for raw in f:
            line = raw.split("#", 1)[0]
            if not line.strip():
                continue
            nested = line[0] in " \t-"
            if not nested:
                k, _, v = line.partition(":")
                inside = k.strip() == "proteins"
                if k.strip() == "KBT":
                    kbt = float(v)
                continue
            if not inside:
                continue
            t = line.strip()
            if t.startswith("-"):
                cur = {}
                entries.append(cur)
                t = t[1:].strip()
            if ":" not in t or cur is None:
                continue
            k, v = (x.strip() for x in t.split(":", 1))
            cur[k] = val(v) if v else []
    species = []
    for e in entries:
        pair = {k: tuple(float(x) for x in (e.get(k) or [0.0, 0.0])) for k in _PROTEIN_KEYS_PAIR}
        species.append(make_protein_type(
            tag=int(e.get("tag", 0)), freeLength=float(e.get("freeLength", 0.05)), rc=float(e.get("rc", 0.0)),
            kappa=float(e.get("kappa", 204.7)), lambda_=float(e.get("lambda", 0.0)),
            diffUnbound=float(e.get("diffUnbound", 4.5)), useBindVol=bool(e.get("useBindVol", 0)),
            eps=float(e.get("eps", 0.0)), PtoAPratio=float(e.get("PtoAPratio", 1.0)),
            fixedEnd0=bool(e.get("fixedEnd0", 0)), lookupType=int(e.get("lookupType", 0)),
            walkOff=bool(e.get("walkOff", 1)), fstall=float(e.get("fstall", 1.0)),
            vmax=tuple(float(x) for x in (e.get("vmax") or [0.0, 0.0])),
            vmaxAP=tuple(float(x) for x in (e.get("vmaxAP") or e.get("vmax") or [0.0, 0.0])),
            vdrag=tuple(bool(x) for x in (e.get("vdrag") or [0, 0])),
            diffBoundS=tuple(float(x) for x in (e.get("diffBoundS") or [0.0, 0.0])),
            diffBoundD=tuple(float(x) for x in (e.get("diffBoundD") or [0.0, 0.0])), **pair))
    return kbt, species, entries


def read_protein_ascii(path):
    """ProteinAscii_<id>.dat / ProteinInitial.dat: two header lines (count,
    time), then 'P gid tag x0 y0 z0 x1 y1 z1 idBind0 idBind1' lines
    (Protein/ProteinData.hpp:545-564; read as
    TubuleSystem::setInitialProteinFromFile, SRC/TubuleSystem.cpp:761-789).
    idBind are rod gids (-1 unbound)."""
    gid, tag, end0, end1, ids = [], [], [], [], []
    with open(path) as f:
        lines = f.read().splitlines()
    for ln in lines[2:]:
        p = ln.split()
        if len(p) < 11 or p[0] != "P":
            continue
        gid.append(int(p[1]))
        tag.append(int(p[2]))
        end0.append([float(x) for x in p[3:6]])
        end1.append([float(x) for x in p[6:9]])
        ids.append([int(p[9]), int(p[10])])
    return {"gid": np.array(gid, np.int64), "tag": np.array(tag, np.int32),
            "end0": np.array(end0, float).reshape(-1, 3), "end1": np.array(end1, float).reshape(-1, 3),
            "idBind": np.array(ids, np.int64).reshape(-1, 2)}


def proteins_from_ascii(rec, rods: RodState, species, cfg: AlensConfig):
    """AlensProtein records from read_protein_ascii's output: the binding of
    each end rebuilt from its position as TubuleSystem::updateBindWithGid
    does with reconstruct = true (SRC/TubuleSystem.cpp:482-563): the bound
    rod's periodic image nearest the protein, distBind = (end - centre) .
    direction; kept inside L/2, clamped within 1.01 L/2 (or on a sphere),
    the end released otherwise.  Tags select the species (list order)."""
    from .capi import protein_array
    n = rec["gid"].shape[0]
    out = protein_array(n)
    index = {int(g): i for i, g in enumerate(rods.gid)}
    tag_index = {int(t.tag): k for k, t in enumerate(species)}
    axis = quat_to_axis(rods.quat)
    lo = np.array([cfg.simBoxLow[d] for d in range(3)])
    L = np.array([cfg.simBoxHigh[d] - cfg.simBoxLow[d] for d in range(3)])
    pbc = [bool(cfg.simBoxPBC[d]) for d in range(3)]
    for p in range(n):
        t = int(rec["tag"][p])
        if t not in tag_index:
            raise ValueError(f"protein {int(rec['gid'][p])}: tag {t} not in the species list")
        out["gid"][p] = rec["gid"][p]
        out["type"][p] = tag_index[t]
        ends = (rec["end0"][p], rec["end1"][p])
        pos = 0.5 * (ends[0] + ends[1])
        out["pos"][p] = pos
        for e in range(2):
            g = int(rec["idBind"][p, e])
            if g == -1:
                continue
            if g not in index:
                raise ValueError(f"protein {int(rec['gid'][p])}: rod gid {g} not found")
            r = index[g]
            c = rods.pos[r].copy()
            for d in range(3):
                if pbc[d]:
                    c[d] += L[d] * np.round((pos[d] - c[d]) / L[d])
            dist = float(np.dot(ends[e] - c, axis[r]))
            half = 0.5 * float(rods.length[r])
            sphere = rods.length[r] < 2.0 * rods.radius[r]
            if -half < dist < half:
                pass
            elif -1.01 * half < dist < 1.01 * half or sphere:
                dist = min(max(dist, -half), half)
            else:
                continue
            out["idBind"][p, e] = r
            out["distBind"][p, e] = dist
    return out


def write_protein_ascii(path, proteins, species, rod_gid, time: float = 0.0):
    """ProteinAscii_<id>.dat: the header of ProteinAsciiHeader::writeAscii
    and one line per protein as ProteinData::writeAscii
    (Protein/ProteinData.hpp:545-564, 705-718): the heads' positions when
    both are bound, the centre twice otherwise; bound rods as gids.  Same
    bytes as the C++ facade's writer."""
    n = proteins.shape[0]
    lines = [f"{n} \n {time:f}\n"]
    for p in proteins:
        ids = [int(rod_gid[i]) if i >= 0 else -1 for i in p["idBind"]]
        if ids[0] != -1 and ids[1] != -1:
            a, b = p["posEnd"][0], p["posEnd"][1]
        else:
            a = b = p["pos"]
        tag = int(species[int(p["type"])].tag)
        lines.append("P %d %d %.6g %.6g %.6g %.6g %.6g %.6g %d %d\n"
                     % (int(p["gid"]), tag, a[0], a[1], a[2], b[0], b[1], b[2], ids[0], ids[1]))
    with open(path, "w") as f:
        f.write("".join(lines))


def read_init_box(path):
    """initBoxLow / initBoxHigh of a RunConfig.yaml (default: the sim box)."""
    vals = {}
    with open(path) as f:
        for line in f:
            line = line.split("#", 1)[0]
            if ":" in line and line[:1] not in " \t-":
                k, v = line.split(":", 1)
                vals[k.strip()] = v.strip()

    def vec(key, default):
        v = vals.get(key, vals.get(default))
        return np.array([float(x) for x in v.strip("[] ").split(",")])
    return vec("initBoxLow", "simBoxLow"), vec("initBoxHigh", "simBoxHigh")


def proteins_from_config(entries, species, rods: RodState, init_low, init_high, seed: int = 0):
    """Initial proteins from ProteinConfig.yaml's numbers, as
    TubuleSystem::setInitialProteinFromConfig (SRC/TubuleSystem.cpp:331-442):
    per species, freeNumber unbound proteins uniform in the init box, then
    for every rod one singly bound protein (end 0) per fixedLocationPerMT
    entry, at entry x L/2 from the centre (uniform on the rod when the entry
    lies outside [-1, 1]).  Gids run over all species without repeats (the
    reference numbers each species from 0, which would give proteins of
    different species the same rolls); the random numbers come from numpy
    (seed), not the reference's generator.  initCircularX is not applied."""
    from .capi import protein_array
    rng = np.random.default_rng(seed)
    parts = []
    gid = 0
    for k, e in enumerate(entries):
        nfree = int(e.get("freeNumber", 0) or 0)
        locs = e.get("fixedLocationPerMT") or []
        locs = locs if isinstance(locs, list) else [locs]
        p = protein_array(nfree)
        p["gid"] = gid + np.arange(nfree)
        p["type"] = k
        p["pos"] = init_low + rng.uniform(0.0, 1.0, (nfree, 3)) * (init_high - init_low)
        gid += nfree
        parts.append(p)
        if locs:
            nf = rods.n * len(locs)
            q = protein_array(nf)
            q["gid"] = gid + np.arange(nf)
            q["type"] = k
            r = np.repeat(np.arange(rods.n), len(locs))
            loc = np.tile(np.array(locs, float), rods.n)
            dist = np.where(np.abs(loc) > 1.0, (rng.uniform(0.0, 1.0, nf) - 0.5) * rods.length[r],
                            loc * rods.length[r] * 0.5)
            q["idBind"][:, 0] = r
            q["distBind"][:, 0] = dist
            gid += nf
            parts.append(q)
    return np.concatenate(parts) if parts else protein_array(0)
