"""Output and restart files of the relaxation: the host side of the
reference's writers (Particle_binary_writer, particle_binary_writer.cpp:12-400;
Mesh_binary_writer, mesh_binary_writer.cpp:36-390) and of its particle restart
(Save_particle_post_file / Load_data_for_post, sph_mesh_generation.cpp:2624-2660,
426-590).  The GPU engine holds the state; these functions read it through
the C ABI (mrsph_get_particles, mrsph_get_neighbors, mrsph_triangulate) and
write the same files, under the same names, a reference run writes:

  outdata/particle_rank_<r>_step_<n>.vtu, particle_step_<n>.pvtu, particle.pvd
  outdata/mesh_tris_rank_<r>_step_<n>.vtu, mesh_tris_step_<n>.pvtu, mesh_tris.pvd
  outdata/mesh_lset_rank_<r>_step_<n>.vti, mesh_lset_step_<n>.pvti, mesh_lset.pvd
  rstfile_particles/step_<run_time>_rank_<r>.pst, rstfile_particles/list.csv

VTU files are VTK XML UnstructuredGrid pieces with raw appended data: every
array is a little-endian UInt32 byte count followed by its values (the
header's offsets count from the byte after the '_' marker).  A .pst file is an
int32 particle count followed by x, y, z as float64 per particle.
"""
from __future__ import annotations

import os
import struct
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# VTK XML type names of the numpy dtypes the writers use
_VTK_TYPE = {np.dtype("<i4"): "Int32", np.dtype("<f4"): "Float32", np.dtype("<f8"): "Float64",
             np.dtype("u1"): "UInt8"}

# Fields written per particle by default (Particle_binary_writer::Particle_binary_writer,
# particle_binary_writer.cpp:12-30): id, local_id, type, h, NN, color, norm.
PARTICLE_FIELDS_DEFAULT = ("id", "local_id", "type", "h", "NN", "color", "norm")
# the reference's PI (glbparam.h:186), which its angle statistics divide by
PI_REF = 3.1415926
PARTICLE_FIELDS_ALL = ("id", "local_id", "type", "phi", "h", "scale", "curv", "NN", "color", "norm", "accel",
                       "vel", "timestep")


# ----------------------------------------------------------------------- VTU
def _le(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a)
    if a.dtype.byteorder == ">":
        a = a.astype(a.dtype.newbyteorder("<"))
    return a


def vtu_bytes(points: np.ndarray, cells: np.ndarray, cell_type: int,
              point_data: Sequence[Tuple[str, np.ndarray]] = (),
              cell_data: Sequence[Tuple[str, np.ndarray]] = ()) -> bytes:
    """One VTK XML UnstructuredGrid piece with raw appended arrays.

    points: (n, 3) positions (written as Float32 'Position', as the reference
    does); cells: (m, k) point indices per cell, all of one VTK cell type
    (1 vertex, 5 triangle, 10 tetrahedron); point_data / cell_data: (name,
    array) pairs, arrays of shape (n,) or (n, c) in int32, float32 or
    float64."""
    points = _le(np.asarray(points, dtype="<f4").reshape(-1, 3))
    cells = _le(np.asarray(cells, dtype="<i4"))
    if cells.ndim == 1:
        cells = cells.reshape(-1, 1)
    n, m, k = len(points), len(cells), cells.shape[1]
    blobs: List[bytes] = []
    offset = 0
    head: List[str] = []

    def add(name: str, arr: np.ndarray, indent: str, components: bool = True) -> None:
        nonlocal offset
        arr = _le(arr)
        t = _VTK_TYPE[arr.dtype]
        nc = f' NumberOfComponents="{1 if arr.ndim == 1 else arr.shape[1]}"' if components else ""
        head.append(f'{indent}<DataArray type="{t}" Name="{name}"{nc} format="appended" offset="{offset}"/>')
        raw = arr.tobytes()
        blobs.append(struct.pack("<I", len(raw)) + raw)
        offset += 4 + len(raw)

    head.append('<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">')
    head.append(" <UnstructuredGrid>")
    head.append(f'  <Piece NumberOfPoints="{n}" NumberOfCells="{m}">')
    head.append('    <PointData Vectors="vector">')
    for name, arr in point_data:
        add(name, np.asarray(arr), "      ")
    head.append("    </PointData>")
    if cell_data:
        head.append('    <CellData Vectors="vector">')
        for name, arr in cell_data:
            add(name, np.asarray(arr), "      ")
        head.append("    </CellData>")
    head.append("    <Points>")
    add("Position", points, "      ")
    head.append("    </Points>")
    head.append("    <Cells>")
    add("connectivity", cells.reshape(-1), "      ", components=False)
    add("offsets", (np.arange(1, m + 1, dtype="<i4") * k), "      ", components=False)
    add("types", np.full(m, cell_type, dtype="u1"), "      ", components=False)
    head.append("    </Cells>")
    head.append("  </Piece>")
    head.append(" </UnstructuredGrid>")
    head.append(' <AppendedData encoding="raw">')
    text = "\n".join(head) + "\n _"
    tail = "\n </AppendedData>\n</VTKFile>\n"
    return text.encode("ascii") + b"".join(blobs) + tail.encode("ascii")


def read_vtu(path: str) -> Dict[str, np.ndarray]:
    """Arrays of a VTU piece with raw appended data, by name ('Position',
    'connectivity', 'offsets', 'types' and the point / cell fields)."""
    with open(path, "rb") as f:
        data = f.read()
    mark = data.index(b'<AppendedData encoding="raw">')
    start = data.index(b"_", mark) + 1
    header = data[:mark].decode("ascii")
    out: Dict[str, np.ndarray] = {}
    inv = {v: k for k, v in _VTK_TYPE.items()}
    for line in header.splitlines():
        line = line.strip()
        if not line.startswith("<DataArray"):
            continue
        attrs = dict(kv.split("=", 1) for kv in line[len("<DataArray"):-2].split())
        attrs = {k: v.strip('"') for k, v in attrs.items()}
        dt = inv[attrs["type"]]
        off = start + int(attrs["offset"])
        nbytes = struct.unpack("<I", data[off:off + 4])[0]
        arr = np.frombuffer(data[off + 4:off + 4 + nbytes], dtype=dt).copy()
        comps = int(attrs.get("NumberOfComponents", "1"))
        if comps > 1:
            arr = arr.reshape(-1, comps)
        out[attrs["Name"]] = arr
    return out


def _pvtu_text(piece_files: Sequence[str], point_fields: Sequence[Tuple[str, str, int]],
               cell_fields: Sequence[Tuple[str, str, int]] = ()) -> str:
    lines = ['<VTKFile type="PUnstructuredGrid" version="0.1" byte_order="LittleEndian">',
             ' <PUnstructuredGrid GhostLevel="0">', "  <PPointData>"]
    for name, t, c in point_fields:
        lines.append(f'    <PDataArray type="{t}" Name="{name}" NumberOfComponents="{c}"/>')
    lines.append("  </PPointData>")
    if cell_fields:
        lines.append("  <PCellData>")
        for name, t, c in cell_fields:
            lines.append(f'    <PDataArray type="{t}" Name="{name}" NumberOfComponents="{c}"/>')
        lines.append("  </PCellData>")
    lines += ["  <PPoints>", '    <PDataArray type="Float32" Name="Position" NumberOfComponents="3"/>',
              "  </PPoints>"]
    for p in piece_files:
        lines.append(f'  <Piece Source="{p}"/>')
    lines += [" </PUnstructuredGrid>", "</VTKFile>"]
    return "\n".join(lines) + "\n"


def update_pvd(path: str, n_out: int, timestep: float, dataset: str) -> None:
    """The collection file of a series: rewritten with one DataSet entry per
    output so far (Output_pvd_file, particle_binary_writer.cpp:53-93; a
    first output, n_out = 0, starts a new collection)."""
    entries: List[str] = []
    if n_out != 0 and os.path.exists(path):
        with open(path) as f:
            entries = [ln.rstrip("\n") for ln in f if ln.strip().startswith("<DataSet")]
    entries.append(f'    <DataSet timestep="{timestep}" group="" part="0" file="{dataset}"/>')
    with open(path, "w") as f:
        f.write('<VTKFile type="Collection" version="0.1">\n  <Collection>\n')
        f.write("\n".join(entries) + "\n")
        f.write("  </Collection>\n</VTKFile>\n")


def _fields_meta(fields: Sequence[Tuple[str, np.ndarray]]) -> List[Tuple[str, str, int]]:
    out = []
    for name, a in fields:
        a = np.asarray(a)
        out.append((name, _VTK_TYPE[_le(a).dtype], 1 if a.ndim == 1 else a.shape[1]))
    return out


# ----------------------------------------------------------- particle output
def particle_point_data(sim, fields: Sequence[str] = PARTICLE_FIELDS_DEFAULT) -> List[Tuple[str, np.ndarray]]:
    """Per-particle arrays in particle-id order, named and typed as the
    reference writes them (Int32 ids, type, NN, color; Float32 scalars and
    3-vectors).  NN is the neighbour count of the last density pass, the
    particle itself included; color is the rank (0 on one GPU)."""
    need = {"xyz"}
    if "type" in fields:
        need.add("type")
    if "phi" in fields:
        need.add("phi")
    if "h" in fields:
        need.add("h")
    if "curv" in fields:
        need.add("curv")
    if "norm" in fields:
        need.add("norm")
    if "accel" in fields:
        need.add("a2")
    if "vel" in fields:
        need.add("v")
    if "scale" in fields:
        need.add("h")
    p = sim.particles(tuple(sorted(need)))
    n = sim.n
    out: List[Tuple[str, np.ndarray]] = []
    for f in fields:
        if f in ("id", "local_id"):
            a = np.arange(n, dtype="<i4")
        elif f == "type":
            a = p["type"].astype("<i4")
        elif f == "NN":
            off, _ = sim.neighbors()
            a = np.diff(off).astype("<i4")
        elif f == "color":
            a = np.zeros(n, dtype="<i4")
        elif f == "norm":
            a = p["norm"].astype("<f4")
        elif f == "accel":
            a = p["a2"].astype("<f4")
        elif f == "vel":
            a = p["v"].astype("<f4")
        elif f == "scale":
            # scale = h * CUT_OFF / CELL_RATIO (Set_particle_info, particle_mesh_generation.cpp:361-381)
            prm = sim.case.params
            a = (p["h"] * prm["cutoff"] / prm["cell_ratio"]).astype("<f4")
        elif f == "timestep":
            a = np.full(n, sim.stats()["dt"], dtype="<f4")
        else:
            a = p[f].astype("<f4")
        out.append((f, a))
    return out


class ParticleWriter:
    """Particle_binary_writer: one VTU piece per output (rank 0), its PVTU
    and the PVD collection under outdir."""

    def __init__(self, outdir: str = "outdata", fields: Sequence[str] = PARTICLE_FIELDS_DEFAULT):
        unknown = set(fields) - set(PARTICLE_FIELDS_ALL)
        if unknown:
            raise ValueError(f"unknown particle fields {sorted(unknown)}")
        self.outdir = outdir
        self.fields = tuple(fields)

    def Output_particle(self, n_out: int, sim, run_time: Optional[float] = None) -> str:
        os.makedirs(self.outdir, exist_ok=True)
        pd = particle_point_data(sim, self.fields)
        xyz = sim.particles(("xyz",))["xyz"]
        piece = f"particle_rank_0_step_{n_out}.vtu"
        with open(os.path.join(self.outdir, piece), "wb") as f:
            f.write(vtu_bytes(xyz, np.arange(len(xyz), dtype="<i4"), 1, pd))
        pvtu = f"particle_step_{n_out}.pvtu"
        with open(os.path.join(self.outdir, pvtu), "w") as f:
            f.write(_pvtu_text([piece], _fields_meta(pd)))
        t = sim.stats()["step"] if run_time is None else run_time
        update_pvd(os.path.join(self.outdir, "particle.pvd"), n_out, t, f"./{pvtu}")
        return os.path.join(self.outdir, piece)


# --------------------------------------------------------------- mesh output
def triangle_quality(xyz: np.ndarray, tris: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Area and aspect ratio (longest / shortest edge) of every triangle, the
    per-triangle 'vol' and 'aspect' of Tri_quality_statistics
    (geometry_tools/graph_mesh.cpp:411-670)."""
    p = np.asarray(xyz, dtype=np.float64)[:, :2]
    a, b, c = p[tris[:, 0]], p[tris[:, 1]], p[tris[:, 2]]
    e = np.stack([np.linalg.norm(b - a, axis=1), np.linalg.norm(c - b, axis=1), np.linalg.norm(a - c, axis=1)], 1)
    area = 0.5 * np.abs((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]))
    return area, e.max(1) / e.min(1)


def tet_quality(xyz: np.ndarray, tets: np.ndarray) -> Tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """Per-tet volume, aspect ratio (longest edge / smallest height), radius
    ratio (3 r_in / r_circ) and smallest dihedral angle in degrees (with the
    reference's PI, glbparam.h:186, as Tet_quality_statistics converts): the
    'vol', 'aspect', 'radius_ratio' and 'mindihedangle' of
    Tet_quality_statistics (geometry_tools/graph_mesh.cpp:1967-2400)."""
    P = np.asarray(xyz, dtype=np.float64)[np.asarray(tets, dtype=np.int64)]  # (m, 4, 3)
    A = P[:, :3] - P[:, 3:4]
    n0, n1, n2 = np.cross(A[:, 1], A[:, 2]), np.cross(A[:, 2], A[:, 0]), np.cross(A[:, 0], A[:, 1])
    det = np.einsum("ij,ij->i", A[:, 0], n0)
    N = np.stack([n0, n1, n2], 1) / det[:, None, None]
    N = np.concatenate([N, -N.sum(1, keepdims=True)], 1)
    H = np.linalg.norm(N, axis=2)
    r2 = 0.5 * np.einsum("ijk,ijk->ij", A, A)
    c = (r2[:, 0:1] * n0 + r2[:, 1:2] * n1 + r2[:, 2:3] * n2) / det[:, None]
    e = [P[:, a] - P[:, b] for a in range(4) for b in range(a + 1, 4)]
    longest = np.sqrt(np.max([np.einsum("ij,ij->i", v, v) for v in e], axis=0))
    u = N / H[:, :, None]
    cosd = np.stack([-np.einsum("ij,ij->i", u[:, a], u[:, b]) for a in range(4) for b in range(a + 1, 4)], 1)
    mind = np.arccos(np.clip(cosd.max(1), -1.0, 1.0)) / PI_REF * 180.0
    return np.abs(det) / 6.0, longest * H.max(1), 3.0 / H.sum(1) / np.linalg.norm(c, axis=1), mind


class MeshWriter:
    """Mesh_binary_writer (mesh_binary_writer.cpp:36-640): in 2D the
    triangle mesh, a VTU piece with one triangle cell per triangle (point
    fields as for particles, cell fields 'vol' and 'aspect'), its PVTU and
    the mesh_tris.pvd collection; in 3D the tet mesh (VTK cell type 10, cell
    fields 'vol', 'aspect', 'radius_ratio', 'mindihedangle'),
    outdata/mesh_tets_rank_0_step_<n>.vtu, mesh_tets_step_<n>.pvtu and
    mesh_tets.pvd."""

    def __init__(self, outdir: str = "outdata", fields: Sequence[str] = PARTICLE_FIELDS_DEFAULT):
        self.outdir = outdir
        self.fields = tuple(fields)

    def Output_mesh(self, n_out: int, sim, tris: Optional[np.ndarray] = None, run_time: Optional[float] = None,
                    tets: Optional[np.ndarray] = None) -> str:
        os.makedirs(self.outdir, exist_ok=True)
        if sim.case.params.get("dim", 2) == 3:
            return self._tets(n_out, sim, tets, run_time)
        if tris is None:
            tris, _ = sim.Reconstruct_tris()
        tris = np.asarray(tris, dtype="<i4").reshape(-1, 3)
        xyz = sim.particles(("xyz",))["xyz"]
        pd = particle_point_data(sim, self.fields)
        vol, aspect = triangle_quality(xyz, tris)
        cd = [("vol", vol.astype("<f4")), ("aspect", aspect.astype("<f4"))]
        piece = f"mesh_tris_rank_0_step_{n_out}.vtu"
        with open(os.path.join(self.outdir, piece), "wb") as f:
            f.write(vtu_bytes(xyz, tris, 5, pd, cd))
        pvtu = f"mesh_tris_step_{n_out}.pvtu"
        with open(os.path.join(self.outdir, pvtu), "w") as f:
            f.write(_pvtu_text([piece], _fields_meta(pd), _fields_meta(cd)))
        t = sim.stats()["step"] if run_time is None else run_time
        update_pvd(os.path.join(self.outdir, "mesh_tris.pvd"), n_out, t, f"./{pvtu}")
        return os.path.join(self.outdir, piece)

    def _tets(self, n_out: int, sim, tets: Optional[np.ndarray], run_time: Optional[float]) -> str:
        if tets is None:
            tets, _ = sim.Reconstruct_tets()
        tets = np.asarray(tets, dtype="<i4").reshape(-1, 4)
        xyz = sim.particles(("xyz",))["xyz"]
        pd = particle_point_data(sim, self.fields)
        vol, aspect, ratio, mind = tet_quality(xyz, tets)
        cd = [("vol", vol.astype("<f4")), ("aspect", aspect.astype("<f4")), ("radius_ratio", ratio.astype("<f4")),
              ("mindihedangle", mind.astype("<f4"))]
        piece = f"mesh_tets_rank_0_step_{n_out}.vtu"
        with open(os.path.join(self.outdir, piece), "wb") as f:
            f.write(vtu_bytes(xyz, tets, 10, pd, cd))
        pvtu = f"mesh_tets_step_{n_out}.pvtu"
        with open(os.path.join(self.outdir, pvtu), "w") as f:
            f.write(_pvtu_text([piece], _fields_meta(pd), _fields_meta(cd)))
        t = sim.stats()["step"] if run_time is None else run_time
        update_pvd(os.path.join(self.outdir, "mesh_tets.pvd"), n_out, t, f"./{pvtu}")
        return os.path.join(self.outdir, piece)


# ---------------------------------------------------------- level-set output
def vti_bytes(extent: Sequence[int], origin: Sequence[float], spacing: Sequence[float],
              point_data: Sequence[Tuple[str, np.ndarray]] = (),
              cell_data: Sequence[Tuple[str, np.ndarray]] = ()) -> bytes:
    """One VTK XML ImageData piece with raw appended arrays; extent is the
    number of cells per axis (points are one more), arrays in x-fastest order."""
    ext = " ".join(f"0 {int(e)}" for e in extent)
    blobs: List[bytes] = []
    offset = 0
    head = ['<VTKFile type="ImageData" version="0.1" byte_order="LittleEndian">',
            f' <ImageData WholeExtent="{ext}" Origin="{" ".join(repr(float(o)) for o in origin)}" '
            f'Spacing="{" ".join(repr(float(h)) for h in spacing)}">',
            f'  <Piece Extent="{ext}">']

    def block(tag: str, fields: Sequence[Tuple[str, np.ndarray]]) -> None:
        nonlocal offset
        head.append(f'    <{tag} Vectors="vector">')
        for name, arr in fields:
            arr = _le(np.asarray(arr))
            comps = 1 if arr.ndim <= 3 else arr.shape[-1]
            head.append(f'      <DataArray type="{_VTK_TYPE[arr.dtype]}" Name="{name}" NumberOfComponents="{comps}" '
                        f'format="appended" offset="{offset}"/>')
            raw = arr.tobytes()
            blobs.append(struct.pack("<I", len(raw)) + raw)
            offset += 4 + len(raw)
        head.append(f"    </{tag}>")

    block("PointData", point_data)
    block("CellData", cell_data)
    head += ["  </Piece>", " </ImageData>", ' <AppendedData encoding="raw">']
    return ("\n".join(head) + "\n _").encode("ascii") + b"".join(blobs) + \
        "\n </AppendedData>\n</VTKFile>\n".encode("ascii")


def corner_average(cells: np.ndarray, margin_cells: int, dim: int) -> np.ndarray:
    """Values at the corners of a level's interior cells: the mean of the 2^D
    cells around each corner (the margin supplies the outer ring), as
    Output_vti_file_lset averages cell values (lset_binary_writer.cpp:87-130).
    cells: (nz, ny, nx) with nz = 1 in 2D."""
    m = margin_cells
    if dim == 2:
        c = cells[0]
        inner = c[m - 1:c.shape[0] - m + 1, m - 1:c.shape[1] - m + 1]
        return 0.25 * (inner[:-1, :-1] + inner[1:, :-1] + inner[:-1, 1:] + inner[1:, 1:])[None]
    inner = cells[m - 1:cells.shape[0] - m + 1, m - 1:cells.shape[1] - m + 1, m - 1:cells.shape[2] - m + 1]
    acc = np.zeros(tuple(s - 1 for s in inner.shape))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                acc += inner[dz:dz + acc.shape[0], dy:dy + acc.shape[1], dx:dx + acc.shape[2]]
    return 0.125 * acc


def cell_scale(sim, level: int) -> np.ndarray:
    """Levelset::Get_scale (level_set.cpp:311-351) on every cell of a level:
    the tanh law of phi, or the curvature law (|curvature| range over the CUT
    cells of all levels) when the case selects it."""
    prm = sim.case.params
    dim = prm["dim"]
    lv = sim.case.levels[level]
    f = sim.levelset_fields(level)
    phi = lv.phi
    mp = f["max_phi"]
    dl0 = min(sim.case.levels[0].dpkg[d] / 4.0 for d in range(dim))
    lo = np.full(phi.shape, float(prm["min_dl"]))
    if prm.get("scale_law", 0) == 1:
        cut = [sim.levelset_fields(l) for l in range(len(sim.case.levels))]
        vals = np.concatenate([np.abs(g["curv"][g["tag"] == 1]) for g in cut])
        cmax, cmin = (vals.max(), vals.min()) if vals.size else (0.0, 1e20)
        mid = prm.get("middle_dl", 0.0) or 5.0 * dl0
        q = np.clip((cmax - np.abs(f["curv"])) / (cmax - cmin + 1e-20), 0.0, 1.0)
        lo = prm["min_dl"] + q * q * (mid - prm["min_dl"])
    s = lo + np.tanh(2.5 * np.abs(phi) / mp) / np.tanh(2.5) * (prm["max_dl"] - lo)
    return np.where((phi > 0) | (np.abs(phi) < dl0), s, prm["min_dl"])


class LevelSetWriter:
    """Level_set_binary_writer (lset_binary_writer.cpp:12-510) for one level:
    an ImageData piece over the level's interior cells with phi, curv and
    scale at the cell corners and the cut-cell tag ('interface') and
    characteristic tag ('char': tag_characteristic, 1 SINGULARITY, 2 SEGMENT)
    per cell, the
    cut-cell volume 'vol' and surface area 'area' per cell (the GPU's
    Calculate_volume_mass pass, zero outside the counted cells), its PVTI
    and the mesh_lset.pvd collection."""

    def __init__(self, outdir: str = "outdata"):
        self.outdir = outdir

    def Output_lset(self, n_out: int, sim, level: int = 0, run_time: Optional[float] = None) -> str:
        os.makedirs(self.outdir, exist_ok=True)
        dim = sim.case.params["dim"]
        lv = sim.case.levels[level]
        f = sim.levelset_fields(level)
        m = 4 * lv.margin
        ncell = [4 * lv.num_pkg[d] if d < dim else 0 for d in range(3)]
        spacing = [lv.dpkg[d] / 4.0 if d < dim else 1.0 for d in range(3)]
        origin = [lv.box_l[d] if d < dim else 0.0 for d in range(3)]
        pd = [("phi", corner_average(lv.phi, m, dim).astype("<f4")),
              ("curv", corner_average(f["curv"], m, dim).astype("<f4")),
              ("scale", corner_average(cell_scale(sim, level), m, dim).astype("<f4"))]
        sl = (slice(None),) if dim == 2 else (slice(m, -m),)
        tag = f["tag"][sl + (slice(m, -m), slice(m, -m))].astype("<i4")
        vm = sim.volume_mass(level, cells=True)
        inner = sl + (slice(m, -m), slice(m, -m))
        extra = getattr(sim.case, "extra", None) or {}
        if len(extra.get("singularities", ())) or len(extra.get("segments", ())):
            ctag = characteristic_fields(sim.characteristic_tags(level)[inner])[0].astype("<i4")
        else:
            ctag = np.zeros_like(tag)
        cd = [("interface", tag), ("char", ctag), ("vol", vm["vol"][inner].astype("<f4")),
              ("area", vm["area"][inner].astype("<f4"))]
        piece = f"mesh_lset_rank_0_step_{n_out}.vti"
        with open(os.path.join(self.outdir, piece), "wb") as fh:
            fh.write(vti_bytes(ncell, origin, spacing, pd, cd))
        pvti = f"mesh_lset_step_{n_out}.pvti"
        ext = " ".join(f"0 {e}" for e in ncell)
        with open(os.path.join(self.outdir, pvti), "w") as fh:
            fh.write(f'<VTKFile type="PImageData" version="0.1" byte_order="LittleEndian">\n'
                     f' <PImageData WholeExtent="{ext}" GhostLevel="0" Origin="{" ".join(map(repr, map(float, origin)))}" '
                     f'Spacing="{" ".join(map(repr, map(float, spacing)))}">\n  <PPointData>\n')
            for name, t, c in _fields_meta(pd):
                fh.write(f'    <PDataArray type="{t}" Name="{name}" NumberOfComponents="{c}"/>\n')
            fh.write("  </PPointData>\n  <PCellData>\n")
            for name, t, c in _fields_meta(cd):
                fh.write(f'    <PDataArray type="{t}" Name="{name}" NumberOfComponents="{c}"/>\n')
            fh.write(f'  </PCellData>\n  <Piece Extent="{ext}" Source="{piece}"/>\n </PImageData>\n</VTKFile>\n')
        t = sim.stats()["step"] if run_time is None else run_time
        update_pvd(os.path.join(self.outdir, "mesh_lset.pvd"), n_out, t, f"./{pvti}")
        return os.path.join(self.outdir, piece)


# ------------------------------------------------------------------ restarts
def write_pst(path: str, xyz: np.ndarray) -> None:
    """int32 count, then x, y, z (float64) per particle."""
    xyz = np.ascontiguousarray(np.asarray(xyz, dtype="<f8").reshape(-1, 3))
    with open(path, "wb") as f:
        f.write(struct.pack("<i", len(xyz)))
        f.write(xyz.tobytes())


def read_pst(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        n = struct.unpack("<i", f.read(4))[0]
        xyz = np.frombuffer(f.read(24 * n), dtype="<f8")
    if len(xyz) != 3 * n:
        raise ValueError(f"{path}: truncated particle file ({len(xyz) // 3} of {n} particles)")
    return xyz.reshape(n, 3).copy()


# Level-set restart (SPH_mesh_generation::Save_restart_file,
# sph_mesh_generation.cpp:2671-2736; Levelset::Save_lset_restart_file,
# level_set.cpp:1022-1094; Levelset_levelinfo::Write_level_set_rstfile,
# lset_level_infor.cpp:695-929): native-endian binary, written here
# little-endian.  Header: DIM, domain, box_l, box_r, particle_box,
# particle_box_l, particle_box_r (float64 x 3 each), resolution (int32 x 3),
# Lmin, Lmax, ini_num_cell (int32 x 3), num_level; level set: convergence
# error, the singularity count (int32) and points (float64 x 3 each), the
# segment count (int32) and segments (float64 x 6 each, start then end),
# the dl factors, maximum_curv_artificial,
# the cut-cell totals, maximum phi / psi, maximum / middle / minimum dl,
# maximum / minimum curvature, interface cells; level: package counts and
# ranges, dpkg, dcell; then per interior cell (x fastest) phi, n_x, n_y, n_z,
# curv, psi (float64), tag_interface, tag_characteristic (0 NORMAL, 1
# SINGULARITY, 2 SEGMENT), idx_characteristic (-1 without) (int32) and
# scale (float64).  One level, as the reference writes.
_RST_HEAD = "<i" + "d" * 18 + "i" * 3 + "ii" + "i" * 3 + "i"
_RST_LSET = "<" + "d" * 17 + "i"
_RST_LEVEL = "<idd" + "i" * 21 + "d" * 6


def characteristic_fields(chr_encoded: np.ndarray):
    """(tag_characteristic, idx_characteristic) of Levelset_cell from the
    engine's encoding (k + 1 on segment k, -(k + 1) at singularity k)."""
    c = np.asarray(chr_encoded).astype(np.int32)
    tag = np.where(c > 0, 2, np.where(c < 0, 1, 0)).astype(np.int32)
    idx = np.where(c > 0, c - 1, np.where(c < 0, -c - 1, -1)).astype(np.int32)
    return tag, idx


def save_lset_restart(sim, path: str = "rstfile/levelset.rst", level: int = -1) -> str:
    """Writes the level-set restart of one level-set level (the finest by
    default) from the engine's fields and its cut-cell volume pass."""
    case = sim.case
    prm = case.params
    dim = prm["dim"]
    nls = len(case.levels)
    level = level % nls
    lv = case.levels[level]
    f = sim.levelset_fields(level)
    vm = sim.volume_mass(level)
    m = 4 * lv.margin
    inner = (slice(None),) if dim == 2 else (slice(m, -m),)
    inner = inner + (slice(m, -m), slice(m, -m))
    box_l = [float(prm["box_l"][d]) if d < dim else 0.0 for d in range(3)]
    box_r = [float(prm["box_r"][d]) if d < dim else 0.0 for d in range(3)]
    domain = [box_r[d] - box_l[d] for d in range(3)]
    npkg = [int(lv.num_pkg[d]) if d < dim else 1 for d in range(3)]
    marg = [int(lv.margin) if d < dim else 0 for d in range(3)]
    dpkg = [float(lv.dpkg[d]) for d in range(3)]
    dcell = [x / 4.0 if d < dim else x for d, x in enumerate(dpkg)]
    dl = min(dcell[d] for d in range(dim))
    dl0 = min(case.levels[0].dpkg[d] / 4.0 for d in range(dim))
    # |curvature| range over the CUT cells of all levels
    cuts = [sim.levelset_fields(l) for l in range(nls)]
    vals = np.concatenate([np.abs(g["curv"][g["tag"] == 1]) for g in cuts])
    cmax, cmin = (float(vals.max()), float(vals.min())) if vals.size else (0.0, 1e20)
    mid = prm.get("middle_dl", 0.0) or 5.0 * dl0
    phi = lv.phi
    # the scale Calculate_volume_mass leaves in the counted cells (0 elsewhere)
    scale = np.where((phi > 0) | (np.abs(phi) < dl), cell_scale(sim, level), 0.0)
    head = struct.pack(_RST_HEAD, dim, *domain, *box_l, *box_r, *domain, *box_l, *box_r,
                       *[4 * npkg[d] if d < dim else 1 for d in range(3)], 0, 0, *npkg, 1)
    extra = getattr(case, "extra", None) or {}
    sing = np.asarray(extra.get("singularities", np.zeros((0, 3))), dtype="<f8").reshape(-1, 3)
    seg = np.asarray(extra.get("segments", np.zeros((0, 6))), dtype="<f8").reshape(-1, 6)
    lset = struct.pack("<di", 1.e-4, len(sing)) + sing.tobytes() + struct.pack("<i", len(seg)) + seg.tobytes()
    lset += struct.pack(_RST_LSET, prm["max_dl"] / dl0, mid / dl0, prm["min_dl"] / dl0,
                       min(1.0, cmax), vm["total_mass"], vm["total_mass_surface"], vm.get("total_mass_segment", 0.0),
                       vm["total_volume"], vm["total_area"], vm.get("total_length", 0.0), float(f["max_phi"]), 0.0,
                       float(prm["max_dl"]), float(mid),
                       float(prm["min_dl"]), cmax, cmin, int(vm["num_interface_cell"]))
    gnum = [npkg[d] + 2 * marg[d] for d in range(3)]
    start = [-marg[d] for d in range(3)]
    end = [npkg[d] + marg[d] for d in range(3)]
    lev = struct.pack(_RST_LEVEL, int(np.prod(gnum)), dpkg[0], dl, *npkg, *gnum, *start, *end, *start, *end, *marg,
                      *dpkg, *dcell)
    cells = [phi, f["nx"], f["ny"], f["nz"], f["curv"], np.zeros_like(phi)]
    body = b"".join(np.ascontiguousarray(c[inner], dtype="<f8").tobytes() for c in cells)
    tag = f["tag"][inner].astype("<i4")
    if len(sing) or len(seg):
        ctag, cidx = characteristic_fields(sim.characteristic_tags(level)[inner])
    else:
        ctag, cidx = np.zeros_like(tag), np.full_like(tag, -1)
    body += tag.tobytes() + ctag.astype("<i4").tobytes() + cidx.astype("<i4").tobytes()
    body += np.ascontiguousarray(scale[inner], dtype="<f8").tobytes()
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    with open(path, "wb") as fh:
        fh.write(head + lset + lev + body)
    return path


def load_lset_restart(path: str) -> dict:
    """Reads a level-set restart written by save_lset_restart (or by the
    reference on a little-endian host, one level): header values and the
    per-cell fields shaped (nz, ny, nx) over the interior cells."""
    data = open(path, "rb").read()
    o = 0
    h = struct.unpack_from(_RST_HEAD, data, o)
    o += struct.calcsize(_RST_HEAD)
    out = {"dim": h[0], "domain": h[1:4], "box_l": h[4:7], "box_r": h[7:10], "resolution": h[19:22],
           "Lmin": h[22], "Lmax": h[23], "ini_num_cell": h[24:27], "num_level": h[27]}
    ls = struct.unpack_from("<di", data, o)
    o += 12
    out["singularities"] = np.frombuffer(data, dtype="<f8", count=3 * ls[1], offset=o).reshape(-1, 3).copy()
    o += 24 * ls[1]
    nseg = struct.unpack_from("<i", data, o)[0]
    o += 4
    out["segments"] = np.frombuffer(data, dtype="<f8", count=6 * nseg, offset=o).reshape(-1, 6).copy()
    o += 48 * nseg
    vals = struct.unpack_from("<" + "d" * 17 + "i", data, o)
    o += 17 * 8 + 4
    keys = ["fac_maximum_dl", "fac_middel_dl", "fac_minimum_dl", "maximum_curv_artificial", "total_mass",
            "total_mass_surface", "total_mass_segment", "total_volume", "total_area", "total_length", "maximum_phi",
            "maximum_psi", "maximum_dl", "middel_dl", "minimum_dl", "maximum_curv", "minimum_curv"]
    out.update(dict(zip(keys, vals[:17])))
    out["convergence_error"] = ls[0]
    out["glbl_num_interface_cell"] = vals[17]
    lv = struct.unpack_from(_RST_LEVEL, data, o)
    o += struct.calcsize(_RST_LEVEL)
    npkg = lv[3:6]
    out.update(glbl_total_num_pkg=lv[0], scale=lv[1], dl=lv[2], num_pkg=npkg, glbl_num_pkg=lv[6:9],
               num_pkg_margin=lv[21:24], dpkg=lv[24:27], dcell=lv[27:30])
    shape = (npkg[2] * (4 if out["dim"] == 3 else 1), npkg[1] * 4, npkg[0] * 4)
    nc = int(np.prod(shape))
    for k in ("phi", "n_x", "n_y", "n_z", "curv", "psi"):
        out[k] = np.frombuffer(data, dtype="<f8", count=nc, offset=o).reshape(shape).copy()
        o += 8 * nc
    for k in ("tag_interface", "tag_characteristic", "idx_characteristic"):
        out[k] = np.frombuffer(data, dtype="<i4", count=nc, offset=o).reshape(shape).copy()
        o += 4 * nc
    out["scale_cells"] = np.frombuffer(data, dtype="<f8", count=nc, offset=o).reshape(shape).copy()
    o += 8 * nc
    if o != len(data):
        raise ValueError("trailing bytes in level-set restart")
    return out


def save_particle_post_file(sim, root: str = ".", run_time: Optional[int] = None, first: bool = False) -> str:
    """Save_particle_post_file (sph_mesh_generation.cpp:2624-2660): positions
    of every particle (in id order) to rstfile_particles/step_<run_time>_rank_0.pst
    and a '<run_time> <particle count>' line in rstfile_particles/list.csv,
    whose first line is the rank count (written when first is true)."""
    d = os.path.join(root, "rstfile_particles")
    os.makedirs(d, exist_ok=True)
    t = int(sim.stats()["step"] if run_time is None else run_time)
    lst = os.path.join(d, "list.csv")
    mode = "w" if first or not os.path.exists(lst) else "a"
    with open(lst, mode) as f:
        if mode == "w":
            f.write("1\n")
        f.write(f"{t} {sim.n}\n")
    path = os.path.join(d, f"step_{t}_rank_0.pst")
    write_pst(path, sim.particles(("xyz",))["xyz"])
    return path


def read_particle_list(root: str = ".") -> Tuple[int, List[Tuple[int, int]]]:
    """(rank count, [(run_time, particle count), ...]) of list.csv."""
    with open(os.path.join(root, "rstfile_particles", "list.csv")) as f:
        lines = [ln.split() for ln in f if ln.strip()]
    return int(lines[0][0]), [(int(a), int(b)) for a, b in lines[1:]]


def load_data_for_post(sim, path: str, pre_run: bool = True) -> int:
    """Load_data_for_post (sph_mesh_generation.cpp:426-590) for positions: the
    particles of a .pst file become the state (REAL, zero velocity); with
    pre_run the map and Pre_run follow, as in the reference."""
    xyz = read_pst(path)
    sim.set_state({"xyz": xyz}, pre_run=pre_run)
    return len(xyz)
