"""OpenFOAM polyMesh import (ASCII) and the collapse of one-cell-thick 2D cases.

The reader follows the reference's import path (``aquaflux/io/openfoam/reader.py:34-146``):

* ``points`` / ``faces`` / ``owner`` / ``neighbour`` / ``boundary`` / ``cellZones`` are FoamFile
  text files: a ``FoamFile { ... }`` header, then a counted list ``N ( ... )``
  (``io/openfoam/foamfile.py:38-120``, ``io/openfoam/grammar.py:27-136``); ``format binary`` is
  refused rather than misread, ``neighbour`` and ``cellZones`` are optional;
* faces keep OpenFOAM's numbering (interior faces first, then each patch as a contiguous block),
  the interior-only ``neighbour`` list is padded with ``-1``, the cell count is one past the
  largest referenced cell, and the patch names ``interior`` / ``boundary`` are refused
  (``io/openfoam/assembler.py:24-115``);
* a case whose ``boundary`` file holds ``empty`` patches is a 2D case stored one cell thick, and is
  collapsed to a genuine 2D mesh (``aquaflux/mesh/collapse.py:37-239``, restated in
  :func:`collapse_extruded_direction`).

The field readers (``io/openfoam/fields.py:41-229``) read the internal values of a cell field and a
face flux laid out on the imported face order.  :func:`write_polymesh` and :func:`extrude_2d` are
the inverse direction (a 2D mesh extruded one cell thick and written as a polyMesh), which the
reference does not have; they make imported meshes testable without OpenFOAM.

Everything here is host-side numpy: the output is a :class:`~aquaflux_gb300.mesh.MeshData` that
:class:`~aquaflux_gb300.fv.DeviceMesh` uploads once.
"""
from __future__ import annotations

import dataclasses
import re
from pathlib import Path

import numpy as np

from .mesh import MeshData

__all__ = [
    "FoamPatch", "PolyMesh", "OpenFOAMReader", "read_openfoam", "read_foam_file",
    "parse_points", "parse_labels", "parse_faces", "parse_boundary", "parse_cell_zones",
    "assemble", "collapse_extruded_direction", "parse_field", "read_volume_field",
    "read_surface_scalar_field", "extrude_2d", "write_polymesh", "write_volume_field",
]

# Patch names the reference assigns by itself from the boundary mask (assembler.py:20-22).
RESERVED_PATCH_NAMES = ("interior", "boundary")
# Coincidence tolerance of the collapse, relative to the mesh's largest extent (collapse.py:34).
COLLAPSE_RELATIVE_TOLERANCE = 1e-8

_COMMENT = re.compile(r"/\*.*?\*/|//[^\n]*", re.DOTALL)
_HEADER = re.compile(r"FoamFile\s*\{([^{}]*)\}", re.DOTALL)
_ENTRY = re.compile(r"(\w+)\s+([^;{}]+);")
_LIST_START = re.compile(r"(\d+)\s*\(")
_GROUP = re.compile(r"(\d+)\s*\(([^()]*)\)")
_BLOCK = re.compile(r"(\w+)\s*\{([^{}]*)\}", re.DOTALL)


@dataclasses.dataclass(frozen=True)
class FoamPatch:
    """One entry of the ``boundary`` file: faces ``[start_face, start_face + n_faces)``."""

    name: str
    type: str
    start_face: int
    n_faces: int


@dataclasses.dataclass
class PolyMesh:
    """The parsed polyMesh files before assembly (``io/openfoam/records.py``)."""

    points: np.ndarray  # (n_points, 3) float64
    fn_offsets: np.ndarray  # (n_faces + 1,) int64
    fn_indices: np.ndarray  # int64, perimeter order
    owner: np.ndarray  # (n_faces,) int64
    neighbour_internal: np.ndarray  # (n_internal_faces,) int64
    patches: tuple  # FoamPatch, file order
    cell_zones: dict  # zone name -> int64 cell labels


# ----------------------------------------------------------------------------- file envelope

def read_foam_file(path) -> tuple[dict, str]:
    """Header dictionary and comment-free payload of one FoamFile; refuses ``format binary``."""
    path = Path(path)
    if not path.exists():
        raise FileNotFoundError(f"OpenFOAM file not found: {path}")
    text = _COMMENT.sub(" ", path.read_text())
    head = _HEADER.search(text)
    if head is None:
        raise ValueError(f"{path}: not an OpenFOAM file (no 'FoamFile {{ ... }}' header)")
    header = {k: v.strip().strip('"') for k, v in _ENTRY.findall(head.group(1))}
    if header.get("format", "ascii").strip().lower() == "binary":
        raise NotImplementedError(f"{path} is in binary format; only ASCII files are supported")
    return header, text[head.end():]


def _counted_list(body: str, what: str) -> tuple[int, str]:
    """Declared count and inner text of the first ``N ( ... )`` list, matched by depth."""
    m = _LIST_START.search(body)
    if m is None:
        raise ValueError(f"{what}: expected a 'N ( ... )' list")
    depth, start = 0, m.end() - 1
    for i in range(start, len(body)):
        c = body[i]
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
            if depth == 0:
                return int(m.group(1)), body[start + 1:i]
    raise ValueError(f"{what}: unbalanced parentheses")


def _check_count(what: str, declared: int, found: int) -> None:
    if declared != found:
        raise ValueError(f"{what} declares {declared} entries but lists {found}")


# ----------------------------------------------------------------------------- payload grammars

def parse_points(body: str) -> np.ndarray:
    """``vectorField`` payload -> ``(n, 3)`` float64."""
    count, inner = _counted_list(body, "points")
    rows = re.findall(r"\(([^()]*)\)", inner)
    _check_count("points", count, len(rows))
    if count == 0:
        return np.zeros((0, 3))
    tokens = " ".join(rows).split()
    if len(tokens) != 3 * count:
        raise ValueError("each point must have three coordinates")
    pts = np.array(tokens, dtype=np.float64).reshape(count, 3)
    widths = np.fromiter((len(r.split()) for r in rows), dtype=np.int64, count=count)
    if np.any(widths != 3):
        raise ValueError("each point must have three coordinates")
    return pts


def parse_labels(body: str) -> np.ndarray:
    """``labelList`` payload (``owner`` / ``neighbour``) -> int64."""
    count, inner = _counted_list(body, "label list")
    tokens = inner.split()
    _check_count("label list", count, len(tokens))
    return np.array(tokens, dtype=np.int64) if tokens else np.zeros(0, dtype=np.int64)


def parse_faces(body: str) -> tuple[np.ndarray, np.ndarray]:
    """``faceList`` payload ``n(i0 .. i{n-1})`` -> CSR ``(offsets, indices)`` (int64)."""
    count, inner = _counted_list(body, "faces")
    groups = _GROUP.findall(inner)
    _check_count("face list", count, len(groups))
    declared = np.fromiter((int(g[0]) for g in groups), dtype=np.int64, count=count)
    flat = " ".join(g[1] for g in groups).split()
    listed = np.fromiter((len(g[1].split()) for g in groups), dtype=np.int64, count=count)
    bad = np.flatnonzero(declared != listed)
    if bad.size:
        f = int(bad[0])
        raise ValueError(f"face {f} declares {declared[f]} nodes but lists {listed[f]}")
    offsets = np.concatenate([[0], np.cumsum(listed)]).astype(np.int64)
    return offsets, (np.array(flat, dtype=np.int64) if flat else np.zeros(0, dtype=np.int64))


def _dict_entries(block: str) -> dict:
    return {k: v.strip() for k, v in _ENTRY.findall(block)}


def parse_boundary(body: str) -> tuple:
    """``polyBoundaryMesh`` payload -> :class:`FoamPatch` records in file order."""
    count, inner = _counted_list(body, "boundary")
    patches = []
    for name, block in _BLOCK.findall(inner):
        e = _dict_entries(block)
        try:
            patches.append(FoamPatch(name, e.get("type", ""), int(e["startFace"]),
                                     int(e["nFaces"])))
        except KeyError as missing:
            raise ValueError(f"boundary patch '{name}' is missing {missing}") from None
    _check_count("boundary", count, len(patches))
    return tuple(patches)


def parse_cell_zones(body: str) -> dict:
    """``cellZones`` payload -> ``{name: int64 cell labels}``."""
    count, inner = _counted_list(body, "cellZones")
    zones = {}
    for name, block in _BLOCK.findall(inner):
        m = re.search(r"cellLabels\s+(?:List<label>\s*)?(\d+)\s*\(([^()]*)\)", block)
        if m is None:
            raise ValueError(f"cellZone '{name}' has no cellLabels list")
        tokens = m.group(2).split()
        _check_count(f"cellZone '{name}'", int(m.group(1)), len(tokens))
        zones[name] = np.array(tokens, dtype=np.int64) if tokens else np.zeros(0, dtype=np.int64)
    _check_count("cellZones", count, len(zones))
    return zones


# ----------------------------------------------------------------------------- reader

def _polymesh_dir(path) -> Path:
    """``path`` itself or ``path/constant/polyMesh``, whichever holds ``points``
    (reader.py:34-48)."""
    path = Path(path)
    for cand in (path, path / "constant" / "polyMesh"):
        if (cand / "points").exists():
            return cand
    raise FileNotFoundError(f"no polyMesh found at {path} (looked for a 'points' file there and "
                            "in constant/polyMesh)")


class OpenFOAMReader:
    """Reads a polyMesh (or case) directory; :meth:`read` returns the mesh, collapsed to 2D when
    the case has ``empty`` patches (reader.py:51-130)."""

    def __init__(self, directory):
        self.directory = str(_polymesh_dir(directory))
        self.kept_axes: tuple | None = None  # the axes a 2D collapse kept, after read()

    def _file(self, name: str, parser, required: bool = True):
        path = Path(self.directory) / name
        if not path.exists():
            if required:
                raise FileNotFoundError(f"polyMesh file not found: {path}")
            return None
        return parser(read_foam_file(path)[1])

    def read_polymesh(self) -> PolyMesh:
        """The parsed files (the reader's only file I/O)."""
        points = self._file("points", parse_points)
        offsets, indices = self._file("faces", parse_faces)
        owner = self._file("owner", parse_labels)
        nb = self._file("neighbour", parse_labels, required=False)
        patches = self._file("boundary", parse_boundary)
        zones = self._file("cellZones", parse_cell_zones, required=False)
        return PolyMesh(points, offsets, indices, owner,
                        np.zeros(0, dtype=np.int64) if nb is None else nb, patches,
                        {} if zones is None else zones)

    def read(self) -> MeshData:
        poly = self.read_polymesh()
        mesh = assemble(poly)
        caps = [p.name for p in poly.patches if p.type == "empty"]
        self.kept_axes = (0, 1, 2)
        if caps:
            mesh, self.kept_axes = collapse_extruded_direction(mesh, caps, return_axes=True)
        return mesh


def read_openfoam(directory) -> MeshData:
    """A polyMesh or case directory as a mesh: 3D, or 2D for an ``empty``-capped one-cell-thick
    case (reader.py:133-146)."""
    return OpenFOAMReader(directory).read()


def assemble(poly: PolyMesh) -> MeshData:
    """The parsed arrays as a validated 3D mesh, faces in OpenFOAM order (assembler.py:24-115)."""
    owner = np.asarray(poly.owner, dtype=np.int64)
    nbi = np.asarray(poly.neighbour_internal, dtype=np.int64)
    n_faces = owner.size
    if n_faces == 0:
        raise ValueError("polyMesh has no faces")
    if nbi.size > n_faces:
        raise ValueError(f"neighbour list ({nbi.size}) is longer than the face count ({n_faces})")
    clash = [p.name for p in poly.patches if p.name in RESERVED_PATCH_NAMES]
    if clash:
        raise ValueError(f"boundary patch name(s) {clash} collide with reserved patch names "
                         f"{list(RESERVED_PATCH_NAMES)}; rename them in the polyMesh boundary file")
    if poly.fn_offsets.shape != (n_faces + 1,):
        raise ValueError(f"faces lists {poly.fn_offsets.size - 1} faces but owner has {n_faces}")
    n_cells = int(max(owner.max(), nbi.max() if nbi.size else -1)) + 1
    nb = np.concatenate([nbi, np.full(n_faces - nbi.size, -1, dtype=np.int64)])
    if poly.fn_indices.size and (poly.fn_indices.min() < 0
                                 or poly.fn_indices.max() >= poly.points.shape[0]):
        raise ValueError("a face references a point index out of range")
    patches = {}
    for p in poly.patches:
        if p.start_face < 0 or p.start_face + p.n_faces > n_faces:
            raise ValueError(f"patch '{p.name}' faces [{p.start_face}, "
                             f"{p.start_face + p.n_faces}) exceed the face count {n_faces}")
        patches[p.name] = np.arange(p.start_face, p.start_face + p.n_faces, dtype=np.int32)
    return MeshData(
        nodes=np.ascontiguousarray(poly.points, dtype=np.float64),
        fn_offsets=poly.fn_offsets.astype(np.int32),
        fn_indices=poly.fn_indices.astype(np.int32),
        owner=owner.astype(np.int32),
        neighbour=nb.astype(np.int32),
        n_cells=n_cells,
        patches=patches,
    ).validate()


# ----------------------------------------------------------------------------- 3D -> 2D collapse

def collapse_extruded_direction(mesh: MeshData, cap_patches, *, return_axes: bool = False):
    """Collapse a one-cell-thick extrusion, capped by the named patches, to its 2D mesh.

    Restates ``aquaflux/mesh/collapse.py:37-239``:

    * tolerance = 1e-8 x the largest extent of the node cloud;
    * the cap faces of all named patches are pooled; each must be flat along exactly one axis
      (node spread <= tolerance), the same axis for all, and their mean positions along it must
      form exactly two planes (values within tolerance merged);
    * in-plane node coordinates are quantised to the tolerance; the distinct quantised rows, in
      lexicographic order, are the 2D nodes (``np.unique(axis=0)`` order), each taking the
      coordinates of the originals that map to it;
    * every other face must project onto exactly two distinct 2D nodes: its first node and the
      first later node mapping elsewhere form the edge;
    * cells keep their indices, faces keep their relative order, caps are dropped and the other
      patches are renumbered onto the kept faces.

    Returns the 2D mesh (and the two kept axes when ``return_axes``).
    """
    caps = list(cap_patches)
    if not caps:
        raise ValueError("expected at least one capping patch to remove; got none")
    X = np.asarray(mesh.nodes, dtype=np.float64)
    if X.ndim != 2 or X.shape[1] != 3:
        raise ValueError(f"collapse_extruded_direction expects a 3D mesh; got dim {mesh.dim}")
    scale = float(np.max(X.max(axis=0) - X.min(axis=0)))
    if scale <= 0.0:
        raise ValueError("mesh has zero spatial extent")
    tol = COLLAPSE_RELATIVE_TOLERANCE * scale
    off = np.asarray(mesh.fn_offsets, dtype=np.int64)
    idx = np.asarray(mesh.fn_indices, dtype=np.int64)
    is_cap = np.zeros(mesh.n_faces, dtype=bool)
    for name in caps:
        if name not in mesh.patches:
            raise ValueError(f"capping patch '{name}' is not a patch of the mesh")
        is_cap[np.asarray(mesh.patches[name], dtype=np.int64)] = True
    cap_faces = np.flatnonzero(is_cap)
    if cap_faces.size == 0:
        raise ValueError(f"capping patches {caps} contain no faces")

    # per-face node spread and mean along each axis (segment reductions over the CSR lists)
    counts = np.diff(off)
    lo = np.minimum.reduceat(X[idx], off[:-1], axis=0) if idx.size else np.zeros((0, 3))
    hi = np.maximum.reduceat(X[idx], off[:-1], axis=0) if idx.size else np.zeros((0, 3))
    flat = (hi - lo)[cap_faces] <= tol
    n_flat = flat.sum(axis=1)
    bad = np.flatnonzero(n_flat != 1)
    if bad.size:
        f = int(cap_faces[bad[0]])
        raise ValueError(f"capping face {f} is not planar and normal to a single axis (constant "
                         f"along {int(n_flat[bad[0]])} axes); patches {caps} are not extrusion caps")
    axes = np.argmax(flat, axis=1)
    if np.any(axes != axes[0]):
        j = int(np.flatnonzero(axes != axes[0])[0])
        raise ValueError(f"capping faces are normal to different axes ({int(axes[0])} and "
                         f"{int(axes[j])}); patches {caps} must be the two ends of one extrusion")
    ax = int(axes[0])
    sums = np.add.reduceat(X[idx, ax], off[:-1])[cap_faces]
    planes = np.sort(sums / counts[cap_faces])
    n_planes = 1 + int(np.count_nonzero(np.diff(planes) > tol))
    if n_planes != 2:
        raise ValueError(f"capping patches {caps} must lie on exactly two parallel planes normal "
                         f"to one axis (the front and back of the extrusion); found {n_planes}")
    kept_axes = tuple(a for a in range(3) if a != ax)

    q = np.round(X[:, kept_axes] / tol).astype(np.int64)
    order = np.lexsort((q[:, 1], q[:, 0]))
    qs = q[order]
    new_row = np.concatenate([[True], np.any(qs[1:] != qs[:-1], axis=1)]) if q.shape[0] else \
        np.zeros(0, dtype=bool)
    node_map = np.empty(q.shape[0], dtype=np.int64)
    node_map[order] = np.cumsum(new_row) - 1
    nodes2 = np.zeros((int(new_row.sum()), 2))
    nodes2[node_map] = X[:, kept_axes]

    kept = np.flatnonzero(~is_cap)
    edges = np.empty((kept.size, 2), dtype=np.int64)
    for r, f in enumerate(kept):
        mapped = node_map[idx[off[f]:off[f + 1]]]
        other = mapped[mapped != mapped[0]]
        if other.size == 0 or np.any(other != other[0]):
            n_distinct = np.unique(mapped).size
            raise ValueError(f"face {int(f)} reduces to {n_distinct} distinct in-plane node(s), "
                             "not 2; the mesh is not a one-cell-thick extrusion of the removed "
                             "patches")
        edges[r] = (mapped[0], other[0])

    new_of_old = np.full(mesh.n_faces, -1, dtype=np.int64)
    new_of_old[kept] = np.arange(kept.size)
    patches = {name: new_of_old[np.asarray(faces, dtype=np.int64)].astype(np.int32)
               for name, faces in mesh.patches.items()
               if name not in caps and name not in RESERVED_PATCH_NAMES}
    out = MeshData(
        nodes=np.ascontiguousarray(nodes2),
        fn_offsets=(np.arange(kept.size + 1) * 2).astype(np.int32),
        fn_indices=edges.ravel().astype(np.int32),
        owner=np.asarray(mesh.owner)[kept].astype(np.int32),
        neighbour=np.asarray(mesh.neighbour)[kept].astype(np.int32),
        n_cells=mesh.n_cells,
        patches=patches,
    ).validate()
    return (out, kept_axes) if return_axes else out


# ----------------------------------------------------------------------------- fields

_UNIFORM = re.compile(r"\buniform\s+(\([^()]*\)|[-+\d.eE]+)")


def _matching(text: str, start: int, open_c: str = "{", close_c: str = "}") -> int:
    depth = 0
    for i in range(start, len(text)):
        if text[i] == open_c:
            depth += 1
        elif text[i] == close_c:
            depth -= 1
            if depth == 0:
                return i
    raise ValueError("unbalanced braces")


def _entry_values(text: str, count: int, ncomp: int, what: str) -> np.ndarray:
    """``uniform X`` / ``uniform (x y z)`` / ``nonuniform List<..> N ( ... )`` -> ``count`` rows
    (fields.py:54-71)."""
    if "nonuniform" in text:
        declared, inner = _counted_list(text[text.index("nonuniform"):], what)
        if ncomp == 1:
            tokens = inner.split()
            listed = len(tokens)
        else:
            rows = re.findall(r"\(([^()]*)\)", inner)
            listed = len(rows)
            tokens = " ".join(rows).split()
        if declared != listed:
            raise ValueError(f"{what} declares {declared} values but lists {listed}")
        if declared != count:
            raise ValueError(f"{what} has {declared} values but {count} are expected")
        if len(tokens) != count * ncomp:
            raise ValueError(f"{what}: each value must have {ncomp} component(s)")
        vals = np.array(tokens, dtype=np.float64) if tokens else np.zeros(0)
        return vals if ncomp == 1 else vals.reshape(count, ncomp)
    m = _UNIFORM.search(text)
    if m is None:
        raise ValueError(f"{what} is neither a 'uniform' nor a 'nonuniform' entry")
    v = np.array(m.group(1).strip("()").split(), dtype=np.float64)
    if v.size != ncomp:
        raise ValueError(f"{what}: uniform value has {v.size} component(s), expected {ncomp}")
    return np.full(count, v[0]) if ncomp == 1 else np.tile(v, (count, 1))


def parse_field(body: str, n_internal: int, patch_sizes: dict, ncomp: int = 1) -> np.ndarray:
    """Field payload -> ``[internal, patch_0, patch_1, ...]`` values (fields.py:74-123);
    ``patch_sizes`` lists the patches in the order their values are laid out."""
    im = re.search(r"\binternalField\b", body)
    if im is None:
        raise ValueError("field has no internalField entry")
    bm = re.search(r"\bboundaryField\s*\{", body)
    end = bm.start() if bm else len(body)
    parts = [_entry_values(body[im.end():end], n_internal, ncomp, "internalField")]
    if patch_sizes and bm is None:
        raise ValueError("field has no boundaryField entry")
    blocks = {}
    if bm is not None:
        open_i = bm.end() - 1
        inner = body[open_i + 1:_matching(body, open_i)]
        cur = 0
        while (b := inner.find("{", cur)) != -1:
            words = inner[cur:b].split()
            close = _matching(inner, b)
            blocks[words[-1] if words else ""] = inner[b + 1:close]
            cur = close + 1
    for name, size in patch_sizes.items():
        if name not in blocks:
            raise ValueError(f"field has no boundaryField entry for patch '{name}'")
        parts.append(_entry_values(blocks[name], size, ncomp, f"patch '{name}'"))
    return np.concatenate(parts, axis=0)


def read_volume_field(path, mesh: MeshData, kept_axes=None) -> np.ndarray:
    """Internal (cell) values of a ``volScalarField`` ``(n_cells,)`` or ``volVectorField``
    ``(n_cells, len(kept_axes))`` (fields.py:126-156).  ``kept_axes`` selects the vector
    components (default: all three; the collapse's kept axes for a 2D case)."""
    header, body = read_foam_file(path)
    cls = header.get("class", "volScalarField")
    if cls == "volVectorField":
        vals = parse_field(body, mesh.n_cells, {}, ncomp=3)
        return vals[:, list(kept_axes if kept_axes is not None else (0, 1, 2))]
    if cls != "volScalarField":
        raise ValueError(f"{path}: expected a volScalarField or volVectorField, got {cls}")
    return parse_field(body, mesh.n_cells, {})


def read_surface_scalar_field(path, mesh: MeshData) -> np.ndarray:
    """A ``surfaceScalarField`` (e.g. ``phi``) on the mesh's face order, after checking that the
    order is OpenFOAM's: interior faces leading, each patch one contiguous ascending block, every
    boundary face in a patch (fields.py:159-229)."""
    interior = np.asarray(mesh.neighbour) >= 0
    n_int = int(interior.sum())
    if not interior[:n_int].all() or interior[n_int:].any():
        raise ValueError("mesh face ordering is not OpenFOAM's (interior faces are not the "
                         "leading block), so field values cannot be placed by index")
    covered = np.zeros(mesh.n_faces, dtype=bool)
    sizes = {}
    for name, faces in mesh.patches.items():
        faces = np.asarray(faces, dtype=np.int64)
        if faces.size == 0:
            continue
        if faces[0] < n_int:
            raise ValueError(f"patch '{name}' includes an interior face; ordering is not "
                             "OpenFOAM's")
        if not np.array_equal(faces, np.arange(faces[0], faces[0] + faces.size)):
            raise ValueError(f"patch '{name}' is not a contiguous block of faces")
        covered[faces] = True
        sizes[name] = int(faces.size)
    missing = int(np.count_nonzero(~covered[n_int:]))
    if missing:
        raise ValueError(f"{missing} boundary faces are not in a named patch, so the field has no "
                         "values for them; the polyMesh must tile its boundary with named patches")
    ordered = dict(sorted(sizes.items(), key=lambda kv: int(mesh.patches[kv[0]][0])))
    header, body = read_foam_file(path)
    vals = parse_field(body, n_int, ordered)
    if vals.shape[0] != mesh.n_faces:
        raise ValueError(f"field has {vals.shape[0]} values but the mesh has {mesh.n_faces} faces")
    return vals


# ----------------------------------------------------------------------------- writing

def _cell_polygons(mesh: MeshData) -> list:
    """Each 2D cell's node loop (counter-clockwise), chained from its edges."""
    E = np.asarray(mesh.fn_indices, dtype=np.int64).reshape(-1, 2)
    own = np.asarray(mesh.owner, dtype=np.int64)
    nb = np.asarray(mesh.neighbour, dtype=np.int64)
    cells = np.concatenate([own, nb[nb >= 0]])
    faces = np.concatenate([np.arange(mesh.n_faces), np.flatnonzero(nb >= 0)])
    order = np.argsort(cells, kind="stable")
    starts = np.searchsorted(cells[order], np.arange(mesh.n_cells + 1))
    X = mesh.nodes
    loops = []
    for c in range(mesh.n_cells):
        fs = faces[order[starts[c]:starts[c + 1]]]
        nxt = {}
        for a, b in E[fs]:
            nxt.setdefault(int(a), []).append(int(b))
            nxt.setdefault(int(b), []).append(int(a))
        start = int(E[fs[0], 0])
        loop, prev, cur = [start], -1, start
        for _ in range(len(fs) - 1):
            cand = [n for n in nxt[cur] if n != prev]
            if not cand:
                raise ValueError(f"cell {c}: edges do not form a closed loop")
            prev, cur = cur, cand[0]
            loop.append(cur)
        if len(set(loop)) != len(fs):
            raise ValueError(f"cell {c}: edges do not form a simple polygon")
        p = X[loop]
        area2 = np.sum(p[:, 0] * np.roll(p[:, 1], -1) - np.roll(p[:, 0], -1) * p[:, 1])
        loops.append(loop if area2 > 0 else loop[::-1])
    return loops


def extrude_2d(mesh: MeshData, thickness: float = 1.0, *, caps: tuple = ("front", "back")
               ) -> MeshData:
    """A 2D mesh extruded one cell thick along z: side faces first (quads ``a b b' a'`` in the 2D
    face order, normals out of the owner), then one cap per cell on ``z = 0`` and one on
    ``z = thickness``.  ``caps`` names the back and front cap patches (one name: a single
    ``frontAndBack``-style patch holding both)."""
    if mesh.dim != 2:
        raise ValueError("extrude_2d needs a 2D mesh")
    N = mesh.n_nodes
    X = np.concatenate([np.c_[mesh.nodes, np.zeros(N)], np.c_[mesh.nodes, np.full(N, thickness)]])
    loops = _cell_polygons(mesh)
    E = np.asarray(mesh.fn_indices, dtype=np.int64).reshape(-1, 2)
    own = np.asarray(mesh.owner, dtype=np.int64)
    # orient each side face out of its owner: the in-plane normal (dy, -dx) of a->b must point
    # from the owner's node centroid to the edge midpoint
    cent = np.array([mesh.nodes[lp].mean(axis=0) for lp in loops])
    a, b = E[:, 0], E[:, 1]
    d = mesh.nodes[b] - mesh.nodes[a]
    mid = 0.5 * (mesh.nodes[a] + mesh.nodes[b])
    flip = (d[:, 1] * (mid - cent[own])[:, 0] - d[:, 0] * (mid - cent[own])[:, 1]) < 0
    a, b = np.where(flip, b, a), np.where(flip, a, b)
    side = np.stack([a, b, b + N, a + N], axis=1)
    back = [lp[::-1] for lp in loops]  # outward normal -z
    front = [[n + N for n in lp] for lp in loops]  # outward normal +z
    cap_lists = back + front
    sizes = np.concatenate([np.full(mesh.n_faces, 4), [len(lp) for lp in cap_lists]])
    fn = np.concatenate([side.ravel(), np.concatenate(cap_lists)])
    C = mesh.n_cells
    F = mesh.n_faces
    patches = {k: np.asarray(v, dtype=np.int32) for k, v in mesh.patches.items()}
    caps = tuple(caps)
    if len(caps) == 1:
        patches[caps[0]] = np.arange(F, F + 2 * C, dtype=np.int32)
    elif len(caps) == 2:
        patches[caps[1]] = np.arange(F, F + C, dtype=np.int32)  # z = 0
        patches[caps[0]] = np.arange(F + C, F + 2 * C, dtype=np.int32)  # z = thickness
    else:
        raise ValueError("caps names one or two patches")
    return MeshData(
        nodes=X,
        fn_offsets=np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32),
        fn_indices=fn.astype(np.int32),
        owner=np.concatenate([own, np.arange(C), np.arange(C)]).astype(np.int32),
        neighbour=np.concatenate([mesh.neighbour, np.full(2 * C, -1)]).astype(np.int32),
        n_cells=C,
        patches=patches,
    ).validate()


def _header(cls: str, obj: str, note: str | None = None) -> str:
    lines = ["FoamFile", "{", "    version     2.0;", "    format      ascii;",
             f"    class       {cls};"]
    if note:
        lines.append(f'    note        "{note}";')
    lines += [f"    object      {obj};", "}", ""]
    return "\n".join(lines) + "\n"


def _fmt(x: float) -> str:
    return repr(float(x))


def write_polymesh(mesh: MeshData, directory, patch_types: dict | None = None) -> np.ndarray:
    """Write a 3D mesh as an ASCII polyMesh in OpenFOAM's face order and return that order
    (written face ``i`` is mesh face ``order[i]``).

    Interior faces come first, upper-triangular (sorted by owner, then neighbour, with
    ``owner < neighbour``: a face whose owner is the larger cell is swapped and its node list
    reversed), then each patch's faces as a contiguous block in ``mesh.patches`` order.  Every
    boundary face must be in exactly one patch.  ``patch_types`` maps patch names to their type
    (default ``patch``).  Coordinates are written with ``repr`` (exact round trip)."""
    if mesh.dim != 3:
        raise ValueError("write_polymesh writes 3D meshes (extrude a 2D one with extrude_2d)")
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    own = np.asarray(mesh.owner, dtype=np.int64)
    nb = np.asarray(mesh.neighbour, dtype=np.int64)
    off = np.asarray(mesh.fn_offsets, dtype=np.int64)
    idx = np.asarray(mesh.fn_indices, dtype=np.int64)
    interior = np.flatnonzero(nb >= 0)
    swap = own[interior] > nb[interior]
    lo = np.where(swap, nb[interior], own[interior])
    hi = np.where(swap, own[interior], nb[interior])
    o = np.lexsort((hi, lo))
    order = [interior[o]]
    seen = np.zeros(mesh.n_faces, dtype=np.int64)
    seen[interior] = 1
    patch_rows = []
    start = interior.size
    for name, faces in mesh.patches.items():
        faces = np.asarray(faces, dtype=np.int64)
        if faces.size and np.any(nb[faces] >= 0):
            raise ValueError(f"patch '{name}' contains interior faces")
        seen[faces] += 1
        order.append(faces)
        patch_rows.append((name, start, faces.size))
        start += faces.size
    if np.any(seen != 1):
        f = int(np.flatnonzero(seen != 1)[0])
        raise ValueError(f"face {f} is in {int(seen[f])} patches; every boundary face must be in "
                         "exactly one")
    order = np.concatenate(order)
    flip = np.zeros(mesh.n_faces, dtype=bool)
    flip[interior[swap]] = True
    w_own = np.where(flip, nb, own)[order]
    w_nb = np.where(flip, own, nb)[order][:interior.size]
    face_txt = []
    for f in order:
        nodes = idx[off[f]:off[f + 1]]
        if flip[f]:
            nodes = nodes[::-1]
        face_txt.append(f"{nodes.size}(" + " ".join(map(str, nodes.tolist())) + ")")
    pts = "\n".join("(" + " ".join(_fmt(v) for v in row) + ")" for row in mesh.nodes)
    note = (f"nPoints:{mesh.n_nodes}  nCells:{mesh.n_cells}  nFaces:{mesh.n_faces}  "
            f"nInternalFaces:{interior.size}")
    (d / "points").write_text(_header("vectorField", "points")
                              + f"\n{mesh.n_nodes}\n(\n{pts}\n)\n")
    (d / "faces").write_text(_header("faceList", "faces")
                             + f"\n{mesh.n_faces}\n(\n" + "\n".join(face_txt) + "\n)\n")
    (d / "owner").write_text(_header("labelList", "owner", note) + f"\n{w_own.size}\n(\n"
                             + "\n".join(map(str, w_own.tolist())) + "\n)\n")
    (d / "neighbour").write_text(_header("labelList", "neighbour", note) + f"\n{w_nb.size}\n(\n"
                                 + "\n".join(map(str, w_nb.tolist())) + "\n)\n")
    types = patch_types or {}
    blocks = []
    for name, s, n in patch_rows:
        blocks.append(f"    {name}\n    {{\n        type            {types.get(name, 'patch')};\n"
                      f"        nFaces          {n};\n        startFace       {s};\n    }}")
    (d / "boundary").write_text(_header("polyBoundaryMesh", "boundary")
                                + f"\n{len(patch_rows)}\n(\n" + "\n".join(blocks) + "\n)\n")
    return order


def write_volume_field(path, values, *, name: str, patches: dict | None = None) -> None:
    """Write cell values as a ``volScalarField`` (``(n,)``) or ``volVectorField`` (``(n, 3)``);
    ``patches`` maps patch names to a boundaryField entry body (e.g. ``"type zeroGradient;"``)."""
    v = np.asarray(values, dtype=np.float64)
    cls = "volScalarField" if v.ndim == 1 else "volVectorField"
    kind = "scalar" if v.ndim == 1 else "vector"
    if v.ndim == 1:
        body = "\n".join(_fmt(x) for x in v)
    else:
        if v.shape[1] != 3:
            raise ValueError("a vector field needs three components")
        body = "\n".join("(" + " ".join(_fmt(x) for x in row) + ")" for row in v)
    bf = "\n".join(f"    {k}\n    {{\n        {e}\n    }}" for k, e in (patches or {}).items())
    Path(path).write_text(_header(cls, name) + f"\ndimensions      [0 0 0 0 0 0 0];\n\n"
                          f"internalField   nonuniform List<{kind}>\n{v.shape[0]}\n(\n{body}\n)\n;\n\n"
                          f"boundaryField\n{{\n{bf}\n}}\n")
