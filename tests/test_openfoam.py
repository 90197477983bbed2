"""OpenFOAM polyMesh import: the reference's own meshes (digests of its importer's output), written
round trips, the 2D collapse, the field readers and every error the reference's importer raises
(``tests/unit/test_openfoam_reader.py``, ``tests/unit/test_collapse.py`` read as specification)."""
import os

import numpy as np
import pytest

from aquaflux_gb300 import openfoam as of
from aquaflux_gb300.mesh import backward_step_2d, structured_grid_2d, structured_grid_3d
from oracle import fv_oracle as fo

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "openfoam.npz"))
# the reference checkout (its fixture and validation meshes); tests that read it skip without it
REFERENCE = os.environ.get("AQUAFLUX_REFERENCE", "")
POLYMESH_DIRS = {
    "slab2d": "tests/fixtures/polymesh_2d_slab",
    "slab2d_fb": "tests/fixtures/polymesh_2d_slab_frontandback",
    "cubes3d": "tests/fixtures/polymesh_3d_two_cubes",
    "pitzdaily": "validation/pitzdaily_openfoam/of_case",
    "bfs3d": "validation/bfs3d_species/of_case",
}


def _digest(a, dtype):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(np.asarray(a), dtype=dtype).tobytes()).hexdigest()


def _geometry(mesh):
    topo = fo.Topology(mesh.owner, mesh.neighbour, mesh.n_cells, mesh.fn_offsets, mesh.fn_indices)
    return fo.geometry(topo, fo._t(mesh.nodes))


@pytest.mark.parametrize("key", list(POLYMESH_DIRS))
def test_reference_meshes_import_identically(key):
    """Bit-identical to ``read_openfoam`` (``aquaflux/io/openfoam/reader.py:133``) on the
    reference's fixture and validation polyMeshes, collapse included."""
    path = os.path.join(REFERENCE, POLYMESH_DIRS[key])
    if not REFERENCE or not os.path.isdir(path):
        pytest.skip("reference checkout not present")
    m = of.read_openfoam(path)
    assert [m.dim, m.n_cells, m.n_faces, m.n_nodes] == GOLDEN[f"{key}_counts"].tolist()
    got = [_digest(m.nodes, np.float64), _digest(m.fn_offsets, np.int64),
           _digest(m.fn_indices, np.int64), _digest(m.owner, np.int64),
           _digest(m.neighbour, np.int64)]
    assert got == GOLDEN[f"{key}_digest"].tolist()
    names = GOLDEN[f"{key}_patch_names"].tolist()
    assert sorted(m.patches) == sorted(names)
    assert [_digest(m.patches[n], np.int64) for n in names] == GOLDEN[f"{key}_patch_digest"].tolist()
    g = _geometry(m)
    vol = g["volume"].numpy()
    totals = np.array([vol.sum(), np.abs(g["area"].numpy()).sum(),
                       *(vol[:, None] * g["cell_centroid"].numpy()).sum(0)])
    np.testing.assert_allclose(totals, GOLDEN[f"{key}_geometry"], rtol=1e-12, atol=1e-15)
    assert np.all(vol > 0)


def _same_2d_mesh(a, b, face_order=None):
    """Same cells, faces (in ``face_order`` of ``b``) and edge geometry, node numbering aside."""
    order = np.arange(b.n_faces) if face_order is None else face_order
    assert a.n_cells == b.n_cells and a.n_faces == b.n_faces
    ea = a.nodes[a.fn_indices.reshape(-1, 2)]
    eb = b.nodes[b.fn_indices.reshape(-1, 2)][order]
    same = np.all(ea == eb, axis=(1, 2)) | np.all(ea == eb[:, ::-1], axis=(1, 2))
    assert same.all()
    pair_a = np.sort(np.stack([a.owner, a.neighbour], 1), 1)
    pair_b = np.sort(np.stack([b.owner, b.neighbour], 1), 1)[order]
    np.testing.assert_array_equal(pair_a, pair_b)


@pytest.mark.parametrize("caps", [("front", "back"), ("frontAndBack",)])
def test_extruded_round_trip_collapses_to_the_2d_mesh(tmp_path, caps):
    m2 = backward_step_2d(n_step=4, n_channel=6, n_upstream=5, n_downstream=12)
    m3 = of.extrude_2d(m2, 0.1, caps=caps)
    types = {c: "empty" for c in caps}
    order = of.write_polymesh(m3, tmp_path / "constant" / "polyMesh",
                              {**types, "step": "wall", "top": "wall", "bottom": "wall"})
    reader = of.OpenFOAMReader(tmp_path)  # a case directory resolves to constant/polyMesh
    back = reader.read()
    assert back.dim == 2 and reader.kept_axes == (0, 1)
    side = order[order < m2.n_faces]  # caps are written after every side face
    _same_2d_mesh(back, m2, side)
    # geometry of the imported mesh equals the native one's, face for face
    ga, gb = _geometry(back), _geometry(m2)
    np.testing.assert_array_equal(ga["area"].numpy(), gb["area"].numpy()[side])
    np.testing.assert_allclose(ga["volume"].numpy(), gb["volume"].numpy(), rtol=1e-14)
    np.testing.assert_allclose(ga["cell_centroid"].numpy(), gb["cell_centroid"].numpy(),
                               rtol=1e-13, atol=1e-15)
    for name in ("inlet", "outlet", "step", "top", "bottom"):
        np.testing.assert_array_equal(np.sort(side[back.patches[name]]), np.sort(m2.patches[name]))
    assert not set(caps) & set(back.patches)


def test_3d_round_trip_is_exact(tmp_path):
    m = structured_grid_3d(3, 2, 2, 1.5, 1.0, 0.5)
    rng = np.random.default_rng(1)
    m = m.with_nodes(m.nodes + rng.uniform(-0.01, 0.01, m.nodes.shape))
    order = of.write_polymesh(m, tmp_path)
    back = of.read_openfoam(tmp_path)
    assert back.dim == 3 and back.n_cells == m.n_cells
    np.testing.assert_array_equal(back.nodes, m.nodes)  # repr round trip is exact
    # OpenFOAM order: interior first, upper triangular, owner < neighbour
    n_int = back.n_interior
    assert np.all(back.neighbour[:n_int] >= 0) and np.all(back.neighbour[n_int:] == -1)
    assert np.all(back.owner[:n_int] < back.neighbour[:n_int])
    key = back.owner[:n_int].astype(np.int64) * back.n_cells + back.neighbour[:n_int]
    assert np.all(np.diff(key) > 0)
    for name, faces in m.patches.items():
        np.testing.assert_array_equal(order[back.patches[name]], faces)
    ga, gb = _geometry(back), _geometry(m)
    np.testing.assert_allclose(ga["volume"].numpy(), gb["volume"].numpy(), rtol=1e-13)
    np.testing.assert_allclose(ga["area"].numpy(), gb["area"].numpy()[order], rtol=1e-14)


def _write(d, name, cls, body, fmt="ascii"):
    d.mkdir(parents=True, exist_ok=True)
    (d / name).write_text("/* banner */\nFoamFile\n{\n    version 2.0;\n    format " + fmt
                          + ";\n    class " + cls + ";\n    object " + name + ";\n}\n// c\n" + body)


def _slab(d, boundary_types=("empty", "empty"), front_x=None):
    """Two hexes side by side along x, one cell thick in z (the reference's slab fixture shape,
    written here from scratch)."""
    pts = [(x, y, z) for z in (0.0, 0.1) for y in (0.0, 1.0) for x in (0.0, 1.0, 2.0)]
    if front_x is not None:
        pts[6] = (front_x, 0.0, 0.1)

    def n(ix, iy, iz):
        return iz * 6 + iy * 3 + ix
    faces = [[n(1, 0, 0), n(1, 1, 0), n(1, 1, 1), n(1, 0, 1)],  # interior x = 1
             [n(0, 0, 0), n(0, 0, 1), n(0, 1, 1), n(0, 1, 0)],  # left
             [n(2, 0, 0), n(2, 1, 0), n(2, 1, 1), n(2, 0, 1)],  # right
             [n(0, 0, 0), n(1, 0, 0), n(1, 0, 1), n(0, 0, 1)],  # bottom cell 0
             [n(1, 0, 0), n(2, 0, 0), n(2, 0, 1), n(1, 0, 1)],  # bottom cell 1
             [n(0, 1, 0), n(0, 1, 1), n(1, 1, 1), n(1, 1, 0)],  # top cell 0
             [n(1, 1, 0), n(1, 1, 1), n(2, 1, 1), n(2, 1, 0)],  # top cell 1
             [n(0, 0, 0), n(0, 1, 0), n(1, 1, 0), n(1, 0, 0)],  # back cell 0
             [n(1, 0, 0), n(1, 1, 0), n(2, 1, 0), n(2, 0, 0)],  # back cell 1
             [n(0, 0, 1), n(1, 0, 1), n(1, 1, 1), n(0, 1, 1)],  # front cell 0
             [n(1, 0, 1), n(2, 0, 1), n(2, 1, 1), n(1, 1, 1)]]  # front cell 1
    owner = [0, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1]
    _write(d, "points", "vectorField",
           f"{len(pts)}\n(\n" + "\n".join("(%r %r %r)" % p for p in pts) + "\n)\n")
    _write(d, "faces", "faceList", f"{len(faces)}\n(\n"
           + "\n".join(f"{len(f)}(" + " ".join(map(str, f)) + ")" for f in faces) + "\n)\n")
    _write(d, "owner", "labelList", "11\n(\n" + "\n".join(map(str, owner)) + "\n)\n")
    _write(d, "neighbour", "labelList", "1\n(\n1\n)\n")
    t_back, t_front = boundary_types
    _write(d, "boundary", "polyBoundaryMesh", f"""5
(
    left {{ type patch; nFaces 1; startFace 1; }}
    right {{ type patch; nFaces 1; startFace 2; }}
    walls {{ type wall; inGroups List<word> 1(wall); nFaces 4; startFace 3; }}
    back {{ type {t_back}; nFaces 2; startFace 7; }}
    front {{ type {t_front}; nFaces 2; startFace 9; }}
)
""")


def test_slab_collapse_matches_a_2d_grid(tmp_path):
    _slab(tmp_path)
    m = of.read_openfoam(tmp_path)
    assert m.dim == 2 and m.n_cells == 2 and m.n_faces == 7 and m.n_nodes == 6
    # nodes in lexicographic (x, y) order of the quantised in-plane positions
    np.testing.assert_array_equal(m.nodes, [[0, 0], [0, 1], [1, 0], [1, 1], [2, 0], [2, 1]])
    assert sorted(m.patches) == ["left", "right", "walls"]
    np.testing.assert_array_equal(m.patches["walls"], [3, 4, 5, 6])
    g = _geometry(m)
    np.testing.assert_allclose(g["volume"].numpy(), [1.0, 1.0])
    ref = _geometry(structured_grid_2d(2, 1, 2.0, 1.0))
    np.testing.assert_allclose(np.sort(g["cell_centroid"].numpy(), 0),
                               np.sort(ref["cell_centroid"].numpy(), 0))


def test_cell_zones_and_optional_files(tmp_path):
    _slab(tmp_path, ("patch", "patch"))
    _write(tmp_path, "cellZones", "regIOobject",
           "2\n(\nleftZone\n{\n type cellZone;\ncellLabels List<label> 1(0);\n}\n"
           "empty\n{\n type cellZone;\ncellLabels List<label> 0();\n}\n)\n")
    poly = of.OpenFOAMReader(tmp_path).read_polymesh()
    assert list(poly.cell_zones) == ["leftZone", "empty"]
    np.testing.assert_array_equal(poly.cell_zones["leftZone"], [0])
    assert poly.cell_zones["empty"].size == 0
    m = of.read_openfoam(tmp_path)  # no empty patches: stays 3D
    assert m.dim == 3 and set(m.patches) == {"left", "right", "walls", "back", "front"}
    (tmp_path / "neighbour").unlink()  # optional: every face becomes a boundary face
    (tmp_path / "cellZones").unlink()
    m = of.read_openfoam(tmp_path)
    assert m.n_cells == 2 and np.all(m.neighbour == -1)


@pytest.mark.parametrize("case, match", [
    ("binary", "binary format"),
    ("count", "declares 12 entries but lists 11"),
    ("face_n", "declares 5 nodes but lists 4"),
    ("no_header", "no 'FoamFile"),
    ("reserved", "reserved"),
    ("long_nb", "longer than the face count"),
    ("missing_startface", "missing 'startFace'"),
    ("no_points", "no polyMesh found"),
    ("no_faces", "polyMesh file not found"),
    ("bad_point", "three coordinates"),
])
def test_reader_errors(tmp_path, case, match):
    _slab(tmp_path, ("patch", "patch"))
    body = lambda n: (tmp_path / n).read_text()  # noqa: E731
    if case == "binary":
        (tmp_path / "faces").write_text(body("faces").replace("format ascii", "format binary"))
    elif case == "count":
        (tmp_path / "faces").write_text(body("faces").replace("11\n(", "12\n(", 1))
    elif case == "face_n":
        (tmp_path / "faces").write_text(body("faces").replace("\n4(1 4 10 7)", "\n5(1 4 10 7)"))
    elif case == "no_header":
        (tmp_path / "owner").write_text("11\n(\n0 0 1 0 1 0 1 0 1 0 1\n)\n")
    elif case == "reserved":
        (tmp_path / "boundary").write_text(body("boundary").replace("left {", "boundary {"))
    elif case == "long_nb":
        (tmp_path / "neighbour").write_text(body("neighbour").replace(
            "1\n(\n1\n)", "12\n(\n" + "1\n" * 12 + ")"))
    elif case == "missing_startface":
        (tmp_path / "boundary").write_text(body("boundary").replace(
            "nFaces 1; startFace 1;", "nFaces 1;"))
    elif case == "no_points":
        (tmp_path / "points").unlink()
    elif case == "no_faces":
        (tmp_path / "faces").unlink()
    elif case == "bad_point":
        (tmp_path / "points").write_text(body("points").replace("(0.0 0.0 0.0)", "(0.0 0.0)"))
    with pytest.raises((ValueError, FileNotFoundError, NotImplementedError), match=match):
        of.read_openfoam(tmp_path)


def test_collapse_errors(tmp_path):
    _slab(tmp_path, ("patch", "patch"))
    m3 = of.read_openfoam(tmp_path)
    with pytest.raises(ValueError, match="at least one capping patch"):
        of.collapse_extruded_direction(m3, [])
    with pytest.raises(ValueError, match="normal to different axes"):
        of.collapse_extruded_direction(m3, ["back", "left"])
    with pytest.raises(ValueError, match="exactly two parallel planes"):
        of.collapse_extruded_direction(m3, ["back"])
    with pytest.raises(ValueError, match="normal to different axes"):
        of.collapse_extruded_direction(m3, ["back", "front", "left", "right"])
    with pytest.raises(ValueError, match="expects a 3D mesh"):
        of.collapse_extruded_direction(structured_grid_2d(2, 2), ["left"])
    # a warped cap (one front node pushed along x) is still planar in z: the side faces then
    # project onto three in-plane nodes
    _slab(tmp_path / "w", front_x=0.25)
    with pytest.raises(ValueError, match="distinct in-plane node"):
        of.read_openfoam(tmp_path / "w")
    # a cap that is not flat along any single axis
    pts = (tmp_path / "points").read_text().replace("(1.0 0.0 0.1)", "(1.0 0.0 0.15)")
    (tmp_path / "points").write_text(pts)
    m3 = of.read_openfoam(tmp_path)
    with pytest.raises(ValueError, match="not planar and normal to a single axis"):
        of.collapse_extruded_direction(m3, ["back", "front"])


def test_field_readers(tmp_path):
    m2 = structured_grid_2d(3, 2)
    m3 = of.extrude_2d(m2, 0.2)
    d = tmp_path / "constant" / "polyMesh"
    order = of.write_polymesh(m3, d, {"front": "empty", "back": "empty", "top": "wall"})
    reader = of.OpenFOAMReader(tmp_path)
    mesh = reader.read()
    rng = np.random.default_rng(0)
    U = rng.standard_normal((mesh.n_cells, 3))
    p = rng.standard_normal(mesh.n_cells)
    of.write_volume_field(tmp_path / "U", U, name="U",
                          patches={"left": "type fixedValue; value uniform (1 0 0);"})
    of.write_volume_field(tmp_path / "p", p, name="p")
    np.testing.assert_array_equal(of.read_volume_field(tmp_path / "U", mesh, reader.kept_axes),
                                  U[:, :2])
    np.testing.assert_array_equal(of.read_volume_field(tmp_path / "p", mesh), p)
    # a face flux: internal list, uniform and nonuniform patches, empty caps without values
    n_int = mesh.n_interior
    sizes = {name: mesh.patches[name].size for name in ("left", "right", "bottom", "top")}
    starts = {name: int(mesh.patches[name][0]) for name in sizes}
    assert sorted(starts.values()) == list(starts.values())  # written in patch order
    vals = rng.standard_normal(n_int)
    right = rng.standard_normal(sizes["right"])
    text = ("FoamFile { format ascii; class surfaceScalarField; object phi; }\n"
            f"internalField nonuniform List<scalar> {n_int} (" + " ".join(repr(float(x)) for x in vals) + ");\n"
            "boundaryField {\n left { type calculated; value uniform -0.5; }\n"
            f" right {{ type calculated; value nonuniform List<scalar> {sizes['right']} ("
            + " ".join(repr(float(x)) for x in right) + "); }\n"
            " bottom { type calculated; value uniform 0; }\n top { type calculated; value uniform 0; }\n"
            " front { type empty; value nonuniform List<scalar> 0(); }\n back { type empty; }\n}\n")
    (tmp_path / "phi").write_text(text)
    phi = of.read_surface_scalar_field(tmp_path / "phi", mesh)
    np.testing.assert_array_equal(phi[:n_int], vals)
    np.testing.assert_array_equal(phi[mesh.patches["left"]], -0.5)
    np.testing.assert_array_equal(phi[mesh.patches["right"]], right)
    (tmp_path / "phi").write_text(text.replace(" left { type calculated; value uniform -0.5; }\n",
                                               ""))
    with pytest.raises(ValueError, match="no boundaryField entry for patch 'left'"):
        of.read_surface_scalar_field(tmp_path / "phi", mesh)
    # a mesh not in OpenFOAM's face order is refused
    with pytest.raises(ValueError, match="not OpenFOAM's"):
        of.read_surface_scalar_field(tmp_path / "phi", m2)
    assert order.size == m3.n_faces


def test_writer_rejects_uncovered_boundary_faces(tmp_path):
    m = structured_grid_3d(2, 1, 1)
    m.patches.pop("left")
    with pytest.raises(ValueError, match="exactly one"):
        of.write_polymesh(m, tmp_path)
    with pytest.raises(ValueError, match="3D"):
        of.write_polymesh(structured_grid_2d(2, 2), tmp_path)
