"""Host-side mesh data: structured generators, seeded node recipes, cell relabelling.

The mesh is plain struct-of-arrays numpy data (:class:`MeshData`) that the device handle
(:class:`aquaflux_gb300.residual.DeviceMesh`) uploads once.  Topology follows the reference's
conventions exactly, because connectivity must be bit-identical to it:

* owner / neighbour per face with ``-1`` marking a boundary face
  (``aquaflux/mesh/connectivity.py:81-140``);
* ragged CSR face->node lists in perimeter order (``aquaflux/mesh/connectivity.py:362-475``);
* structured grids emit face *families* normal to x, then y, then z, each family enumerated in
  ``meshgrid(..., indexing="ij")`` ravel order, owner = the low-side cell when it exists
  (``aquaflux/mesh/structured.py:63-152, 155-375``);
* relabelling keeps the face order and maps cell ``c`` to ``perm[c]``
  (``aquaflux/mesh/reorder.py:38-98``).
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class MeshData:
    """An unstructured cell-centred mesh as host arrays (int32 indices, float64 coordinates)."""

    nodes: np.ndarray  # (n_nodes, dim) float64
    fn_offsets: np.ndarray  # (n_faces + 1,) int32, CSR row pointers of the face->node lists
    fn_indices: np.ndarray  # (n_incidences,) int32, node indices in perimeter order
    owner: np.ndarray  # (n_faces,) int32
    neighbour: np.ndarray  # (n_faces,) int32, -1 on boundary faces
    n_cells: int
    patches: dict  # patch name -> int32 array of boundary face indices (ordered)

    @property
    def dim(self) -> int:
        return int(self.nodes.shape[1])

    @property
    def n_faces(self) -> int:
        return int(self.owner.shape[0])

    @property
    def n_nodes(self) -> int:
        return int(self.nodes.shape[0])

    @property
    def n_interior(self) -> int:
        return int(np.count_nonzero(self.neighbour >= 0))

    def with_nodes(self, nodes: np.ndarray) -> "MeshData":
        nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        if nodes.shape != self.nodes.shape:
            raise ValueError(f"node array must have shape {self.nodes.shape}, got {nodes.shape}")
        return dataclasses.replace(self, nodes=nodes)

    def validate(self) -> "MeshData":
        """Topological checks of ``aquaflux/mesh/mesh.py:208-319`` that matter to the kernels."""
        n_faces = self.n_faces
        if self.fn_offsets.shape != (n_faces + 1,) or int(self.fn_offsets[0]) != 0:
            raise ValueError("fn_offsets must be a CSR pointer array of length n_faces + 1")
        if int(self.fn_offsets[-1]) != self.fn_indices.shape[0]:
            raise ValueError("fn_offsets[-1] must equal len(fn_indices)")
        counts = np.diff(self.fn_offsets)
        if self.dim == 2 and np.any(counts != 2):
            raise ValueError("a 2D face must be an edge (exactly 2 nodes)")
        if self.dim == 3 and np.any(counts < 3):
            raise ValueError("a 3D face needs >= 3 nodes")
        if self.owner.min() < 0 or self.owner.max() >= self.n_cells:
            raise ValueError(f"owner index out of range [0, {self.n_cells})")
        if self.neighbour.min() < -1 or self.neighbour.max() >= self.n_cells:
            raise ValueError(f"neighbour index out of range [-1, {self.n_cells})")
        interior = self.neighbour >= 0
        if np.any(self.owner[interior] == self.neighbour[interior]):
            raise ValueError("an interior face has the same cell as owner and neighbour")
        referenced = np.zeros(self.n_cells, dtype=bool)
        referenced[self.owner] = True
        referenced[self.neighbour[interior]] = True
        if not referenced.all():
            raise ValueError(f"cell {int(np.argmin(referenced))} is not referenced by any face")
        if not np.isfinite(self.nodes).all():
            raise ValueError("node coordinates contain a non-finite value")
        return self


def graded_nodes(n: int, length: float, growth: float, *, both_sides: bool = True) -> np.ndarray:
    """Geometric wall grading, the node recipe of ``aquaflux/mesh/structured.py:19-60``."""
    if n < 1:
        raise ValueError(f"n must be >= 1, got {n}")
    if growth <= 0.0:
        raise ValueError(f"growth must be > 0, got {growth}")
    i = np.arange(n)
    power = np.minimum(i, n - 1 - i) if both_sides else i
    cum = np.concatenate([[0.0], np.cumsum(np.asarray(growth, dtype=float) ** power)])
    return length * cum / cum[-1]


def _family(owner_parts, nb_parts, node_parts, patches, counter, lo_cell, hi_cell, lo_ok, hi_ok,
            corners, lo_name, hi_name):
    owner_parts.append(np.where(lo_ok, lo_cell, hi_cell))
    nb_parts.append(np.where(lo_ok & hi_ok, hi_cell, -1))
    node_parts.append(np.stack(corners, axis=1))
    ids = counter[0] + np.arange(lo_ok.size)
    patches[lo_name] = ids[~lo_ok].astype(np.int32)
    patches[hi_name] = ids[~hi_ok].astype(np.int32)
    counter[0] += lo_ok.size


def _assemble(nodes, n_cells, owner_parts, nb_parts, node_parts, patches) -> MeshData:
    fnodes = np.concatenate(node_parts, axis=0)
    n_faces, k = fnodes.shape
    return MeshData(
        nodes=np.ascontiguousarray(nodes, dtype=np.float64),
        fn_offsets=(np.arange(n_faces + 1) * k).astype(np.int32),
        fn_indices=fnodes.ravel().astype(np.int32),
        owner=np.concatenate(owner_parts).astype(np.int32),
        neighbour=np.concatenate(nb_parts).astype(np.int32),
        n_cells=int(n_cells),
        patches=patches,
    ).validate()


def structured_grid_2d(nx: int, ny: int, lx: float = 1.0, ly: float = 1.0, *,
                       x_nodes: np.ndarray | None = None,
                       y_nodes: np.ndarray | None = None) -> MeshData:
    """Quad grid on ``[0,lx]x[0,ly]`` with patches left/right/bottom/top.

    Same face numbering as ``aquaflux/mesh/structured.py:155-282`` (non-periodic form): the
    ``(nx+1)*ny`` x-normal edges ordered by ``(i, j)`` with ``j`` fastest, then the ``nx*(ny+1)``
    y-normal edges likewise.
    """
    x = np.linspace(0.0, lx, nx + 1) if x_nodes is None else np.asarray(x_nodes, dtype=float)
    y = np.linspace(0.0, ly, ny + 1) if y_nodes is None else np.asarray(y_nodes, dtype=float)
    if x.shape != (nx + 1,) or y.shape != (ny + 1,):
        raise ValueError("node coordinate arrays must have n + 1 entries")

    def node(i, j):
        return j * (nx + 1) + i

    def cell(i, j):
        return j * nx + i

    jj, ii = np.meshgrid(np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    nodes = np.stack([x[ii].ravel(), y[jj].ravel()], axis=1)
    own, nb, fn, patches, counter = [], [], [], {}, [0]
    i, j = (a.ravel() for a in np.meshgrid(np.arange(nx + 1), np.arange(ny), indexing="ij"))
    _family(own, nb, fn, patches, counter, cell(np.clip(i - 1, 0, nx - 1), j),
            cell(np.clip(i, 0, nx - 1), j), i > 0, i < nx, [node(i, j), node(i, j + 1)],
            "left", "right")
    i, j = (a.ravel() for a in np.meshgrid(np.arange(nx), np.arange(ny + 1), indexing="ij"))
    _family(own, nb, fn, patches, counter, cell(i, np.clip(j - 1, 0, ny - 1)),
            cell(i, np.clip(j, 0, ny - 1)), j > 0, j < ny, [node(i, j), node(i + 1, j)],
            "bottom", "top")
    return _assemble(nodes, nx * ny, own, nb, fn, patches)


def structured_grid_3d(nx: int, ny: int, nz: int, lx: float = 1.0, ly: float = 1.0,
                       lz: float = 1.0) -> MeshData:
    """Hex grid on ``[0,lx]x[0,ly]x[0,lz]`` with patches left/right/bottom/top/back/front.

    Same face numbering as ``aquaflux/mesh/structured.py:285-375``: x-, then y-, then z-normal
    quad families, each in ``(i, j, k)`` ij-ravel order, with the reference's perimeter winding.
    """
    hx, hy, hz = lx / nx, ly / ny, lz / nz

    def node(i, j, k):
        return (k * (ny + 1) + j) * (nx + 1) + i

    def cell(i, j, k):
        return (k * ny + j) * nx + i

    kk, jj, ii = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    nodes = np.stack([(ii * hx).ravel(), (jj * hy).ravel(), (kk * hz).ravel()], axis=1)
    own, nb, fn, patches, counter = [], [], [], {}, [0]
    i, j, k = (a.ravel() for a in np.meshgrid(np.arange(nx + 1), np.arange(ny), np.arange(nz),
                                              indexing="ij"))
    _family(own, nb, fn, patches, counter, cell(np.clip(i - 1, 0, nx - 1), j, k),
            cell(np.clip(i, 0, nx - 1), j, k), i > 0, i < nx,
            [node(i, j, k), node(i, j + 1, k), node(i, j + 1, k + 1), node(i, j, k + 1)],
            "left", "right")
    i, j, k = (a.ravel() for a in np.meshgrid(np.arange(nx), np.arange(ny + 1), np.arange(nz),
                                              indexing="ij"))
    _family(own, nb, fn, patches, counter, cell(i, np.clip(j - 1, 0, ny - 1), k),
            cell(i, np.clip(j, 0, ny - 1), k), j > 0, j < ny,
            [node(i, j, k), node(i + 1, j, k), node(i + 1, j, k + 1), node(i, j, k + 1)],
            "bottom", "top")
    i, j, k = (a.ravel() for a in np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz + 1),
                                              indexing="ij"))
    _family(own, nb, fn, patches, counter, cell(i, j, np.clip(k - 1, 0, nz - 1)),
            cell(i, j, np.clip(k, 0, nz - 1)), k > 0, k < nz,
            [node(i, j, k), node(i + 1, j, k), node(i + 1, j + 1, k), node(i, j + 1, k)],
            "back", "front")
    return _assemble(nodes, nx * ny * nz, own, nb, fn, patches)


def jitter_interior_nodes(nodes: np.ndarray, n_per_axis, extent_per_axis, perturb: float,
                          seed: int) -> np.ndarray:
    """Displace strictly-interior lattice nodes by seeded uniform noise, ``+-perturb*h`` per axis.

    The recipe of the reference's skewed-grid helper (``tests/support/meshes.py:39-83``): the
    lattice is indexed slowest-to-fastest over the reversed axes, one ``rng.uniform`` draw of the
    whole lattice per axis in x, y[, z] order, masked to interior nodes.  ``h`` is the uniform
    spacing ``extent / n`` on each axis.
    """
    if not perturb:
        return np.array(nodes, dtype=np.float64, copy=True)
    steps = [length / n for length, n in zip(extent_per_axis, n_per_axis)]
    counts = [n + 1 for n in reversed(n_per_axis)]
    grids = np.meshgrid(*[np.arange(c) for c in counts], indexing="ij")
    interior = np.ones(grids[0].shape, dtype=bool)
    for g, n in zip(grids, reversed(n_per_axis)):
        interior &= (g > 0) & (g < n)
    rng = np.random.default_rng(seed)
    offsets = np.stack([(interior * rng.uniform(-perturb * h, perturb * h, interior.shape)).ravel()
                        for h in steps], axis=1)
    return np.asarray(nodes, dtype=np.float64) + offsets


def bump_channel_nodes_3d(shape, extent, bump_height: float, jitter: float, seed: int) -> np.ndarray:
    """Node coordinates of a hex channel with a seeded Gaussian bump on the lower (y = 0) wall.

    The bump ``h(x, z) = bump_height * exp(-((x-xc)^2 + (z-zc)^2) / (2 s^2))`` lifts every node
    by ``h(x, z) * (1 - y / ly)``, so the lower wall carries the full bump and the upper wall none.
    Its centre and width are drawn from ``default_rng(seed)``: ``xc = lx (0.3 + 0.2 u0)``,
    ``zc = lz (0.4 + 0.2 u1)``, ``s = 0.12 lx (0.8 + 0.4 u2)``.  Interior nodes are then jittered
    by :func:`jitter_interior_nodes` with amplitude ``jitter`` and seed ``seed + 1``.
    """
    nx, ny, nz = shape
    lx, ly, lz = extent
    hx, hy, hz = lx / nx, ly / ny, lz / nz
    kk, jj, ii = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    x = (ii * hx).ravel()
    y = (jj * hy).ravel()
    z = (kk * hz).ravel()
    u = np.random.default_rng(seed).random(3)
    xc, zc, s = lx * (0.3 + 0.2 * u[0]), lz * (0.4 + 0.2 * u[1]), 0.12 * lx * (0.8 + 0.4 * u[2])
    bump = bump_height * np.exp(-((x - xc) ** 2 + (z - zc) ** 2) / (2.0 * s * s))
    nodes = np.stack([x, y + bump * (1.0 - y / ly), z], axis=1)
    return jitter_interior_nodes(nodes, shape, extent, jitter, seed + 1)


def permute_cells(mesh: MeshData, perm: np.ndarray) -> MeshData:
    """Relabel cell ``c`` as ``perm[c]``; faces keep their order (``aquaflux/mesh/reorder.py:38-98``)."""
    perm = np.asarray(perm)
    if perm.shape != (mesh.n_cells,) or not np.array_equal(np.sort(perm), np.arange(mesh.n_cells)):
        raise ValueError(f"perm must be a permutation of [0, {mesh.n_cells})")
    owner = perm[mesh.owner].astype(np.int32)
    nb = np.where(mesh.neighbour >= 0, perm[np.clip(mesh.neighbour, 0, None)], -1).astype(np.int32)
    return dataclasses.replace(mesh, owner=owner, neighbour=nb).validate()


def random_permutation(n_cells: int, seed: int = 0) -> np.ndarray:
    """``RandomReordering.permutation`` (``aquaflux/mesh/reorder.py:162-176``)."""
    return np.random.default_rng(seed).permutation(n_cells)


def cell_adjacency_csr(mesh: MeshData) -> tuple[np.ndarray, np.ndarray]:
    """Symmetric cell graph of the interior faces as sorted CSR (``aquaflux/mesh/graph.py:29-91``)."""
    interior = mesh.neighbour >= 0
    o = mesh.owner[interior].astype(np.int64)
    n = mesh.neighbour[interior].astype(np.int64)
    rows = np.concatenate([o, n])
    cols = np.concatenate([n, o])
    order = np.lexsort((cols, rows))
    rows, cols = rows[order], cols[order]
    keep = np.ones(rows.size, dtype=bool)
    keep[1:] = (rows[1:] != rows[:-1]) | (cols[1:] != cols[:-1])
    rows, cols = rows[keep], cols[keep]
    indptr = np.zeros(mesh.n_cells + 1, dtype=np.int64)
    np.add.at(indptr, rows + 1, 1)
    return np.cumsum(indptr).astype(np.int32), cols.astype(np.int32)


def remove_cells(mesh: MeshData, keep: np.ndarray, patch: str) -> MeshData:
    """The sub-mesh of the cells with ``keep[c]``; kept cells are renumbered in order, faces keep
    their order.  Interior faces between a kept and a removed cell become boundary faces of the
    kept cell in the new patch ``patch``; faces touching no kept cell are dropped, and so are the
    nodes no remaining face references."""
    keep = np.asarray(keep, dtype=bool)
    new_id = np.full(mesh.n_cells, -1, dtype=np.int64)
    new_id[keep] = np.arange(int(keep.sum()))
    o = mesh.owner.astype(np.int64)
    nb = mesh.neighbour.astype(np.int64)
    ko = keep[o]
    kn = np.where(nb >= 0, keep[np.clip(nb, 0, None)], False)
    live = ko | kn
    owner = np.where(ko, new_id[o], new_id[np.clip(nb, 0, None)])
    neighbour = np.where(ko & kn, new_id[np.clip(nb, 0, None)], -1)
    exposed = (nb >= 0) & (ko ^ kn)
    face_ids = np.flatnonzero(live)
    remap = np.full(mesh.n_faces, -1, dtype=np.int64)
    remap[face_ids] = np.arange(face_ids.size)
    counts = np.diff(mesh.fn_offsets)
    rows = np.repeat(np.arange(mesh.n_faces), counts)
    fn = mesh.fn_indices[live[rows]]
    used = np.zeros(mesh.n_nodes, dtype=bool)
    used[fn] = True
    node_id = np.cumsum(used) - 1
    patches = {}
    for name, faces in mesh.patches.items():
        faces = np.asarray(faces, dtype=np.int64)
        kept = faces[live[faces]]
        patches[name] = remap[kept].astype(np.int32)
    patches[patch] = remap[np.flatnonzero(exposed)].astype(np.int32)
    return MeshData(
        nodes=np.ascontiguousarray(mesh.nodes[used]),
        fn_offsets=np.concatenate([[0], np.cumsum(counts[live])]).astype(np.int32),
        fn_indices=node_id[fn].astype(np.int32),
        owner=owner[live].astype(np.int32),
        neighbour=neighbour[live].astype(np.int32),
        n_cells=int(keep.sum()),
        patches=patches,
    ).validate()


def backward_step_2d(*, n_step: int = 48, n_channel: int = 96, n_upstream: int = 120,
                     n_downstream: int = 1300, step: float = 0.5, height: float = 1.5,
                     upstream: float = 5.0, downstream: float = 25.0, ratio_y: float = 8.0,
                     ratio_upstream: float = 5.0, ratio_downstream: float = 20.0,
                     jitter: float = 0.15, seed: int = 0) -> MeshData:
    """Two-block quad mesh of a backward-facing step (the reference ships no generator for it).

    The inlet channel ``[-upstream, 0] x [step, height]`` opens at ``x = 0`` into the channel
    ``[0, downstream] x [0, height]``; with ``height = 1.5`` and ``step = 0.5`` the inlet height is
    1 (the length unit ``h``) and the expansion ratio ``height / (height - step)`` is 1.5 on a
    ``30h x 1.5h`` domain.  Node lines are graded (:func:`graded_nodes`, geometric ``growth``)
    toward the walls, the step corner line ``y = step`` and the step face ``x = 0``, each block's
largest to smallest spacing being the given ``ratio_*``.  Every node
    strictly inside the fluid is displaced by a seeded uniform ``+-jitter`` of its local spacing
    per axis (the smaller of the two adjacent spacings).  Patches: ``inlet``, ``outlet``, ``top``,
    ``bottom`` (the lower wall downstream of the step) and ``step`` (the step face and the inlet
    channel's lower wall).
    """
    def growth(ratio, n_cells):  # geometric growth reaching `ratio` over n_cells cells
        return float(ratio) ** (1.0 / max(n_cells - 1, 1))

    y = np.concatenate([graded_nodes(n_step, step, growth(ratio_y, (n_step + 1) // 2)),
                        step + graded_nodes(n_channel, height - step,
                                            growth(ratio_y, (n_channel + 1) // 2))[1:]])
    # cells shrink toward the step face x = 0 on both sides of it
    x_up = -graded_nodes(n_upstream, upstream, growth(ratio_upstream, n_upstream),
                         both_sides=False)[::-1]
    x_down = graded_nodes(n_downstream, downstream, growth(ratio_downstream, n_downstream),
                          both_sides=False)
    x = np.concatenate([x_up, x_down[1:]])
    nx, ny = x.size - 1, y.size - 1
    full = structured_grid_2d(nx, ny, x_nodes=x, y_nodes=y)
    # jitter the strictly interior nodes of the full lattice by the local spacing
    rng = np.random.default_rng(seed)
    jj, ii = np.meshgrid(np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    dx, dy = np.diff(x), np.diff(y)
    hx = np.minimum(np.concatenate([[dx[0]], dx]), np.concatenate([dx, [dx[-1]]]))
    hy = np.minimum(np.concatenate([[dy[0]], dy]), np.concatenate([dy, [dy[-1]]]))
    ux = rng.uniform(-jitter, jitter, jj.shape)
    uy = rng.uniform(-jitter, jitter, jj.shape)
    xn, yn = x[ii], y[jj]
    inside = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)
    on_step = (xn <= 0.0) & (yn <= step)  # the step's faces and the removed block
    free = inside & ~on_step
    nodes = full.nodes.copy()
    nodes[:, 0] += (free * ux * hx[ii]).ravel()
    nodes[:, 1] += (free * uy * hy[jj]).ravel()
    full = full.with_nodes(nodes)
    ci, cj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    cell = (cj * nx + ci).ravel()
    keep = np.ones(nx * ny, dtype=bool)
    in_step = (x[ci + 1] <= 0.0) & (y[cj + 1] <= step)
    keep[cell[in_step.ravel()]] = False
    mesh = remove_cells(full, keep, "step")
    mesh.patches["inlet"] = mesh.patches.pop("left")
    mesh.patches["outlet"] = mesh.patches.pop("right")
    return mesh


def disjoint_union(meshes) -> tuple[MeshData, np.ndarray]:
    """One mesh holding independent meshes side by side: cells, faces and nodes of mesh ``i`` follow
    those of mesh ``i - 1``; patch ``name`` of mesh ``i`` becomes ``"i:name"``.  Returns the mesh and
    the cell offsets (``len(meshes) + 1``) delimiting each instance."""
    nodes, fo, fi, own, nb, patches = [], [], [], [], [], {}
    cell0 = node0 = face0 = inc0 = 0
    offsets = [0]
    for i, m in enumerate(meshes):
        nodes.append(m.nodes)
        fo.append(np.asarray(m.fn_offsets[1:], dtype=np.int64) + inc0)
        fi.append(np.asarray(m.fn_indices, dtype=np.int64) + node0)
        own.append(np.asarray(m.owner, dtype=np.int64) + cell0)
        nb.append(np.where(m.neighbour >= 0, np.asarray(m.neighbour, dtype=np.int64) + cell0, -1))
        for name, faces in m.patches.items():
            patches[f"{i}:{name}"] = (np.asarray(faces, dtype=np.int64) + face0).astype(np.int32)
        cell0 += m.n_cells
        node0 += m.n_nodes
        face0 += m.n_faces
        inc0 += int(m.fn_offsets[-1])
        offsets.append(cell0)
    union = MeshData(
        nodes=np.ascontiguousarray(np.concatenate(nodes), dtype=np.float64),
        fn_offsets=np.concatenate([np.zeros(1, dtype=np.int64)] + fo).astype(np.int32),
        fn_indices=np.concatenate(fi).astype(np.int32),
        owner=np.concatenate(own).astype(np.int32),
        neighbour=np.concatenate(nb).astype(np.int32),
        n_cells=int(cell0),
        patches=patches,
    ).validate()
    return union, np.asarray(offsets, dtype=np.int32)
