"""Cell partitions with ghost layers: the residual, its JVP and VJP evaluated partition by partition.

The reference shards its residual by cell partition with owned and ghost cells
(``build_distributed_residual`` / ``DistributedResidual.residual``,
``aquaflux/parallel/distributed.py:153-275``), refreshing the ghost rows by an all-to-all of the
partition-boundary cells (``AllToAllHaloExchange.fill``, ``aquaflux/parallel/halo.py:218-225``) once
for the state and once more for the reconstructed gradient inside the residual.  Here a partition
carries enough ghost layers that its owned rows are exact after ONE exchange of the state, so the
GPU kernels run unchanged on the local mesh with no exchange inside the residual:

* the compact residual's owned rows depend on cells up to three faces away (gradients of the
  neighbours' neighbours enter the momentum-diagonal coefficients of the neighbours), so three
  ghost layers; every corrected Green-Gauss sweep after the first reaches one layer further, and
  the limited reconstruction one more;
* the local mesh is the global mesh restricted to owned + ghost cells (``mesh.remove_cells``): the
  faces beyond the last ghost layer become boundary faces of a ``__cut__`` patch, so every local
  cell keeps its full face set and its geometry (computed on the device from the nodes) is the
  global one; only the outermost layers' rows are wrong, and they are never read;
* turbulent partitions take the global SST wall distance (gathered), not one searched over their
  own wall faces.

Partitions are contiguous blocks of the cell order (RCM-renumbered meshes give compact blocks,
the reference's ``RcmPartitioner`` choice).  :class:`PartitionedResidual` evaluates every
partition in one process (one GPU, partitions in turn: the exchange is a gather);
:class:`DistributedResidual` is one partition per rank of a ``torch.distributed`` group, the
exchange point-to-point sends and receives of the boundary cells, the VJP's ghost rows sent back
and added to their owners, dot products reduced in rank order (bitwise reproducible).
"""
from __future__ import annotations

import dataclasses

import numpy as np
import torch

from . import mesh as fm

CUT_PATCH = "__cut__"


def partition_cells(n_cells: int, n_parts: int) -> np.ndarray:
    """Partition id of every cell: ``n_parts`` contiguous, balanced blocks of the cell order."""
    if n_parts < 1 or n_parts > n_cells:
        raise ValueError(f"n_parts must be in [1, {n_cells}], got {n_parts}")
    bounds = np.linspace(0, n_cells, n_parts + 1).round().astype(np.int64)
    return np.repeat(np.arange(n_parts), np.diff(bounds))


def ghost_layers_needed(gradient_sweeps: int = 0, limited: bool = False) -> int:
    """Ghost layers that make a partition's owned rows exact with one state exchange."""
    return 3 + max(0, int(gradient_sweeps) - 1) + (1 if limited else 0)


@dataclasses.dataclass
class Partition:
    rank: int
    cells: np.ndarray      # local -> global cell id (ascending)
    owned: np.ndarray      # local positions of the owned cells (ascending)
    layer: np.ndarray      # per local cell: 0 owned, k = k-th ghost layer
    mesh: fm.MeshData      # the local mesh (``__cut__`` patch beyond the last ghost layer)

    @property
    def n_local(self) -> int:
        return int(self.cells.size)

    @property
    def ghosts(self) -> np.ndarray:
        return np.flatnonzero(self.layer > 0)


def build_partitions(mesh: fm.MeshData, parts: np.ndarray, layers: int) -> list[Partition]:
    """Owned cells ``parts == p`` plus ``layers`` ghost layers (breadth-first over the cell graph)
    for every partition ``p``."""
    ip, ix = fm.cell_adjacency_csr(mesh)
    ip = ip.astype(np.int64)
    n = mesh.n_cells
    out = []
    for p in range(int(parts.max()) + 1):
        layer = np.full(n, -1, dtype=np.int64)
        front = np.flatnonzero(parts == p)
        layer[front] = 0
        for k in range(1, layers + 1):
            if front.size == 0:
                break
            starts, ends = ip[front], ip[front + 1]
            nbrs = ix[np.concatenate([np.arange(a, b) for a, b in zip(starts, ends)])] \
                if front.size else np.zeros(0, dtype=np.int64)
            nbrs = np.unique(nbrs)
            front = nbrs[layer[nbrs] < 0]
            layer[front] = k
        keep = layer >= 0
        cells = np.flatnonzero(keep)
        local = fm.remove_cells(mesh, keep, CUT_PATCH)
        lay = layer[cells]
        out.append(Partition(p, cells, np.flatnonzero(lay == 0), lay, local))
    return out


def local_flow_bc(flow_bc: dict, part: Partition) -> dict:
    """The global boundary conditions plus a zero-gradient outflow on the cut faces (only the
    outermost ghost layer, whose rows are never read, sees it)."""
    bc = {k: v for k, v in flow_bc.items() if k in part.mesh.patches}
    if CUT_PATCH in part.mesh.patches:
        bc[CUT_PATCH] = ("outlet", 0.0)
    return bc


def local_sst(sst: dict | None, part: Partition) -> dict | None:
    if sst is None:
        return None
    out = dict(sst)
    out["walls"] = [w for w in sst["walls"] if w in part.mesh.patches]
    for key in ("k", "omega"):
        spec = {k: v for k, v in sst[key].items() if k in part.mesh.patches}
        if CUT_PATCH in part.mesh.patches:
            spec[CUT_PATCH] = ("zerograd",)
        out[key] = spec
    return out


def flow_case_factory(workload, global_wall_distance=None):
    """``make_local`` for :class:`PartitionedResidual` / :class:`DistributedResidual`: a
    :class:`aquaflux_gb300.fv.FlowCase` of ``workload``'s physics on each partition's local mesh,
    turbulent partitions taking ``global_wall_distance`` (per global cell)."""
    from . import fv

    def make(part: Partition):
        wl = workload
        mu = wl.mu
        if np.ndim(mu) == 1:
            mu = np.asarray(mu)[part.cells]
        pin = None
        if wl.pressure_pin is not None:
            hit = np.flatnonzero(part.cells == wl.pressure_pin)
            pin = int(hit[0]) if hit.size else None
        case = fv.FlowCase(fv.DeviceMesh(part.mesh), mu=mu, rho=wl.rho,
                           flow_bc=local_flow_bc(wl.flow_bc, part), pressure_pin=pin,
                           sst=local_sst(wl.sst, part), gradient=wl.gradient,
                           advection=wl.advection, k_transform=wl.k_transform,
                           omega_transform=wl.omega_transform,
                           scalar_advection=wl.scalar_advection)
        if wl.sst is not None:
            if global_wall_distance is None:
                raise ValueError("a turbulent workload needs the global wall distance")
            case.set_wall_distance(np.asarray(global_wall_distance)[part.cells])
        return case

    return make


def _gather(x: torch.Tensor, nfld: int, idx: torch.Tensor) -> torch.Tensor:
    """Field-major rows ``idx`` of every field: ``x.view(nfld, -1)[:, idx]`` flattened."""
    return x.view(nfld, -1).index_select(1, idx).reshape(-1)


class PartitionedResidual:
    """The residual, JVP and VJP of a global field-major state evaluated partition by partition in
    one process, each partition by its own evaluator on its local mesh.

    ``make_local(part) -> evaluator`` with ``residual(s)``, ``jvp(s, v)``, ``vjp(s, w)`` on local
    field-major vectors (a :class:`aquaflux_gb300.fv.FlowCase` on ``part.mesh``, or the oracle in
    the CPU tests)."""

    def __init__(self, mesh: fm.MeshData, n_fields: int, n_parts: int, layers: int, make_local,
                 device: str = "cuda"):
        self.n, self.nfld = mesh.n_cells, int(n_fields)
        self.parts = build_partitions(mesh, partition_cells(mesh.n_cells, n_parts), layers)
        self.local = [make_local(p) for p in self.parts]
        self.device = device
        self._cells = [torch.as_tensor(p.cells, device=device) for p in self.parts]
        self._owned = [torch.as_tensor(p.owned, device=device) for p in self.parts]
        self._owned_global = [torch.as_tensor(p.cells[p.owned], device=device)
                              for p in self.parts]

    def _loc(self, x, p):
        return _gather(torch.as_tensor(x, dtype=torch.float64, device=self.device), self.nfld,
                       self._cells[p])

    def _put_owned(self, out, p, local_vals):
        o = out.view(self.nfld, -1)
        o[:, self._owned_global[p]] = local_vals.view(self.nfld, -1)[:, self._owned[p]]

    def residual(self, state) -> torch.Tensor:
        out = torch.empty(self.nfld * self.n, dtype=torch.float64, device=self.device)
        for p, ev in enumerate(self.local):
            self._put_owned(out, p, ev.residual(self._loc(state, p)))
        return out

    def jvp(self, state, v) -> torch.Tensor:
        out = torch.empty(self.nfld * self.n, dtype=torch.float64, device=self.device)
        for p, ev in enumerate(self.local):
            self._put_owned(out, p, ev.jvp(self._loc(state, p), self._loc(v, p)))
        return out

    def vjp(self, state, w) -> torch.Tensor:
        """``J^T w``: each partition's VJP with the cotangent on its owned rows only, its local
        result added into the global one in partition order."""
        w = torch.as_tensor(w, dtype=torch.float64, device=self.device)
        out = torch.zeros(self.nfld * self.n, dtype=torch.float64, device=self.device)
        o = out.view(self.nfld, -1)
        for p, ev in enumerate(self.local):
            wl = torch.zeros(self.nfld * self.parts[p].n_local, dtype=torch.float64,
                             device=self.device)
            wl.view(self.nfld, -1)[:, self._owned[p]] = \
                w.view(self.nfld, -1)[:, self._owned_global[p]]
            g = ev.vjp(self._loc(state, p), wl).view(self.nfld, -1)
            o.index_add_(1, self._cells[p], g)
        return out


@dataclasses.dataclass
class HaloPlan:
    """Rank ``me``'s side of the ghost exchange: for every peer ``q``, the positions in my owned
    block of the cells ``q`` holds as ghosts (``send[q]``) and the local positions of my ghosts
    that ``q`` owns (``recv[q]``), both ordered by global cell id."""

    me: int
    send: dict
    recv: dict


def halo_plans(parts: list[Partition], owner_of: np.ndarray) -> list[HaloPlan]:
    plans = []
    owned_pos = []
    for p in parts:  # position of every owned global cell inside its owner's owned block
        pos = np.full(owner_of.size, -1, dtype=np.int64)
        pos[p.cells[p.owned]] = np.arange(p.owned.size)
        owned_pos.append(pos)
    for p in parts:
        recv, send = {}, {}
        ghosts = p.ghosts
        g_owner = owner_of[p.cells[ghosts]]
        for q in range(len(parts)):
            if q == p.rank:
                continue
            sel = ghosts[g_owner == q]  # ascending local position = ascending global id
            if sel.size:
                recv[q] = sel
            # what q needs from me: my owned cells among q's ghosts
            qp = parts[q]
            qg = qp.cells[qp.ghosts]
            mine = qg[owner_of[qg] == p.rank]
            if mine.size:
                send[q] = owned_pos[p.rank][mine]
        plans.append(HaloPlan(p.rank, send, recv))
    return plans


class DistributedResidual:
    """One partition per rank of a ``torch.distributed`` process group: states and results live
    as each rank's owned block (field-major ``(n_fields, n_owned)`` flattened).

    ``fill`` is the ghost exchange (point-to-point sends and receives of the boundary cells, the
    role of ``AllToAllHaloExchange.fill``); ``vjp`` sends each ghost row's cotangent back to its
    owner, added in rank order; ``dot`` gathers the per-rank partial sums and adds them in rank
    order, so every rank holds the same, reproducible value."""

    def __init__(self, mesh: fm.MeshData, n_fields: int, layers: int, make_local, *, rank: int,
                 world: int, device: str = "cpu"):
        import torch.distributed as dist

        self.dist = dist
        self.rank, self.world = rank, world
        self.nfld = int(n_fields)
        owner_of = partition_cells(mesh.n_cells, world)
        parts = build_partitions(mesh, owner_of, layers)
        self.part = parts[rank]
        self.plan = halo_plans(parts, owner_of)[rank]
        self.local = make_local(self.part)
        self.device = device
        self.n_owned = int(self.part.owned.size)
        self._owned = torch.as_tensor(self.part.owned, device=device)
        self._owned_pos = torch.arange(self.n_owned, device=device)

    def owned_of(self, global_vec) -> torch.Tensor:
        """This rank's owned block of a global field-major vector."""
        g = torch.as_tensor(global_vec, dtype=torch.float64, device=self.device)
        idx = torch.as_tensor(self.part.cells[self.part.owned], device=self.device)
        return _gather(g, self.nfld, idx)

    def _exchange(self, payloads: dict, shapes: dict) -> dict:
        """Send ``payloads[q]`` to every q, receive a tensor of ``shapes[q]`` from every q."""
        reqs, got, held = [], {}, []
        for q, t in payloads.items():
            buf = t.contiguous()
            held.append(buf)  # alive until every request has completed
            reqs.append(self.dist.isend(buf, q))
        for q, n in shapes.items():
            buf = torch.empty(n, dtype=torch.float64, device=self.device)
            got[q] = buf
            reqs.append(self.dist.irecv(buf, q))
        for r in reqs:
            r.wait()
        return got

    def fill(self, owned: torch.Tensor) -> torch.Tensor:
        """Owned block -> local vector (owned + ghost rows), ghosts from their owners."""
        own = owned.view(self.nfld, -1)
        local = torch.zeros(self.nfld, self.part.n_local, dtype=torch.float64, device=self.device)
        local[:, self._owned] = own
        send = {q: own[:, torch.as_tensor(pos, device=self.device)].reshape(-1)
                for q, pos in self.plan.send.items()}
        shapes = {q: self.nfld * pos.size for q, pos in self.plan.recv.items()}
        for q, buf in self._exchange(send, shapes).items():
            local[:, torch.as_tensor(self.plan.recv[q], device=self.device)] = \
                buf.view(self.nfld, -1)
        return local.reshape(-1)

    def residual(self, owned_state) -> torch.Tensor:
        r = self.local.residual(self.fill(owned_state))
        return r.view(self.nfld, -1)[:, self._owned].reshape(-1)

    def jvp(self, owned_state, owned_v) -> torch.Tensor:
        jv = self.local.jvp(self.fill(owned_state), self.fill(owned_v))
        return jv.view(self.nfld, -1)[:, self._owned].reshape(-1)

    def vjp(self, owned_state, owned_w) -> torch.Tensor:
        wl = torch.zeros(self.nfld, self.part.n_local, dtype=torch.float64, device=self.device)
        wl[:, self._owned] = owned_w.view(self.nfld, -1)
        g = self.local.vjp(self.fill(owned_state), wl.reshape(-1)).view(self.nfld, -1)
        # ghost rows' cotangents go back to their owners (the reverse of fill)
        send = {q: g[:, torch.as_tensor(pos, device=self.device)].reshape(-1)
                for q, pos in self.plan.recv.items()}
        shapes = {q: self.nfld * pos.size for q, pos in self.plan.send.items()}
        got = self._exchange(send, shapes)
        got[self.rank] = g[:, self._owned].reshape(-1)
        out = torch.zeros(self.nfld, self.n_owned, dtype=torch.float64, device=self.device)
        for q in sorted(got):  # rank order, own contribution included: reproducible sums
            pos = self._owned_pos if q == self.rank else \
                torch.as_tensor(self.plan.send[q], device=self.device)
            out.index_add_(1, pos, got[q].view(self.nfld, -1))
        return out.reshape(-1)

    def dot(self, a: torch.Tensor, b: torch.Tensor) -> float:
        if a.is_cuda:  # the library's fixed-order reduction (fv_dot_f64): reproducible partials
            from .sparse import dot as device_dot

            part = device_dot(a.contiguous(), b.contiguous()).reshape(1)
        else:
            part = torch.dot(a, b).reshape(1).to(torch.float64)
        parts = [torch.empty_like(part) for _ in range(self.world)]
        self.dist.all_gather(parts, part)
        total = parts[0].clone()
        for t in parts[1:]:
            total += t
        return float(total)
