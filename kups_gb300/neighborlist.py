"""Neighbour lists on the GPU behind kUPS's ``NearestNeighborList`` protocol.

Mirrors src/kups/core/neighborlist.py: ``Edges`` (:115-212),
``NearestNeighborList.__call__(lh, rh, systems, cutoffs, rh_index_remap)``
(:226-255), ``CellListNeighborList`` (:985-1077) and
``DenseNearestNeighborList`` (:902-982).  Both classes return the same edge
set (the reference's shared test suite holds them to that); here both run the
``kups_neighborlist_build`` CUDA kernel.  Capacities follow
``UniversalNeighborlistParameters`` (:1353-1417): ``avg_edges`` edges per
particle; an overflow raises ``CapacityError`` carrying the required size,
and ``fix`` grows the capacity to the next power of two as ``LensCapacity``
does (src/kups/core/capacity.py:135-240).
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, replace
from typing import NamedTuple

import torch

from . import _lib
from .unitcell import as_tril


@dataclass
class Edges:
    """Directed edges (i = lh, j = rh) padded with the out-of-bounds index N.

    indices: int32 [capacity, 2];  shifts: int32 [capacity, 1, 3];
    n_edges: number of valid leading rows.
    """

    indices: torch.Tensor
    shifts: torch.Tensor
    n_edges: int

    def valid(self) -> tuple[torch.Tensor, torch.Tensor]:
        return self.indices[: self.n_edges], self.shifts[: self.n_edges, 0]

    def difference_vectors(self, positions: torch.Tensor, system: torch.Tensor, tril: torch.Tensor):
        """x_j - x_i + s @ L (neighborlist.py:164-184)."""
        idx, sh = self.valid()
        i, j = idx[:, 0].long(), idx[:, 1].long()
        t = tril[system[i].long()]
        s = sh.to(t.dtype)
        sl = torch.stack(
            [s[:, 0] * t[:, 0] + s[:, 1] * t[:, 1] + s[:, 2] * t[:, 3], s[:, 1] * t[:, 2] + s[:, 2] * t[:, 4], s[:, 2] * t[:, 5]],
            -1,
        )
        return positions[j] - positions[i] + sl


@dataclass
class NeighborListPoints:
    """Particle columns a neighbour list reads (``NeighborListPoints``, :217-223)."""

    positions: torch.Tensor  # f64 [N, 3]
    system: torch.Tensor  # int [N]; values outside [0, S) are empty slots
    inclusion: torch.Tensor | None = None  # int [N], defaults to system
    exclusion: torch.Tensor | None = None  # int [N], defaults to arange(N)
    n_inclusion: int | None = None


def _i32(x: torch.Tensor) -> torch.Tensor:
    return x.to(device="cuda", dtype=torch.int32).contiguous()


def _f64(x: torch.Tensor) -> torch.Tensor:
    return x.to(device="cuda", dtype=torch.float64).contiguous()


def _stream() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclass
class CellListNeighborList:
    """GPU cell-list neighbour list; ``avg_edges`` = edge slots per particle."""

    avg_edges: int = 64

    def __call__(self, lh: NeighborListPoints, rh: NeighborListPoints | None = None, systems=None, cutoffs=None,
                 rh_index_remap=None) -> Edges:
        if rh is not None:
            return self._call_rh(lh, rh, systems, cutoffs, rh_index_remap)
        if rh_index_remap is not None:
            raise ValueError("rh_index_remap needs an rh table")
        lib = _lib.load()
        pos = _f64(lh.positions)
        n = pos.shape[0]
        system = _i32(lh.system)
        incl = _i32(lh.inclusion) if lh.inclusion is not None else system
        excl = _i32(lh.exclusion) if lh.exclusion is not None else torch.arange(n, device="cuda", dtype=torch.int32)
        tril = _f64(as_tril(systems))
        s = tril.shape[0]
        n_incl = lh.n_inclusion if lh.n_inclusion is not None else s
        cut = _f64(torch.as_tensor(cutoffs, dtype=torch.float64).reshape(-1).expand(s))
        cap = max(1, self.avg_edges * n)
        edges = torch.empty((cap, 2), device="cuda", dtype=torch.int32)
        shifts = torch.empty((cap, 3), device="cuda", dtype=torch.int32)
        n_edges = torch.zeros(1, device="cuda", dtype=torch.int64)
        ws_bytes = lib.kups_neighborlist_workspace_bytes(n, s)
        ws = torch.empty(ws_bytes, device="cuda", dtype=torch.uint8)
        status = new_status()
        rc = lib.kups_neighborlist_build(
            pos.data_ptr(), system.data_ptr(), incl.data_ptr(), excl.data_ptr(), n, n_incl, tril.data_ptr(),
            cut.data_ptr(), s, edges.data_ptr(), shifts.data_ptr(), cap, n_edges.data_ptr(), ws.data_ptr(),
            ws_bytes, status.data_ptr(), _stream(),
        )
        _lib.check(rc, "kups_neighborlist_build")
        st = read_status(status)
        _lib.raise_status(st)
        return Edges(edges, shifts.view(cap, 1, 3), int(n_edges.item()))

    def _call_rh(self, lh: NeighborListPoints, rh: NeighborListPoints, systems, cutoffs, rh_index_remap) -> Edges:
        """Edges (i in lh, j in rh) (kups_neighborlist_build_rh); with ``rh_index_remap`` the
        rh particles stand for lh particles and the edges come in both directions."""
        lib = _lib.load()
        lp = _f64(lh.positions)
        rp = _f64(rh.positions)
        n_lh, n_rh = lp.shape[0], rp.shape[0]
        lsys, rsys = _i32(lh.system), _i32(rh.system)
        lincl = _i32(lh.inclusion) if lh.inclusion is not None else lsys
        rincl = _i32(rh.inclusion) if rh.inclusion is not None else rsys
        lexcl = _i32(lh.exclusion) if lh.exclusion is not None else torch.arange(n_lh, device="cuda",
                                                                                   dtype=torch.int32)
        remap = _i32(torch.as_tensor(rh_index_remap)) if rh_index_remap is not None else None
        if rh.exclusion is not None:
            rexcl = _i32(rh.exclusion)
        elif remap is not None:
            rexcl = remap  # an rh particle standing for lh particle r shares r's label
        else:
            rexcl = torch.arange(n_lh, n_lh + n_rh, device="cuda", dtype=torch.int32)
        tril = _f64(as_tril(systems))
        s = tril.shape[0]
        n_incl = lh.n_inclusion if lh.n_inclusion is not None else s
        cut = _f64(torch.as_tensor(cutoffs, dtype=torch.float64).reshape(-1).expand(s))
        cap = max(1, self.avg_edges * max(n_rh, 1) * (2 if remap is not None else 1))
        edges = torch.empty((cap, 2), device="cuda", dtype=torch.int32)
        shifts = torch.empty((cap, 3), device="cuda", dtype=torch.int32)
        n_edges = torch.zeros(1, device="cuda", dtype=torch.int64)
        ws_bytes = lib.kups_neighborlist_rh_workspace_bytes(n_lh, n_rh, s)
        ws = torch.empty(ws_bytes, device="cuda", dtype=torch.uint8)
        status = new_status()
        rc = lib.kups_neighborlist_build_rh(
            lp.data_ptr(), lsys.data_ptr(), lincl.data_ptr(), lexcl.data_ptr(), n_lh, rp.data_ptr(), rsys.data_ptr(),
            rincl.data_ptr(), rexcl.data_ptr(), n_rh, remap.data_ptr() if remap is not None else None, n_incl,
            tril.data_ptr(), cut.data_ptr(), s, edges.data_ptr(), shifts.data_ptr(), cap, n_edges.data_ptr(),
            ws.data_ptr(), ws_bytes, status.data_ptr(), _stream())
        _lib.check(rc, "kups_neighborlist_build_rh")
        _lib.raise_status(read_status(status))
        return Edges(edges, shifts.view(cap, 1, 3), int(n_edges.item()))

    def fix(self, err: _lib.CapacityError, n_particles: int) -> "CellListNeighborList":
        per = err.required / max(1, n_particles)
        return replace(self, avg_edges=int(2 ** math.ceil(math.log2(max(per, 1.0)))))

    def call_and_fix(self, lh, rh=None, systems=None, cutoffs=None, rh_index_remap=None, max_tries=8):
        """Grow-and-retry loop of propagate_and_fix (src/kups/core/propagator.py:137-172)."""
        nl = self
        per = lh.positions.shape[0] if rh is None else max(1, rh.positions.shape[0]) * (
            2 if rh_index_remap is not None else 1)
        for _ in range(max_tries):
            try:
                return nl(lh, rh, systems, cutoffs, rh_index_remap), nl
            except _lib.CapacityError as err:
                nl = nl.fix(err, per)
        raise _lib.KupsError("neighbour list capacity did not converge")


class DenseNearestNeighborList(CellListNeighborList):
    """Same edge set as the cell list (neighborlist.py:902-982)."""


class NeighborListChangesResult(NamedTuple):
    added: Edges
    removed: Edges


def neighborlist_changes(neighborlist: CellListNeighborList, lh: NeighborListPoints, rh_indices,
                         rh: NeighborListPoints, systems, cutoffs, compaction: float = 0.5) -> NeighborListChangesResult:
    """Edges removed and added when the particles ``rh_indices`` of ``lh`` take the data ``rh``
    (``neighborlist_changes``, src/kups/core/neighborlist.py:1425-1515): one rh call with
    lh = originals followed by the proposed particles and rh = the changed particles' old
    copies followed by the proposed ones (remap = [rh_indices, N + arange(k)]), then the split
    of ``kups_neighborlist_split_changes``.  Each output holds ``compaction`` of the combined
    call's rows (all of them for compaction >= 1), padded with N."""
    lib = _lib.load()
    p_idx = _i32(torch.as_tensor(rh_indices))
    n, k = lh.positions.shape[0], p_idx.shape[0]
    pl = p_idx.long()
    lsys = _i32(lh.system)
    lincl = _i32(lh.inclusion) if lh.inclusion is not None else lsys
    lexcl = _i32(lh.exclusion) if lh.exclusion is not None else torch.arange(n, device="cuda", dtype=torch.int32)
    rsys = _i32(rh.system) if rh.system is not None else lsys[pl]
    rincl = _i32(rh.inclusion) if rh.inclusion is not None else rsys
    rexcl = _i32(rh.exclusion) if rh.exclusion is not None else lexcl[pl]
    lh_c = NeighborListPoints(torch.cat([_f64(lh.positions), _f64(rh.positions)]), torch.cat([lsys, rsys]),
                              torch.cat([lincl, rincl]), torch.cat([lexcl, rexcl]), lh.n_inclusion)
    rh_c = NeighborListPoints(torch.cat([_f64(lh.positions)[pl], _f64(rh.positions)]), torch.cat([lsys[pl], rsys]),
                              torch.cat([lincl[pl], rincl]), torch.cat([lexcl[pl], rexcl]))
    remap = torch.cat([p_idx, torch.arange(n, n + k, device="cuda", dtype=torch.int32)])
    edges, _ = neighborlist.call_and_fix(lh_c, rh_c, systems, cutoffs, remap)
    rows = edges.indices.shape[0]
    cap = rows if compaction >= 1.0 else max(1, int(rows * compaction))
    out = []
    for _ in range(4):
        ae = torch.empty((cap, 2), device="cuda", dtype=torch.int32)
        as_ = torch.empty((cap, 3), device="cuda", dtype=torch.int32)
        re = torch.empty((cap, 2), device="cuda", dtype=torch.int32)
        rs = torch.empty((cap, 3), device="cuda", dtype=torch.int32)
        na = torch.zeros(1, device="cuda", dtype=torch.int64)
        nr = torch.zeros(1, device="cuda", dtype=torch.int64)
        n_e = torch.tensor([edges.n_edges], device="cuda", dtype=torch.int64)
        ws_bytes = lib.kups_neighborlist_split_workspace_bytes(rows, n)
        ws = torch.empty(ws_bytes, device="cuda", dtype=torch.uint8)
        status = new_status()
        rc = lib.kups_neighborlist_split_changes(
            edges.indices.data_ptr(), edges.shifts.data_ptr(), n_e.data_ptr(), rows, n, p_idx.data_ptr(), k,
            ae.data_ptr(), as_.data_ptr(), cap, na.data_ptr(), re.data_ptr(), rs.data_ptr(), cap, nr.data_ptr(),
            ws.data_ptr(), ws_bytes, status.data_ptr(), _stream())
        _lib.check(rc, "kups_neighborlist_split_changes")
        st = read_status(status)
        if st.code == _lib.KUPS_ERR_CAPACITY and cap < rows:
            cap = min(rows, max(cap * 2, int(st.required)))  # the reference's capacity assertion, grown
            continue
        _lib.raise_status(st)
        out = [Edges(ae, as_.view(cap, 1, 3), int(na.item())), Edges(re, rs.view(cap, 1, 3), int(nr.item()))]
        break
    if not out:
        raise _lib.KupsError("neighborlist_changes capacity did not converge")
    return NeighborListChangesResult(*out)


def read_status(status: torch.Tensor) -> _lib.Status:
    """Copy a device status word (int64[4]: code|detail, required, first_bad) to the host."""
    h = status.cpu()
    raw = int(h[0])
    code = raw & 0xFFFFFFFF
    detail = (raw >> 32) & 0xFFFFFFFF
    return _lib.Status(code, detail, int(h[1]), int(h[2]))


def new_status(device="cuda") -> torch.Tensor:
    """Zeroed status word (kups_status is 24 bytes: i32, i32, i64, i64)."""
    st = torch.zeros(3, device=device, dtype=torch.int64)
    st[2:].fill_(-1)  # a device fill, safe inside CUDA-graph capture
    return st


def estimate_avg_edges(n_particles: int, volume: float, cutoff: float, multiplier: float = 1.0) -> int:
    """Neighbours within the cutoff at uniform density, rounded up to a power of 2
    (``_estimate_avg_num_edges``, neighborlist.py:789-817)."""
    est = multiplier * 4.0 / 3.0 * math.pi * cutoff**3 * n_particles / volume
    return int(2 ** math.ceil(math.log2(max(est, 1.0))))
