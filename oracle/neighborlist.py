"""Reference-exact periodic neighbour list in float64 (oracle, test infrastructure).

Restates the edge SET produced by src/kups/core/neighborlist.py
``basic_neighborlist`` (:743-786) for both ``DenseNearestNeighborList``
(:902-982) and ``CellListNeighborList`` (:985-1077); the two differ only in
candidate order, which the reference's own shared test suite
(test/core/test_neighborlist.py:191-296) already treats as irrelevant.

Semantics restated, per system s with cutoff rc and lattice L:

* fractional coordinates f = r @ L^-1 (``basic_neighborlist`` :766-777), not wrapped;
* images per axis n_a = ceil(2 rc / w_a), made odd, 1 for an infinite cutoff
  (``_get_candidate_images`` :461-466);
* if prod(n_a) == 1: shift s = round(f_i - f_j), candidate delta
  f_i - f_j - s (``_compute_distances_pbc_sq`` :542-564);
* else every offset o of the centred n_x x n_y x n_z grid is tried, delta
  f_i - f_j - o; the minimum-image flag is (o == round(f_i - f_j))
  (``_apply_distance_cutoff_w_images`` :595-624).  Axes with n_a == 1 use
  offset 0 on that axis, exactly as the reference does;
* d^2 = |delta @ L|^2 < rc^2 strictly, same system, same valid inclusion
  segment (``_build_segmentation_mask`` :505-539);
* exclusion: dropped when excl_i == excl_j on the minimum image only
  (:731-735);
* edges are directed (i = lh, j = rh) with the integer shift s; the
  difference vector is x_j - x_i + s @ L (``Edges.difference_vectors`` :164-184).
"""

from __future__ import annotations

import numpy as np

from .unitcell import inverse_tril, perpendicular_lengths, row_times_tril


def image_counts(tril: np.ndarray, cutoffs: np.ndarray) -> np.ndarray:
    """Odd number of periodic images per axis and system (neighborlist.py:461-466)."""
    w = perpendicular_lengths(tril)
    rc = np.asarray(cutoffs, dtype=np.float64)[..., None]
    with np.errstate(invalid="ignore", over="ignore"):
        n = np.ceil(2 * rc / w)
    n = np.where(np.isfinite(rc), n, 1).astype(np.int64)
    n = n + (n % 2 == 0)
    return n


def image_offsets(n: np.ndarray) -> np.ndarray:
    """Centred integer offsets of an n0 x n1 x n2 grid (any order; sets only)."""
    h = (np.asarray(n) - 1) // 2
    g = np.stack(
        np.meshgrid(
            np.arange(-h[0], h[0] + 1),
            np.arange(-h[1], h[1] + 1),
            np.arange(-h[2], h[2] + 1),
            indexing="ij",
        ),
        axis=-1,
    ).reshape(-1, 3)
    return g


def neighbor_list(
    positions: np.ndarray,
    system: np.ndarray,
    tril: np.ndarray,
    cutoffs: np.ndarray,
    inclusion: np.ndarray | None = None,
    exclusion: np.ndarray | None = None,
    n_inclusion: int | None = None,
):
    """Directed edge list (i, j) with integer shifts, sorted lexicographically.

    Args:
        positions: float64 [N, 3] Cartesian.
        system: int [N]; values >= n_systems mark empty slots.
        tril: float64 [S, 6].
        cutoffs: float64 [S].
        inclusion: int [N]; defaults to ``system``.  Values outside
            [0, n_inclusion) are invalid (no edges).
        exclusion: int [N]; defaults to arange(N).
        n_inclusion: number of inclusion labels (defaults to S).

    Returns:
        (edges int64 [E, 2], shifts int64 [E, 3]).
    """
    pos = np.asarray(positions, dtype=np.float64)
    sysi = np.asarray(system, dtype=np.int64)
    tril = np.asarray(tril, dtype=np.float64).reshape(-1, 6)
    cut = np.broadcast_to(np.asarray(cutoffs, dtype=np.float64), (tril.shape[0],))
    S = tril.shape[0]
    N = pos.shape[0]
    incl = sysi if inclusion is None else np.asarray(inclusion, dtype=np.int64)
    excl = np.arange(N) if exclusion is None else np.asarray(exclusion, dtype=np.int64)
    n_incl = S if n_inclusion is None else int(n_inclusion)

    inv = inverse_tril(tril)
    nimg = image_counts(tril, cut)
    all_e, all_s = [], []
    for s in range(S):
        idx = np.nonzero(sysi == s)[0]
        if idx.size == 0:
            continue
        f = row_times_tril(pos[idx], inv[s])
        inc = incl[idx]
        rc2 = cut[s] ** 2
        if np.prod(nimg[s]) == 1:
            # rows in blocks, so large systems stay within a few hundred MB
            blk = max(1, 2**22 // max(1, idx.size))
            for r0 in range(0, idx.size, blk):
                r = slice(r0, r0 + blk)
                d0 = f[r, None, :] - f[None, :, :]
                seg = (inc[r, None] == inc[None, :]) & (inc[r, None] >= 0) & (inc[r, None] < n_incl)
                same_ex = excl[idx][r, None] == excl[idx][None, :]
                min_shift = np.round(d0)
                delta = d0 - min_shift
                real = row_times_tril(delta, tril[s])
                d2 = (real[..., 0] * real[..., 0] + real[..., 1] * real[..., 1]) + real[..., 2] * real[..., 2]
                m = seg & (d2 < rc2) & ~same_ex
                ii, jj = np.nonzero(m)
                all_e.append(np.stack([idx[r0 + ii], idx[jj]], -1))
                all_s.append(min_shift[ii, jj].astype(np.int64))
            continue
        d0 = f[:, None, :] - f[None, :, :]  # lh - rh
        seg = (inc[:, None] == inc[None, :]) & (inc[:, None] >= 0) & (inc[:, None] < n_incl)
        same_ex = excl[idx][:, None] == excl[idx][None, :]
        min_shift = np.round(d0)
        for o in image_offsets(nimg[s]):
            delta = d0 - o
            real = row_times_tril(delta, tril[s])
            d2 = (real[..., 0] * real[..., 0] + real[..., 1] * real[..., 1]) + real[..., 2] * real[..., 2]
            is_min = np.all(min_shift == o, axis=-1)
            m = seg & (d2 < rc2) & (~same_ex | ~is_min)
            ii, jj = np.nonzero(m)
            all_e.append(np.stack([idx[ii], idx[jj]], -1))
            all_s.append(np.broadcast_to(o, (ii.size, 3)).astype(np.int64))
    if not all_e:
        return np.zeros((0, 2), np.int64), np.zeros((0, 3), np.int64)
    e = np.concatenate(all_e).astype(np.int64)
    sh = np.concatenate(all_s).astype(np.int64)
    return sort_edges(e, sh)


def sort_edges(edges: np.ndarray, shifts: np.ndarray):
    """Lexicographic (i, j, sx, sy, sz) order: the canonical set representation."""
    edges = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    shifts = np.asarray(shifts, dtype=np.int64).reshape(-1, 3)
    order = np.lexsort((shifts[:, 2], shifts[:, 1], shifts[:, 0], edges[:, 1], edges[:, 0]))
    return edges[order], shifts[order]


def difference_vectors(positions, system, tril, edges, shifts) -> np.ndarray:
    """x_j - x_i + s @ L (neighborlist.py:164-184), L of the lh particle's system."""
    pos = np.asarray(positions, dtype=np.float64)
    tril = np.asarray(tril, dtype=np.float64).reshape(-1, 6)
    i, j = edges[:, 0], edges[:, 1]
    t = tril[np.asarray(system)[i]]
    return pos[j] - pos[i] + row_times_tril(np.asarray(shifts, dtype=np.float64), t)


def neighbor_list_rh(lh_positions, lh_system, rh_positions, rh_system, tril, cutoffs, lh_inclusion=None,
                     rh_inclusion=None, lh_exclusion=None, rh_exclusion=None, rh_index_remap=None, n_inclusion=None):
    """Edges between a left-hand table and a separate right-hand table (float64, sorted).

    Restates basic_neighborlist with rh given (src/kups/core/neighborlist.py:743-786):
    candidate pairs (i in lh, j in rh) of the same system and the same valid inclusion
    label (``_build_segmentation_mask`` :505-539), the image rule of ``neighbor_list`` on
    the difference f_i - f_j, the exclusion label compared between lh and rh dropping only
    the minimum image (:731-735).  With ``rh_index_remap`` (rh particle j stands for lh
    particle remap[j]) a pair whose lh particle is itself remapped is kept only for
    i >= remap[j], and every edge (i, remap[j], s) comes with (remap[j], i, -s)
    (``_compact_edges`` :651-689); without it the edges are (i, j), j indexing rh.
    """
    lp = np.asarray(lh_positions, np.float64).reshape(-1, 3)
    rp = np.asarray(rh_positions, np.float64).reshape(-1, 3)
    ls, rs = np.asarray(lh_system, np.int64), np.asarray(rh_system, np.int64)
    tril = np.asarray(tril, np.float64).reshape(-1, 6)
    S = tril.shape[0]
    cut = np.broadcast_to(np.asarray(cutoffs, np.float64), (S,))
    li = ls if lh_inclusion is None else np.asarray(lh_inclusion, np.int64)
    ri = rs if rh_inclusion is None else np.asarray(rh_inclusion, np.int64)
    le = np.arange(len(lp)) if lh_exclusion is None else np.asarray(lh_exclusion, np.int64)
    remap = None if rh_index_remap is None else np.asarray(rh_index_remap, np.int64)
    re = (remap if remap is not None else np.arange(len(rp)) + len(lp)) if rh_exclusion is None else np.asarray(
        rh_exclusion, np.int64)
    n_incl = S if n_inclusion is None else int(n_inclusion)
    in_remap = np.zeros(len(lp), bool)
    if remap is not None:
        ok = (remap >= 0) & (remap < len(lp))
        in_remap[remap[ok]] = True
    inv = inverse_tril(tril)
    nimg = image_counts(tril, cut)
    out_e, out_s = [], []
    for s in range(S):
        ia = np.nonzero(ls == s)[0]
        ja = np.nonzero(rs == s)[0]
        if ia.size == 0 or ja.size == 0:
            continue
        fi = row_times_tril(lp[ia], inv[s])
        fj = row_times_tril(rp[ja], inv[s])
        d0 = fi[:, None, :] - fj[None, :, :]
        seg = (li[ia][:, None] == ri[ja][None, :]) & (li[ia][:, None] >= 0) & (li[ia][:, None] < n_incl)
        seg &= (ri[ja][None, :] >= 0) & (ri[ja][None, :] < n_incl)
        if remap is not None:
            seg &= ~in_remap[ia][:, None] | (ia[:, None] >= remap[ja][None, :])
        same_ex = le[ia][:, None] == re[ja][None, :]
        rc2 = cut[s] ** 2
        min_shift = np.round(d0)
        offsets = [None] if np.prod(nimg[s]) == 1 else list(image_offsets(nimg[s]))
        for o in offsets:
            sh = min_shift if o is None else np.broadcast_to(o, d0.shape)
            delta = d0 - sh
            real = row_times_tril(delta, tril[s])
            d2 = (real[..., 0] * real[..., 0] + real[..., 1] * real[..., 1]) + real[..., 2] * real[..., 2]
            is_min = np.ones(d0.shape[:2], bool) if o is None else np.all(min_shift == o, axis=-1)
            m = seg & (d2 < rc2) & (~same_ex | ~is_min)
            a, b = np.nonzero(m)
            i, j = ia[a], ja[b]
            shv = sh[a, b].astype(np.int64)
            if remap is None:
                out_e.append(np.stack([i, j], -1))
                out_s.append(shv)
            else:
                out_e += [np.stack([i, remap[j]], -1), np.stack([remap[j], i], -1)]
                out_s += [shv, -shv]
    if not out_e:
        return np.zeros((0, 2), np.int64), np.zeros((0, 3), np.int64)
    return sort_edges(np.concatenate(out_e), np.concatenate(out_s))


def neighborlist_changes(positions, system, changed, new_positions, tril, cutoffs, inclusion=None, exclusion=None):
    """(added, removed) edge sets of moving particles ``changed`` to ``new_positions``
    (``neighborlist_changes``, src/kups/core/neighborlist.py:1425-1515): one rh call with lh =
    originals + proposed and rh = old copies + proposed (remap = [changed, n + arange(k)]), then
    removed = edges between original indices, added = edges touching a proposed particle and no
    old copy, proposed indices rewritten to the particles they replace."""
    pos = np.asarray(positions, np.float64).reshape(-1, 3)
    n = len(pos)
    sysi = np.asarray(system, np.int64)
    incl = sysi if inclusion is None else np.asarray(inclusion, np.int64)
    excl = np.arange(n) if exclusion is None else np.asarray(exclusion, np.int64)
    p = np.asarray(changed, np.int64)
    k = len(p)
    new = np.asarray(new_positions, np.float64).reshape(-1, 3)
    lh_pos = np.concatenate([pos, new])
    lh_sys = np.concatenate([sysi, sysi[p]])
    lh_incl = np.concatenate([incl, incl[p]])
    lh_excl = np.concatenate([excl, excl[p]])
    rh_pos = np.concatenate([pos[p], new])
    remap = np.concatenate([p, n + np.arange(k)])
    e, s = neighbor_list_rh(lh_pos, lh_sys, rh_pos, np.concatenate([sysi[p], sysi[p]]), tril, cutoffs,
                            lh_inclusion=lh_incl, rh_inclusion=np.concatenate([incl[p], incl[p]]),
                            lh_exclusion=lh_excl, rh_exclusion=np.concatenate([excl[p], excl[p]]),
                            rh_index_remap=remap)
    c0, c1 = e[:, 0], e[:, 1]
    removed = (c0 < n) & (c1 < n)
    changed_mask = np.zeros(n, bool)
    changed_mask[p] = True
    stale = ((c0 < n) & changed_mask[np.minimum(c0, n - 1)]) | ((c1 < n) & changed_mask[np.minimum(c1, n - 1)])
    added = (c0 < n + k) & (c1 < n + k) & ((c0 >= n) | (c1 >= n)) & ~stale
    re = np.where(e >= n, p[np.clip(e - n, 0, max(k - 1, 0))], e)
    return sort_edges(re[added], s[added]), sort_edges(re[removed], s[removed])
