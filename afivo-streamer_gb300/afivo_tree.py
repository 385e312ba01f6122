"""Quadtree/octree box lists with afivo's conventions (the host-side ``af_t``).

This module builds the tree tables that a Fortran caller holds in ``af_t``
(``afivo/src/m_af_types.f90:286-393``): 1-based box ids, ``parent``,
``children`` in ``af_child_dix`` order, ``neighbors`` in the order
lowx, highx, lowy, highy(, lowz, highz), ``neighbor_mat(-1:1, -1:1[, -1:1])``
with the first index fastest, ``ix``, ``lvl``, ``r_min`` and ``dr``, plus the
per-level ``ids``/``leaves``/``parents`` lists of ``lvl_t``
(``m_af_types.f90:76-80``).  Special ids follow ``m_af_types.f90:38-41``:
``0`` = no box (refinement boundary), ``-1`` = physical boundary.

It stands in for afivo's own tree construction (``af_init`` /
``af_set_coarse_grid`` / ``af_adjust_refinement``, ``m_af_core.f90:138-340,
697-822``), which stays on the host and is outside the GPU path: trees are
built from a refinement predicate per level and then made 2:1 balanced
(neighbours, diagonal ones included, differ by at most one level), the
property afivo's refinement guarantees.  Floating-point geometry (``r_min``,
``dr``) is computed with the same operation order as ``m_af_core.f90:166,
255-256,1210-1213`` so that coordinates agree bit for bit.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np

AF_NO_BOX = 0
AF_PHYS_BOUNDARY = -1
AF_XYZ = 1
AF_CYL = 2


def child_dix(ndim: int) -> np.ndarray:
    """``af_child_dix`` (m_af_types.f90:131,169-171): child n has offsets
    given by the binary digits of n-1, x fastest."""
    return np.array([[(n >> d) & 1 for d in range(ndim)]
                     for n in range(2 ** ndim)], dtype=np.int64)


def neighb_dix(ndim: int) -> np.ndarray:
    """``af_neighb_dix`` (m_af_types.f90:149,186-187)."""
    out = []
    for d in range(ndim):
        for s in (-1, 1):
            v = [0] * ndim
            v[d] = s
            out.append(v)
    return np.array(out, dtype=np.int64)


def nbmat_offsets(ndim: int) -> np.ndarray:
    """Offsets of ``neighbor_mat`` entries in Fortran (first index fastest)
    order."""
    rng = [-1, 0, 1]
    offs = []
    for t in itertools.product(rng, repeat=ndim):
        offs.append(t[::-1])
    return np.array(offs, dtype=np.int64)


@dataclass
class Tree:
    ndim: int
    n_cell: int
    coord: int
    coarse_grid_size: np.ndarray
    r_base: np.ndarray
    dr_base: np.ndarray
    n_boxes: int = 0
    highest_lvl: int = 0
    lvl: np.ndarray = None            # [n]
    ix: np.ndarray = None             # [n, D]  (1-based like Fortran)
    parent: np.ndarray = None         # [n]
    children: np.ndarray = None       # [n, 2^D]
    neighbors: np.ndarray = None      # [n, 2D]
    neighbor_mat: np.ndarray = None   # [n, 3^D]
    r_min: np.ndarray = None          # [n, D]
    dr: np.ndarray = None             # [n, D]
    lvl_ids: list = field(default_factory=list)      # per level, 1-based ids
    lvl_leaves: list = field(default_factory=list)
    lvl_parents: list = field(default_factory=list)

    @property
    def box_cells(self) -> int:
        return (self.n_cell + 2) ** self.ndim

    def n_cells(self, leaves_only: bool = False) -> int:
        lists = self.lvl_leaves if leaves_only else self.lvl_ids
        return sum(len(x) for x in lists) * self.n_cell ** self.ndim

    def level_cells(self, lvl: int) -> int:
        return len(self.lvl_ids[lvl - 1]) * self.n_cell ** self.ndim

    def flat_lists(self):
        """Concatenated level lists with offsets (the layout of the C-ABI
        tree description)."""
        def cat(lists):
            offs = np.zeros(len(lists) + 1, dtype=np.int32)
            for i, l in enumerate(lists):
                offs[i + 1] = offs[i] + len(l)
            data = (np.concatenate(lists).astype(np.int32) if offs[-1] > 0
                    else np.zeros(1, dtype=np.int32))
            return offs, data
        return cat(self.lvl_ids), cat(self.lvl_leaves), cat(self.lvl_parents)

    def cell_centers(self, ids: np.ndarray) -> np.ndarray:
        """Cell-centre coordinates ``af_r_cc`` (m_af_types.f90:1035-1040)
        for interior cells of boxes ``ids``: shape [len(ids), D, nc, ...]
        in C order (slowest index last dim), i.e. [b, d, (k,) j, i]."""
        nc, D = self.n_cell, self.ndim
        idx = np.arange(1, nc + 1, dtype=np.float64) - 0.5
        out = np.empty((len(ids), D) + (nc,) * D)
        for d in range(D):
            shape = [1] * D
            shape[D - 1 - d] = nc
            r = (self.r_min[ids - 1, d][:, None] +
                 idx[None, :] * self.dr[ids - 1, d][:, None])
            out[:, d] = r.reshape((len(ids),) + tuple(shape))
        return out


def _keys(ix: np.ndarray, n: np.ndarray) -> np.ndarray:
    """Linear keys of 0-based box indices (x fastest), one level."""
    k = np.zeros(len(ix), dtype=np.int64)
    for d in range(ix.shape[1] - 1, -1, -1):
        k = k * int(n[d]) + ix[:, d]
    return k


def _unkey(k: np.ndarray, n: np.ndarray, D: int) -> np.ndarray:
    out = np.empty((len(k), D), dtype=np.int64)
    for d in range(D):
        out[:, d] = k % int(n[d])
        k = k // int(n[d])
    return out


def _lookup(keys_sorted: np.ndarray, q: np.ndarray) -> np.ndarray:
    """Index of q in keys_sorted, -1 where absent."""
    pos = np.searchsorted(keys_sorted, q)
    pos = np.minimum(pos, max(len(keys_sorted) - 1, 0))
    found = (len(keys_sorted) > 0) & (keys_sorted[pos] == q) if len(keys_sorted) else np.zeros(len(q), bool)
    return np.where(found, pos, -1)


def build_tree(ndim: int, n_cell: int, coarse_grid_size, domain_len,
               r_base=None, coord: int = AF_XYZ, max_lvl: int = 1,
               refine=None, face_balance: bool = False) -> Tree:
    """Build a 2:1-balanced tree: by default every refined box has its whole
    3^D neighbourhood on its own level (diagonal neighbours included, the
    seeded benchmark trees); with ``face_balance`` only its face neighbours,
    which is afivo's rule (ensure_two_one_balance, m_af_core.f90:1015-1055).

    ``refine(lvl, centers[m, D], dr[D]) -> bool[m]`` says which boxes of
    level ``lvl`` (given by their centres) want children; ``None`` refines
    everything (uniform grid).  Level 1 is the coarse grid of
    ``coarse_grid_size`` cells, split into boxes like ``af_set_coarse_grid``
    (m_af_core.f90:206-340).  Boxes are kept as sorted index keys per level,
    so deep 3D trees cost memory proportional to the number of boxes.
    """
    D = ndim
    nc = n_cell
    cgs = np.asarray(coarse_grid_size, dtype=np.int64).reshape(D)
    if np.any(cgs % nc):
        raise ValueError("coarse_grid_size must be divisible by n_cell")
    dom = np.asarray(domain_len, dtype=np.float64).reshape(D)
    rb = (np.zeros(D) if r_base is None
          else np.asarray(r_base, dtype=np.float64).reshape(D))
    # af_init: dr_base = (r_max - r_min) / grid_size, r_max = r_min + L
    dr_base = ((rb + dom) - rb) / cgs
    nx1 = cgs // nc
    nlev = [nx1 * 2 ** l for l in range(max_lvl)]

    def lvl_dr(l):
        d = dr_base.copy()
        for _ in range(l):
            d = 0.5 * d
        return d

    cdix = child_dix(D)
    all1 = np.stack(np.meshgrid(*[np.arange(int(n)) for n in nx1], indexing="ij"), -1).reshape(-1, D)
    exists = [np.sort(_keys(all1, nlev[0]))]
    refined = [np.zeros(0, np.int64) for _ in range(max_lvl)]
    for l in range(max_lvl - 1):
        ix = _unkey(exists[l], nlev[l], D)
        if len(ix) == 0:
            break
        if refine is None:
            want = np.ones(len(ix), dtype=bool)
        else:
            drl = lvl_dr(l)
            centers = rb + (ix + 0.5) * drl * nc
            want = np.asarray(refine(l + 1, centers, drl), dtype=bool)
        refined[l] = exists[l][want]
        cix = (2 * ix[want][:, None, :] + cdix[None, :, :]).reshape(-1, D)
        exists.append(np.sort(_keys(cix, nlev[l + 1])))
    # 2:1 balance, fine to coarse: a refined box needs its whole 3^D
    # neighbourhood on its own level; the parents of newly refined boxes are
    # handled by the next, coarser pass through the dilation of refined[l-1]
    offs = np.array(list(itertools.product([-1, 0, 1], repeat=D)), dtype=np.int64)
    if face_balance:
        offs = offs[np.abs(offs).sum(axis=1) <= 1]
    for l in range(max_lvl - 2, 0, -1):
        if len(refined[l]) == 0:
            continue
        ix = _unkey(refined[l], nlev[l], D)
        nbh = (ix[:, None, :] + offs[None, :, :]).reshape(-1, D)
        ok = np.all((nbh >= 0) & (nbh < nlev[l][None, :]), axis=1)
        par = np.unique(_keys(nbh[ok] // 2, nlev[l - 1]))
        refined[l - 1] = np.union1d(refined[l - 1], par)
    exists = exists[:1]
    for l in range(max_lvl - 1):
        if len(refined[l]) == 0:
            break
        ix = _unkey(refined[l], nlev[l], D)
        cix = (2 * ix[:, None, :] + cdix[None, :, :]).reshape(-1, D)
        exists.append(np.sort(_keys(cix, nlev[l + 1])))
    highest = len(exists)

    # ids: level 1 in Fortran order (x fastest), then children of each
    # refined parent in parent-id order, child order af_child_dix
    lvl_ids, ix_of, key_of = [], [], []
    ix1 = _unkey(exists[0], nlev[0], D)
    lvl_ids.append(np.arange(1, len(ix1) + 1, dtype=np.int64))
    ix_of.append(ix1)
    key_of.append(exists[0])
    next_id = len(ix1) + 1
    for l in range(1, highest):
        pkeys = key_of[l - 1]
        is_ref = np.isin(pkeys, refined[l - 1])
        pix = ix_of[l - 1][is_ref]
        cix = (2 * pix[:, None, :] + cdix[None, :, :]).reshape(-1, D)
        cids = next_id + np.arange(len(cix), dtype=np.int64)
        next_id += len(cix)
        lvl_ids.append(cids)
        ix_of.append(cix)
        key_of.append(_keys(cix, nlev[l]))
    n_boxes = next_id - 1

    t = Tree(ndim=D, n_cell=nc, coord=coord, coarse_grid_size=cgs,
             r_base=rb, dr_base=dr_base)
    t.n_boxes = n_boxes
    t.highest_lvl = highest
    t.lvl = np.zeros(n_boxes, dtype=np.int32)
    t.ix = np.zeros((n_boxes, D), dtype=np.int32)
    t.parent = np.zeros(n_boxes, dtype=np.int32)
    t.children = np.zeros((n_boxes, 2 ** D), dtype=np.int32)
    t.neighbors = np.zeros((n_boxes, 2 * D), dtype=np.int32)
    t.neighbor_mat = np.zeros((n_boxes, 3 ** D), dtype=np.int32)
    t.r_min = np.zeros((n_boxes, D))
    t.dr = np.zeros((n_boxes, D))
    nbd = neighb_dix(D)
    nmo = nbmat_offsets(D)

    for l in range(highest):
        ids = lvl_ids[l]
        ixl = ix_of[l]
        rows = ids - 1
        order = np.argsort(key_of[l])
        skeys = key_of[l][order]
        sids = ids[order]

        def find(offsets):
            out = np.empty((len(ixl), len(offsets)), dtype=np.int64)
            for n, off in enumerate(offsets):
                q = ixl + off
                inside = np.all((q >= 0) & (q < nlev[l][None, :]), axis=1)
                res = np.full(len(q), AF_PHYS_BOUNDARY, dtype=np.int64)
                pos = _lookup(skeys, _keys(np.where(inside[:, None], q, 0), nlev[l]))
                res[inside] = np.where(pos[inside] >= 0, sids[np.maximum(pos[inside], 0)], AF_NO_BOX)
                out[:, n] = res
            return out

        t.lvl[rows] = l + 1
        t.ix[rows] = ixl + 1
        t.neighbors[rows] = find(nbd)
        t.neighbor_mat[rows] = find(nmo)
        if l == 0:
            t.parent[rows] = AF_NO_BOX
            # r_base + (ix - 1) * dr_base * n_cell
            t.r_min[rows] = rb + (ixl.astype(np.float64) * dr_base) * nc
            t.dr[rows] = dr_base
        else:
            porder = np.argsort(key_of[l - 1])
            ppos = _lookup(key_of[l - 1][porder], _keys(ixl // 2, nlev[l - 1]))
            pids = lvl_ids[l - 1][porder][ppos]
            t.parent[rows] = pids
            cnum = np.zeros(len(ids), dtype=np.int64)
            for d in range(D):
                cnum += (ixl[:, d] & 1) << d
            t.children[pids - 1, cnum] = ids
            pdr = t.dr[pids - 1]
            dixf = (ixl & 1).astype(np.float64)
            t.r_min[rows] = t.r_min[pids - 1] + ((0.5 * pdr) * dixf) * nc
            t.dr[rows] = 0.5 * pdr

    t.lvl_ids = [np.sort(x).astype(np.int32) for x in lvl_ids]
    t.lvl_leaves = []
    t.lvl_parents = []
    for ids in t.lvl_ids:
        has_c = (t.children[ids - 1] > 0).any(axis=1)
        t.lvl_parents.append(ids[has_c])
        t.lvl_leaves.append(ids[~has_c])
    return t


def uniform_tree(ndim, n_cell, coarse_grid_size, domain_len, max_lvl,
                 coord=AF_XYZ, r_base=None) -> Tree:
    return build_tree(ndim, n_cell, coarse_grid_size, domain_len, r_base,
                      coord, max_lvl, None)


def seeded_refinement(center, sigma, base_lvl, rng=None, frac=0.0):
    """Refinement predicate: refine every box up to ``base_lvl``, then refine
    boxes whose centre lies within ``3*sigma*2**(lvl-base_lvl)``-ish shrinking
    shells of ``center`` (a Gaussian seed); ``frac`` adds a seeded random
    fraction of extra refinements to make per-level box counts uneven."""
    center = np.asarray(center, dtype=np.float64)

    def f(lvl, centers, dr):
        if lvl < base_lvl:
            return np.ones(len(centers), dtype=bool)
        k = lvl - base_lvl
        radius = 4.0 * sigma / (1.4 ** k) + np.max(dr) * 6
        d = np.sqrt(((centers - center) ** 2).sum(axis=1))
        m = d < radius
        if rng is not None and frac > 0:
            m |= (rng.random(len(centers)) < frac) & (d < 2.5 * radius)
        return m
    return f


def forest(trees):
    """Independent trees as one forest for a batched context
    (afg_tree_sync_batched): the box ids of tree q follow those of trees
    0..q-1, every id-valued table is shifted accordingly (0 = no box and -1 =
    physical boundary stay), and each level list is the concatenation of the
    trees' lists of that level.  All trees must share ndim, n_cell, the
    coordinate system and the coarse grid.  Returns the forest and the
    instance (0-based) of each of its boxes."""
    t0 = trees[0]
    for t in trees[1:]:
        if (t.ndim, t.n_cell, t.coord) != (t0.ndim, t0.n_cell, t0.coord) or \
                np.any(np.asarray(t.coarse_grid_size) != np.asarray(t0.coarse_grid_size)):
            raise ValueError("forest trees need the same ndim, n_cell, coordinates and coarse grid")
    offs = np.cumsum([0] + [t.n_boxes for t in trees])

    def shift(a, off):
        a = np.asarray(a)
        return np.where(a > 0, a + off, a)

    H = max(t.highest_lvl for t in trees)
    f = Tree(ndim=t0.ndim, n_cell=t0.n_cell, coord=t0.coord, coarse_grid_size=np.asarray(t0.coarse_grid_size),
             r_base=t0.r_base, dr_base=t0.dr_base, n_boxes=int(offs[-1]), highest_lvl=H)
    f.lvl = np.concatenate([t.lvl for t in trees])
    f.ix = np.concatenate([t.ix for t in trees])
    f.parent = np.concatenate([shift(t.parent, o) for t, o in zip(trees, offs)])
    f.children = np.concatenate([shift(t.children, o) for t, o in zip(trees, offs)])
    f.neighbors = np.concatenate([shift(t.neighbors, o) for t, o in zip(trees, offs)])
    f.neighbor_mat = np.concatenate([shift(t.neighbor_mat, o) for t, o in zip(trees, offs)])
    f.r_min = np.concatenate([t.r_min for t in trees])
    f.dr = np.concatenate([t.dr for t in trees])
    for name in ("lvl_ids", "lvl_leaves", "lvl_parents"):
        per_level = []
        for l in range(H):
            parts = [np.asarray(getattr(t, name)[l]) + o for t, o in zip(trees, offs) if l < t.highest_lvl]
            per_level.append(np.concatenate(parts).astype(np.int64) if parts else np.zeros(0, np.int64))
        setattr(f, name, per_level)
    box_inst = np.concatenate([np.full(t.n_boxes, q, dtype=np.int32) for q, t in enumerate(trees)])
    return f, box_inst


def remap_ids(old: Tree, new: Tree) -> np.ndarray:
    """For each box of `new`, its id in `old` (same level and ix), 0 for a
    box that `old` does not have: the old_id table of afg_tree_remap."""
    def keys(t):
        return {(int(t.lvl[b]),) + tuple(int(v) for v in t.ix[b]): b + 1 for b in range(t.n_boxes)}
    ko = keys(old)
    out = np.zeros(new.n_boxes, dtype=np.int32)
    for b in range(new.n_boxes):
        out[b] = ko.get((int(new.lvl[b]),) + tuple(int(v) for v in new.ix[b]), 0)
    return out


AF_REFINE, AF_DEREFINE = 2, -2     # af_refine / af_derefine (m_af_types.f90)
AF_RM_REF, AF_KEEP_REF, AF_DO_REF = -1, 0, 1


def adjust_refinement(tree: Tree, flags, max_lvl: int) -> Tree:
    """Host side of af_adjust_refinement (afivo/src/m_af_core.f90:697-1091)
    after the flag pass: the max-level clamp (995-999), ensure_two_one_balance
    (1015-1055) and handle_derefinement_flags (1057-1088) on the box flags,
    then the new tree: old leaves flagged for refinement get children, the
    children of parents flagged for derefinement go, everything else stays.
    The tree is rebuilt by build_tree with afivo's 2:1 balance over face
    neighbours only (a box may keep a coarser diagonal neighbour two levels
    down, whose corner ghost cells are then extrapolated as af_gc_box_corner
    does).  When no leaf is refined and no parent derefined the same tree
    object is returned."""
    f = np.asarray(flags, dtype=np.int64).copy()
    H = tree.highest_lvl
    has_ch = (tree.children > 0).any(axis=1)
    if H >= max_lvl:
        ids = tree.lvl_ids[max_lvl - 1] - 1
        f[ids] = np.where(f[ids] == AF_DO_REF, AF_KEEP_REF, f[ids])
    for lvl in range(H, 0, -1):
        for id_ in tree.lvl_leaves[lvl - 1]:
            b = id_ - 1
            if f[b] in (AF_DO_REF, AF_REFINE):
                f[b] = AF_REFINE
                for nb, nb_id in enumerate(tree.neighbors[b]):
                    if nb_id == AF_NO_BOX:
                        p = tree.parent[b]
                        f[tree.neighbors[p - 1][nb] - 1] = AF_REFINE
            elif f[b] == AF_RM_REF:
                for nb_id in tree.neighbors[b]:
                    if nb_id > AF_NO_BOX and (has_ch[nb_id - 1] or f[nb_id - 1] > AF_KEEP_REF):
                        f[b] = AF_KEEP_REF
                        break
    for lvl in range(H - 1, 0, -1):
        for id_ in tree.lvl_parents[lvl - 1]:
            c = tree.children[id_ - 1] - 1
            if np.all(has_ch[c]):
                continue
            if np.all(f[c] == AF_RM_REF) and f[id_ - 1] <= AF_KEEP_REF:
                f[id_ - 1] = AF_DEREFINE
            else:
                f[id_ - 1] = AF_KEEP_REF
                f[c] = np.where(f[c] != AF_DEREFINE, np.maximum(f[c], AF_KEEP_REF), f[c])
    # no leaf refined and no parent derefined: the mesh stays as it is
    leaves = np.concatenate([np.asarray(l, dtype=np.int64) for l in tree.lvl_leaves]) - 1
    parents = [np.asarray(l, dtype=np.int64) for l in tree.lvl_parents if len(l)]
    parents = np.concatenate(parents) - 1 if parents else np.zeros(0, dtype=np.int64)
    if not np.any(f[leaves] == AF_REFINE) and not np.any(f[parents] == AF_DEREFINE):
        return tree
    # boxes of the old tree that have children in the new one, by (lvl, ix)
    wants = {}
    for b in range(tree.n_boxes):
        key = (int(tree.lvl[b]),) + tuple(int(v) for v in tree.ix[b])
        wants[key] = bool(f[b] == AF_REFINE) if not has_ch[b] else bool(f[b] != AF_DEREFINE)
    D, nc = tree.ndim, tree.n_cell
    rb = np.asarray(tree.r_base, dtype=np.float64)

    def refine(lvl, centers, drl):
        ix = np.floor((centers - rb) / (drl * nc)).astype(np.int64) + 1
        return np.array([wants.get((lvl,) + tuple(int(v) for v in row), False) for row in ix], dtype=bool)

    dom = np.asarray(tree.dr_base, dtype=np.float64) * np.asarray(tree.coarse_grid_size)
    return build_tree(D, nc, tree.coarse_grid_size, dom, r_base=tree.r_base, coord=tree.coord,
                      max_lvl=max(max_lvl, H), refine=refine, face_balance=True)
