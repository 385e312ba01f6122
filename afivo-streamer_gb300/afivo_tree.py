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


def _upsample(a: np.ndarray) -> np.ndarray:
    for ax in range(a.ndim):
        a = np.repeat(a, 2, axis=ax)
    return a


def _dilate(a: np.ndarray) -> np.ndarray:
    out = a.copy()
    D = a.ndim
    padded = np.pad(a, 1)
    for off in itertools.product([-1, 0, 1], repeat=D):
        sl = tuple(slice(1 + o, 1 + o + n) for o, n in zip(off, a.shape))
        out |= padded[sl]
    return out


def _coarsen_any(a: np.ndarray) -> np.ndarray:
    D = a.ndim
    shp = []
    for n in a.shape:
        shp += [n // 2, 2]
    r = a.reshape(shp)
    return r.any(axis=tuple(range(1, 2 * D, 2)))


def build_tree(ndim: int, n_cell: int, coarse_grid_size, domain_len,
               r_base=None, coord: int = AF_XYZ, max_lvl: int = 1,
               refine=None) -> Tree:
    """Build a 2:1-balanced tree.

    ``refine(lvl, centers[m, D], dr[D]) -> bool[m]`` says which boxes of
    level ``lvl`` (given by their centres) want children; ``None`` refines
    everything (uniform grid).  Level 1 is the coarse grid of
    ``coarse_grid_size`` cells, split into boxes like ``af_set_coarse_grid``
    (m_af_core.f90:206-340).
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

    # Dense per-level arrays, index order [x, y(, z)] (C order in numpy but
    # we only use them as maps).
    shapes = [tuple(int(n) * 2 ** l for n in nx1) for l in range(max_lvl)]
    exists = [np.zeros(s, dtype=bool) for s in shapes]
    refined = [np.zeros(s, dtype=bool) for s in shapes]
    exists[0][...] = True

    def lvl_dr(l):
        d = dr_base.copy()
        for _ in range(l):
            d = 0.5 * d
        return d

    for l in range(max_lvl - 1):
        ixs = np.argwhere(exists[l])
        if len(ixs) == 0:
            break
        if refine is None:
            want = np.ones(len(ixs), dtype=bool)
        else:
            drl = lvl_dr(l)
            centers = rb + (ixs + 0.5) * drl * nc
            want = np.asarray(refine(l + 1, centers, drl), dtype=bool)
        r = np.zeros(shapes[l], dtype=bool)
        r[tuple(ixs[want].T)] = True
        refined[l] = r
        exists[l + 1] = _upsample(r)

    # 2:1 balance, fine to coarse
    # (a refined box needs its whole 3^D neighbourhood on its own level; the
    # parents of newly refined boxes are handled by the next, coarser pass
    # through the dilation of refined[l-1])
    for l in range(max_lvl - 2, 0, -1):
        refined[l - 1] |= _coarsen_any(_dilate(refined[l]))
    for l in range(max_lvl - 1):
        exists[l + 1] = _upsample(refined[l])
    refined[max_lvl - 1][...] = False

    # Assign ids
    idmaps = []
    lvl_ids = []
    next_id = 1
    # level 1: Fortran order (x fastest)
    idm = np.zeros(shapes[0], dtype=np.int64)
    cnt = int(np.prod(nx1))
    grid = np.arange(cnt, dtype=np.int64).reshape(tuple(nx1[::-1])).T
    idm[...] = grid + 1
    idmaps.append(idm)
    lvl_ids.append(np.arange(1, cnt + 1, dtype=np.int64))
    next_id = cnt + 1
    cdix = child_dix(D)
    all_ix = [None]
    # store ix per level, row = id order
    ix_of = {}
    ixs1 = np.argwhere(np.ones(shapes[0], dtype=bool))
    # order ixs1 by id
    ids1 = idm[tuple(ixs1.T)]
    order = np.argsort(ids1)
    ix_of[0] = ixs1[order]
    highest = 1
    for l in range(1, max_lvl):
        if not exists[l].any():
            break
        highest = l + 1
        pix = ix_of[l - 1]
        pids = lvl_ids[l - 1]
        is_ref = refined[l - 1][tuple(pix.T)]
        pix_r = pix[is_ref]
        n_par = len(pix_r)
        cix = (2 * pix_r[:, None, :] + cdix[None, :, :]).reshape(-1, D)
        cids = next_id + np.arange(n_par * 2 ** D, dtype=np.int64)
        next_id += len(cids)
        idm = np.zeros(shapes[l], dtype=np.int64)
        idm[tuple(cix.T)] = cids
        idmaps.append(idm)
        lvl_ids.append(cids)
        ix_of[l] = cix
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
        t.lvl[rows] = l + 1
        t.ix[rows] = ixl + 1
        pad = np.pad(idmaps[l], 1, constant_values=AF_PHYS_BOUNDARY)
        for n, off in enumerate(nbd):
            t.neighbors[rows, n] = pad[tuple((ixl + 1 + off).T)]
        for n, off in enumerate(nmo):
            t.neighbor_mat[rows, n] = pad[tuple((ixl + 1 + off).T)]
        if l == 0:
            t.parent[rows] = AF_NO_BOX
            # r_base + (ix - 1) * dr_base * n_cell
            t.r_min[rows] = rb + (ixl.astype(np.float64) * dr_base) * nc
            t.dr[rows] = dr_base
        else:
            pidm = idmaps[l - 1]
            pids = pidm[tuple((ixl // 2).T)]
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
