"""Output writers restated on the host (TEST INFRASTRUCTURE ONLY).

numpy/Python restatement of afivo's output routines on host boxes
cc[n_boxes, n_var, (k,) j, i] (the layout of box%cc), used by the tests as
the checker of the device writers; the product never imports it.

- vtk_arrays: the arrays af_write_vtk writes (afivo/src/m_af_output.f90:556-752;
  single-precision points, afivo/src/m_vtk.f90:66-88)
- get_id_at / interp1: af_get_id_at without a guess
  (afivo/src/m_af_utils.f90:248-261, 266-313, 340-356) and af_interp1
  (afivo/src/m_af_interp.f90:43-105)
- line_points, plane_points, numpy_grid: the sample points of af_write_line
  (m_af_output.f90:407-463), af_write_plane (465-552), af_write_numpy (756-901)
- fortran_e and plane_text: the text of af_write_plane's file (E20.8 numbers)
- read_vtu, read_npz_stored: readers of the written files
"""
import math
import re
import struct
import zipfile

import numpy as np


def nint(x):
    """Fortran NINT: nearest integer, halves away from zero."""
    f = math.floor(x)
    d = x - f
    if d > 0.5 or (d == 0.5 and x > 0):
        return int(f) + 1
    return int(f)


def vtk_arrays(tree, cc, ivs):
    D, nc = tree.ndim, tree.n_cell
    bn = nc + 1
    leaves = np.concatenate([np.asarray(l, dtype=np.int64) for l in tree.lvl_leaves])
    nl = len(leaves)
    npb, cpb = bn ** D, nc ** D
    pts = np.zeros((nl * npb, 3), dtype=np.float32)
    conn = np.zeros((nl * cpb, 2 ** D), dtype=np.int32)
    cells = {iv: np.zeros(nl * cpb) for iv in ivs}
    for g, bid in enumerate(leaves):
        rm, dr = tree.r_min[bid - 1], tree.dr[bid - 1]
        node0, cell0 = g * npb, g * cpb
        for n in range(npb):
            idx = [(n // bn ** d) % bn for d in range(D)]
            for d in range(D):
                pts[node0 + n, d] = np.float32(rm[d] + float(idx[d]) * dr[d])
        for c in range(cpb):
            i, j = c % nc, (c // nc) % nc
            k = c // (nc * nc) if D == 3 else 0
            n = node0 + k * bn * bn + j * bn + i
            corner = [n, n + 1, n + bn, n + bn + 1]
            if D == 3:
                corner += [n + bn * bn, n + bn * bn + 1, n + bn * bn + bn, n + bn * bn + bn + 1]
            conn[cell0 + c] = corner
        for iv in ivs:
            box = cc[bid - 1, iv - 1]
            inner = box[(slice(1, nc + 1),) * D]
            cells[iv][cell0:cell0 + cpb] = inner.reshape(-1)
    n_cells = nl * cpb
    offsets = ((np.arange(n_cells, dtype=np.int64) + 1) * 2 ** D).astype(np.int32)
    types = np.full(n_cells, 8 if D == 2 else 11, dtype=np.int32)
    return dict(points=pts, connectivity=conn.reshape(-1), offsets=offsets, types=types, cells=cells)


def _inside(tree, b, r):
    D = tree.ndim
    for d in range(D):
        lo = tree.r_min[b - 1, d]
        hi = lo + tree.dr[b - 1, d] * tree.n_cell
        if not (r[d] >= lo and r[d] <= hi):
            return False
    return True


def get_id_at(tree, r):
    D = tree.ndim
    bid = -1
    for b in tree.lvl_ids[0]:
        if _inside(tree, int(b), r):
            bid = int(b)
            break
    if bid < 0:
        return -1
    while tree.children[bid - 1, 0] > 0:
        ch = 0
        for d in range(D):
            c = tree.r_min[bid - 1, d] + tree.dr[bid - 1, d] * (tree.n_cell >> 1)
            if r[d] > c:
                ch += 1 << d
        bid = int(tree.children[bid - 1, ch])
    return bid


def interp1(tree, cc, r, ivs):
    """(values[len(ivs)], success) at one point r."""
    D = tree.ndim
    bid = get_id_at(tree, r)
    if bid < 0:
        return [0.0] * len(ivs), False
    ix, dv, ov = [], [], []
    for d in range(D):
        rm, dr = tree.r_min[bid - 1, d], tree.dr[bid - 1, d]
        i = nint((r[d] - rm) / dr)
        rloc = rm + (i - 0.5) * dr
        t = (r[d] - rloc) / dr
        ix.append(i)
        dv.append(t)
        ov.append(1.0 - t)
    if D == 2:
        w = [ov[0] * ov[1], dv[0] * ov[1], ov[0] * dv[1], dv[0] * dv[1]]
    else:
        w = [ov[0] * ov[1] * ov[2], dv[0] * ov[1] * ov[2], ov[0] * dv[1] * ov[2], dv[0] * dv[1] * ov[2],
             ov[0] * ov[1] * dv[2], dv[0] * ov[1] * dv[2], ov[0] * dv[1] * dv[2], dv[0] * dv[1] * dv[2]]
    out = []
    for iv in ivs:
        box = cc[bid - 1, iv - 1]
        acc = 0.0
        for e in range(2 ** D):
            o = [(e >> d) & 1 for d in range(D)]
            # box index order (k,) j, i
            idx = tuple(ix[d] + o[d] for d in reversed(range(D)))
            acc = acc + w[e] * float(box[idx])
        out.append(acc)
    return out, True


def line_points(r_min, r_max, n_points):
    D = len(r_min)
    drv = [(r_max[d] - r_min[d]) / max(1, n_points - 1) for d in range(D)]
    return [[r_min[d] + i * drv[d] for d in range(D)] for i in range(n_points)]


def plane_points(r_min, r_max, n_pixels):
    """(points in pixel order i fastest, dims[3], origin[3], spacing[3])"""
    D = len(r_min)
    dvec = [r_max[d] - r_min[d] for d in range(D)]
    n1, n2 = n_pixels[0] - 1, n_pixels[1] - 1
    if D == 2:
        v1, v2 = [dvec[0] / n1, 0.0 / n1], [0.0 / n2, dvec[1] / n2]
        dims = [n_pixels[0], n_pixels[1], 1]
        origin = [r_min[0], r_min[1], 0.0]
        spacing = [v1[0] + v2[0], v1[1] + v2[1], 0.0]
    else:
        a = [abs(x) for x in dvec]
        un = a.index(min(a))
        keep = [d for d in range(3) if d != un]
        v1 = [(dvec[d] if d == keep[0] else 0.0) / n1 for d in range(3)]
        v2 = [(dvec[d] if d == keep[1] else 0.0) / n2 for d in range(3)]
        dims = [[1, n_pixels[0], n_pixels[1]], [n_pixels[0], 1, n_pixels[1]], [n_pixels[0], n_pixels[1], 1]][un]
        origin = list(r_min)
        spacing = [v1[d] + v2[d] for d in range(3)]
    pts = [[r_min[d] + i * v1[d] + j * v2[d] for d in range(D)]
           for j in range(n_pixels[1]) for i in range(n_pixels[0])]
    return pts, dims, origin, spacing


def fortran_e(v, w=20, d=8):
    """Fortran Ew.d of one value (0.d1..dd E+xx), right-justified."""
    if math.isnan(v):
        s = "NaN"
    elif math.isinf(v):
        s = "-Infinity" if v < 0 else "Infinity"
    else:
        m, e = f"{abs(v):.{d - 1}E}".split("E")
        digits = m.replace(".", "")
        e = int(e) + (1 if v != 0 else 0)
        sign = "-" if math.copysign(1.0, v) < 0 else ""
        es = f"E{'-' if e < 0 else '+'}{abs(e):02d}" if abs(e) <= 99 else f"{'-' if e < 0 else '+'}{abs(e):03d}"
        s = f"{sign}0.{digits}{es}"
    return "*" * w if len(s) > w else s.rjust(w)


def plane_text(filename, names, dims, origin, spacing, vals, n_pixels):
    """The file af_write_plane writes; vals[pixel][v] in pixel order."""
    out = ["# vtk DataFile Version 2.0", filename, "ASCII", "DATASET STRUCTURED_POINTS",
           "DIMENSIONS " + "".join(f"{x:10d}" for x in dims),
           "ORIGIN " + "".join(fortran_e(x) for x in origin),
           "SPACING " + "".join(fortran_e(x) for x in spacing),
           f"POINT_DATA {n_pixels[0] * n_pixels[1]}"]
    for v, name in enumerate(names):
        out += [f"SCALARS {name} double 1", "LOOKUP_TABLE default"]
        for j in range(n_pixels[1]):
            out.append("".join(fortran_e(vals[j * n_pixels[0] + i][v]) for i in range(n_pixels[0])))
    return "\n".join(out) + "\n"


def numpy_grid(tree, r_min=None, r_max=None, n_points=None):
    """(points in Fortran order, nx, rmin, rmax, dr) of af_write_numpy."""
    D, nc = tree.ndim, tree.n_cell
    rb = [float(x) for x in tree.r_base]
    db = [float(x) for x in tree.dr_base]
    rmin = list(r_min) if r_min is not None else rb
    rmax = list(r_max) if r_max is not None else [rb[d] + db[d] * int(tree.coarse_grid_size[d]) for d in range(D)]
    if n_points is not None:
        nx = list(n_points)
    else:
        lvl = 1
        while lvl <= tree.highest_lvl - 1:
            found = False
            for b in tree.lvl_leaves[lvl - 1]:
                lo = tree.r_min[b - 1]
                if all(lo[d] <= rmax[d] and lo[d] + nc * tree.dr[b - 1, d] >= rmin[d] for d in range(D)):
                    found = True
                    break
            if found:
                break
            lvl += 1
        nx = [nint((rmax[d] - rmin[d]) / (db[d] * 0.5 ** (lvl - 1))) for d in range(D)]
    dr = [(rmax[d] - rmin[d]) / nx[d] for d in range(D)]
    pts = []
    for p in range(int(np.prod(nx))):
        rem, r = p, []
        for d in range(D):
            i = rem % nx[d] + 1
            rem //= nx[d]
            r.append(rmin[d] + (i - 0.5) * dr[d])
        pts.append(r)
    return pts, nx, rmin, rmax, dr


def read_vtu(path):
    """Header attributes and appended arrays of a .vtu file with raw
    appended data: (xml_text, {name: np.ndarray})."""
    raw = open(path, "rb").read()
    start = raw.index(b'<AppendedData encoding="raw">')
    us = raw.index(b"_", start) + 1
    xml = raw[:us].decode()
    h64 = 'header_type="UInt64"' in xml
    hb = 8 if h64 else 4
    types = {"Float32": np.float32, "Float64": np.float64, "Int32": np.int32}
    arrays = {}
    for m in re.finditer(r'<DataArray type="(\w+)" Name="([^"]+)"[^>]*format="appended" offset="(\d+)"', xml):
        t, name, off = m.group(1), m.group(2), int(m.group(3))
        p = us + off
        n = struct.unpack("<Q" if h64 else "<I", raw[p:p + hb])[0]
        arrays[name] = np.frombuffer(raw[p + hb:p + hb + n], dtype=types[t]).copy()
    return xml, arrays


def read_npz_stored(path):
    """Entries of an .npz archive (zip members must be stored)."""
    out = {}
    with zipfile.ZipFile(path) as z:
        for info in z.infolist():
            assert info.compress_type == zipfile.ZIP_STORED
    with np.load(path) as f:
        for k in f.files:
            out[k] = f[k]
    return out
