"""Output writers on the device state against their host restatement
(oracle_output): af_write_vtk arrays bit for bit (points, connectivity,
offsets, types, cell data), af_interp1 values and success flags bit for bit,
af_write_line numbers exactly, af_write_plane text byte for byte, and
af_write_numpy arrays (.npy, .npz) bit for bit.  Data are random in every
cell including ghost cells, so every value read is checked."""
import os

import numpy as np
import pytest

import afivo_gpu as ag
import oracle_output as oo
from mgcases import random_state, refined_tree

pytestmark = pytest.mark.gpu

TREES = {
    "2d16": lambda: refined_tree(2, 16, [32, 32], [1e-2, 1e-2], 5, 2, [0.5e-2, 0.8e-2], 0.6e-3, seed=1, frac=0.1),
    "2d8cyl": lambda: refined_tree(2, 8, [16, 32], [1e-2, 2e-2], 4, 2, [0.0, 1.2e-2], 0.8e-3,
                                   coord=ag.AFG_CYL, seed=2, frac=0.1),
    "3d4": lambda: refined_tree(3, 4, [8, 8, 8], [1.0, 1.0, 1.0], 4, 1, [0.3, 0.6, 0.5], 0.1, seed=4, frac=0.1),
}
N_VAR = 4
IVS = [1, 3, 4]
NAMES = ["phi", "e", "electric_fld"]


@pytest.fixture(scope="module", params=sorted(TREES))
def state(request):
    tree = TREES[request.param]()
    cc = random_state(tree, N_VAR, seed=11)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, N_VAR, 0)
    ctx.upload(cc)
    yield request.param, tree, cc, ctx
    ctx.close()


def bits_equal(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def domain(tree):
    lo = np.asarray(tree.r_base, dtype=np.float64)
    hi = lo + np.asarray(tree.dr_base) * np.asarray(tree.coarse_grid_size)
    return lo, hi


def test_write_vtk_arrays_bitexact(state, tmp_path):
    name, tree, cc, ctx = state
    base = str(tmp_path / f"out_{name}")
    ctx.write_vtk(base, IVS, NAMES, n_cycle=7, time=1.25e-9)
    xml, arr = oo.read_vtu(base + ".vtu")
    ref = oo.vtk_arrays(tree, cc, IVS)
    n_cells = len(ref["offsets"])
    assert f'NumberOfCells="{n_cells}"' in xml
    assert f'NumberOfPoints="{len(ref["points"])}"' in xml
    assert 'Name="TIME"' in xml and "1.25e-09" in xml and 'Name="CYCLE"' in xml
    assert bits_equal(arr["Points"], ref["points"].reshape(-1))
    assert bits_equal(arr["connectivity"], ref["connectivity"])
    assert bits_equal(arr["offsets"], ref["offsets"])
    assert bits_equal(arr["types"], ref["types"])
    for iv, nm in zip(IVS, NAMES):
        assert bits_equal(arr[nm], ref["cells"][iv]), nm
    # the file ends with the closing tags after the appended data
    assert open(base + ".vtu", "rb").read().endswith(b"</AppendedData>\n</VTKFile>\n")


def test_leaf_cells_bitexact(state):
    name, tree, cc, ctx = state
    ref = oo.vtk_arrays(tree, cc, [2])
    assert bits_equal(ctx.leaf_cells(2), ref["cells"][2])


def sample_points(tree, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = domain(tree)
    D = tree.ndim
    pts = [lo + (hi - lo) * rng.random(D) for _ in range(n)]
    # cell centres, box faces and corners of leaves, the domain corners,
    # points outside the domain
    leaves = np.concatenate(tree.lvl_leaves)
    for b in leaves[:: max(1, len(leaves) // 20)]:
        rm, dr = tree.r_min[b - 1], tree.dr[b - 1]
        pts.append(rm + 0.5 * dr)
        pts.append(rm.copy())
        pts.append(rm + dr * tree.n_cell)
        pts.append(rm + dr * (tree.n_cell // 2))
    pts += [lo, hi, lo - 1e-3 * (hi - lo), hi + 1e-3 * (hi - lo)]
    return np.array(pts)


def test_interp1_bitexact(state):
    name, tree, cc, ctx = state
    pts = sample_points(tree, 300, seed=5)
    vals, ok = ctx.interp1(pts, IVS)
    for p, r in enumerate(pts):
        ref, good = oo.interp1(tree, cc, list(r), IVS)
        assert bool(ok[p]) == good, (p, r)
        assert bits_equal(vals[p], np.array(ref)), (p, r, vals[p], ref)
    assert not ok[-1] and not ok[-2] and ok[-3] and ok[-4]


def test_write_line(state, tmp_path):
    name, tree, cc, ctx = state
    lo, hi = domain(tree)
    r0, r1 = lo + 0.1 * (hi - lo), lo + 0.9 * (hi - lo)
    base = str(tmp_path / "line")
    ctx.write_line(base, IVS, NAMES, r0, r1, 57)
    lines = open(base + ".txt").read().splitlines()
    assert lines[0] == ("# x y" if tree.ndim == 2 else "# x y z") + " " + " ".join(NAMES)
    got = np.array([[float(x) for x in ln.split()] for ln in lines[1:]])
    pts = oo.line_points(list(r0), list(r1), 57)
    ref = np.array([p + oo.interp1(tree, cc, p, IVS)[0] for p in pts])
    assert bits_equal(got, ref)
    # a point outside the tree: error, as the reference's error stop
    with pytest.raises(ag.AfgError):
        ctx.write_line(str(tmp_path / "bad"), IVS, NAMES, lo, hi + 0.5 * (hi - lo), 5)


@pytest.mark.parametrize("unused", [0, 1, 2])
def test_write_plane_text(state, tmp_path, unused):
    name, tree, cc, ctx = state
    D = tree.ndim
    if D == 2 and unused > 0:
        pytest.skip("2D planes have no unused dimension")
    lo, hi = domain(tree)
    r0, r1 = lo + 0.05 * (hi - lo), lo + 0.95 * (hi - lo)
    if D == 3:
        r1[unused] = r0[unused] + 1e-9 * (hi[unused] - lo[unused])
    npx = [23, 17]
    base = str(tmp_path / f"plane{unused}")
    ctx.write_plane(base, IVS, NAMES, r0, r1, npx)
    pts, dims, origin, spacing = oo.plane_points(list(r0), list(r1), npx)
    vals = [oo.interp1(tree, cc, p, IVS)[0] for p in pts]
    ref = oo.plane_text(base, NAMES, dims, origin, spacing, vals, npx)
    assert open(base + ".vtk").read() == ref


@pytest.mark.parametrize("kind", ["npy", "npz", "npz_auto"])
def test_write_numpy(state, tmp_path, kind):
    name, tree, cc, ctx = state
    lo, hi = domain(tree)
    D = tree.ndim
    if kind == "npz_auto":
        # the domain at the spacing of the lowest level with a leaf in it
        r0 = r1 = npt = None
    else:
        r0, r1 = lo + 0.2 * (hi - lo), lo + 0.7 * (hi - lo)
        npt = [13, 9, 5][:D]
    fn = str(tmp_path / ("grid." + ("npy" if kind == "npy" else "npz")))
    ctx.write_numpy(fn, IVS, NAMES, r_min=r0, r_max=r1, n_points=npt, n_cycle=3, time=2e-9)
    pts, nx, rmin, rmax, dr = oo.numpy_grid(tree, None if r0 is None else list(r0),
                                            None if r1 is None else list(r1), npt)
    if kind == "npz_auto" and np.prod(nx) > 20000:
        pytest.skip("grid too large for the Python restatement")
    ref = np.array([oo.interp1(tree, cc, p, IVS)[0] for p in pts])  # [n_points, n_iv]
    if kind == "npy":
        got = np.load(fn)
        assert got.shape == tuple(nx) + (len(IVS),) and np.isfortran(got)
        assert bits_equal(got.reshape(-1, len(IVS), order="F"), ref)
    else:
        z = oo.read_npz_stored(fn)
        for v, nm in enumerate(NAMES):
            assert z[nm].shape == tuple(nx)
            assert bits_equal(np.ascontiguousarray(z[nm].reshape(-1, order="F")), np.ascontiguousarray(ref[:, v]))
        assert list(z["nx"]) == list(nx) and z["nx"].dtype == np.int32
        assert bits_equal(z["r_min"], np.array(rmin)) and bits_equal(z["r_max"], np.array(rmax))
        assert bits_equal(z["dr"], np.array(dr))
        assert list(z["coord_t"]) == [tree.coord]
        assert list(z["time_cycle"]) == [2e-9, 3.0]


def test_output_argument_errors(state, tmp_path):
    name, tree, cc, ctx = state
    with pytest.raises(ag.AfgError):
        ctx.write_vtk(str(tmp_path / "x"), [N_VAR + 1], ["bad"])
    with pytest.raises(ag.AfgError):
        ctx.write_numpy(str(tmp_path / "x.dat"), IVS, NAMES)
    assert not os.path.exists(str(tmp_path / "x.vtu"))
