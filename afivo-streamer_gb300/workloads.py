"""Synthetic streamer workloads (seeded), the inputs of the benchmark.

Four configurations of the hot path are defined here; no public dataset is
involved (each configuration defines its own inputs):

* ``cart2d`` -- the plain method in FP64: 2D Cartesian 1 cm x 1 cm, uniform
  256x256 grid of 16^2-cell boxes with the multigrid hierarchy coarsened to
  one box (5 levels, 341 boxes); electrons plus equal positive ions as a
  Gaussian seed 1e15 exp(-r^2/(2 (0.5 mm)^2)) m^-3 at (0.5 cm, 0.8 cm) on a
  1e9 m^-3 background; phi = 0 at y = 0, -3e4 V at y = 1 cm, Neumann sides;
  mobility 0.03 m^2/Vs, diffusion 0.1 m^2/s, ionization
  alpha(E) = 4.3e5 exp(-2e7/|E|), immobile ions, no photoionization;
  forward Euler at dt = 1e-12 s with one Poisson solve to 1e-10 relative
  residual per step.
* ``cyl2d`` -- 2D axisymmetric streamer, r in [0, 1 cm], z in [0, 2 cm],
  16^2-cell boxes, coarse grid 16x32, uniform to level 5 plus 4 AMR levels
  around the streamer channel (~0.56 M leaf cells, 9 levels); electrons,
  positive and negative ions; ionization alpha(E) = 4.3e5 exp(-2e7/|E|),
  attachment eta = 2e3 1/m, mobility 0.03 m^2/Vs, diffusion 0.1 m^2/s;
  3-term Helmholtz photoionization; applied field 1.5e6 V/m.
* ``3d`` -- 3D streamer, 3 cm cube, 8^3-cell boxes, coarse grid one box,
  uniform to level 6 plus 6 AMR levels around the channel (~99 M leaf cells,
  ~113 M cells, 12 levels); 5 species (e, N2+, O2+, O2-, O-) with 8
  field-dependent reactions k(E) = A exp(-B/|E|), A log-uniform in
  [1e-18, 1e-14] m^3/s and B uniform in [1e7, 3e7] V/m, each evaluated as the
  reference's rate form k13 c1 exp(-(c2/(c3+Td))^c4) with c1 = A,
  c2 = B*1e21/N, c3 = 0, c4 = 1 (src/m_chemistry.f90:117-118,751-752);
  transport as cyl2d; 3-term Helmholtz photoionization; applied field
  1.5e6 V/m.

* ``poisson3d`` -- 3D Poisson + 3 Helmholtz modes, 2 cm cube, 8^3 boxes,
  10 levels (~41 M cells) refined around a Gaussian seed (Poisson3d).
* ``batch`` -- 256 independent 2D axisymmetric Poisson + transport
  instances of uneven size (BatchCyl2d), run as one forest.

The refinement maps stand in for afivo's refinement criterion
(alpha(E)*dx > 0.8 around a developed streamer, src/m_refine.f90:239-245):
nested cylinders around the channel axis whose radius halves per level.
"""
from __future__ import annotations

import numpy as np

import afivo_gpu as ag
import afivo_tree as at
import streamer_model as sm


def channel_refinement(base, radii, z_tail, z_head, axis_xy=None):
    """Refine every box up to level `base`, then boxes within radius
    radii[l - base] of the channel axis between z_tail and z_head."""
    def f(lvl, c, dr):
        if lvl < base:
            return np.ones(len(c), bool)
        R = radii[lvl - base]
        z = c[:, -1]
        if axis_xy is None:
            rr = np.abs(c[:, 0])
        else:
            rr = np.sqrt(((c[:, :-1] - np.asarray(axis_xy)) ** 2).sum(axis=1))
        return (rr < R) & (z > z_tail - R) & (z < z_head + R)
    return f


class Workload:
    name = ""
    voltage = 0.0
    dt = 5e-12
    integrator = "heun"
    max_rel_residual = 1e-8
    use_photoi = True
    noise = 1e-3                                           # relative electron noise
    amplitude = 1e15                                       # seed peak density (1/m^3)
    photoi_lambda = np.array([50.0, 150.0, 500.0])        # 1/m
    photoi_coeffs = np.array([1e-2, 5e-2, 1e-1]) * 1e4     # 1/m^2
    photoi_eta_quench = 0.05 * 0.038

    def run_kwargs(self):
        """Keyword arguments of StreamerRun / OracleStreamerRun."""
        return dict(max_rel_residual=self.max_rel_residual, num_vcycles=30, integrator=self.integrator,
                    photoi=((self.photoi_lambda, self.photoi_coeffs, self.photoi_eta_quench)
                            if self.use_photoi else None))

    def tree(self, reduced=False, coarsen=0):
        raise NotImplementedError

    def model(self):
        raise NotImplementedError

    def seed_center(self):
        raise NotImplementedError

    def initial_host_state(self, tree, model, seed=12345):
        """Potential and species densities (state 0) on every box: host array
        [n_boxes, 1 + n_species, (nc+2)^D] in the reference's per-box layout,
        and the variable indices of its columns."""
        ivs = [model.i_phi] + list(model.species_iv)
        n2 = tree.n_cell + 2
        H = np.empty((tree.n_boxes, len(ivs)) + (n2,) * tree.ndim)
        for v, iv in enumerate(ivs):
            self.fill_variable(tree, model, iv, seed=seed, out=H[:, v])
        return H, ivs

    def fill_variable(self, tree, model, iv, seed=12345, out=None, chunk=8192):
        """Initial value of cell-centred variable iv (1-based) on all boxes,
        ghost cells included: array [n_boxes, (nc+2)^D] (or written into
        `out` of that shape).  Computed in chunks of boxes; the noise of
        chunk c comes from generator (seed, c)."""
        D, nc = tree.ndim, tree.n_cell
        n2 = nc + 2
        if out is None:
            out = np.empty((tree.n_boxes,) + (n2,) * D)
        idx = np.arange(n2) - 0.5
        c = self.seed_center()
        sig = self.seed_sigma
        L = float(tree.dr[0, -1] * tree.coarse_grid_size[-1])
        s = model.species_iv.index(iv) if iv in model.species_iv else -1
        for c0 in range(0, tree.n_boxes, chunk):
            c1 = min(tree.n_boxes, c0 + chunk)
            m = c1 - c0
            X = []  # cell-centre coordinates, broadcastable to [m, (k,) j, i]
            for d in range(D):
                shape = [m] + [1] * D
                shape[1 + (D - 1 - d)] = n2
                X.append((tree.r_min[c0:c1, d][:, None] + idx[None, :] * tree.dr[c0:c1, d][:, None]).reshape(shape))
            o = out[c0:c1]
            if iv == model.i_phi:
                o[...] = self.voltage * np.broadcast_to(X[D - 1], o.shape) / L
                continue
            if s != 0 and s != self.positive_species:
                o[...] = 0.0
                continue
            r2 = sum((X[d] - c[d]) ** 2 for d in range(D))
            g = self.amplitude * np.exp(-r2 / (2 * sig ** 2)) + 1e9
            if s == 0 and self.noise:
                rng = np.random.default_rng([seed, c0 // chunk])
                g = g * (1 + self.noise * rng.standard_normal(g.shape))
            o[...] = g
        return out


class Cart2d(Workload):
    name = "cart2d"
    voltage = -3e4
    dt = 1e-12
    integrator = "forward_euler"
    max_rel_residual = 1e-10
    use_photoi = False
    noise = 0.0
    seed_sigma = 0.5e-3
    positive_species = 1

    def tree(self, reduced=False, coarsen=0):
        return at.build_tree(2, 16, [16, 16], [1e-2, 1e-2], max_lvl=5 - coarsen)

    def model(self):
        return sm.StreamerModel(2, n_states=sm.states_needed(self.integrator),
                                species=[sm.Species("e", -1.0), sm.Species("M+", 1.0)],
                                alpha=sm.baseline_alpha)

    def seed_center(self):
        return (0.5e-2, 0.8e-2)


class Cyl2d(Workload):
    name = "cyl2d"
    voltage = -3e4          # 1.5e6 V/m over 2 cm
    seed_sigma = 0.5e-3
    positive_species = 1

    def tree(self, reduced=False, coarsen=0):
        return at.build_tree(2, 16, [16, 32], [1e-2, 2e-2], coord=ag.AFG_CYL, max_lvl=9,
                             refine=channel_refinement(5, [2e-3, 1e-3, 0.6e-3, 0.35e-3], 0.9e-2, 1.4e-2))

    def model(self):
        return sm.StreamerModel(2, alpha=sm.baseline_alpha, eta=sm.baseline_eta, photoi_modes=3)

    def seed_center(self):
        return (0.0, 1.2e-2)


class Streamer3d(Workload):
    name = "3d"
    voltage = -4.5e4        # 1.5e6 V/m over 3 cm
    seed_sigma = 0.3e-3
    positive_species = 1

    def tree(self, reduced=False, coarsen=0):
        """The full tree, or the same construction `coarsen` levels coarser
        everywhere (each level ~1/8 of the boxes); reduced=True is coarsen=2
        (~1/50 of the cells), the CPU baseline's sample."""
        k = 2 if reduced else coarsen
        return at.build_tree(3, 8, [8, 8, 8], [3e-2] * 3, max_lvl=12 - k,
                             refine=channel_refinement(6 - k, [3.2e-3, 1.7e-3, 1.0e-3, 0.5e-3, 0.25e-3, 0.12e-3],
                                                       1.2e-2, 1.8e-2, axis_xy=(1.5e-2, 1.5e-2)))

    def model(self):
        N = sm.gas_number_density()
        rng = np.random.default_rng(4242)
        A = 10 ** rng.uniform(-18, -14, size=8)
        B = rng.uniform(1e7, 3e7, size=8)
        # species: 0 e, 1 N2+, 2 O2+, 3 O2-, 4 O-
        reac = [([0], [0, 1], [2, 1], 0.79 * N),   # e + N2 -> e + e + N2+
                ([0], [0, 2], [2, 1], 0.21 * N),   # e + O2 -> e + e + O2+
                ([0], [4], [1], 0.21 * N),         # e + O2 -> O-
                ([0], [3], [1], 0.21 * N),         # e + O2 (+M) -> O2-
                ([3], [0], [1], N),                # O2- + M -> e
                ([4], [0], [1], N),                # O- + M -> e
                ([1], [2], [1], 0.21 * N),         # N2+ + O2 -> O2+
                ([0, 2], [], [], 1.0)]             # e + O2+ -> neutrals
        reactions = []
        for n, (ins, outs, mult, fac) in enumerate(reac):
            reactions.append(dict(type=ag.RATE_K13, factor=fac, c=[A[n], B[n] * 1e21 / N, 0.0, 1.0],
                                  ix_in=ins, ix_out=outs, mult=mult))
        species = [sm.Species("e", -1.0), sm.Species("N2+", 1.0), sm.Species("O2+", 1.0),
                   sm.Species("O2-", -1.0), sm.Species("O-", -1.0)]
        m = sm.StreamerModel(3, species=species, alpha=sm.baseline_alpha, eta=sm.baseline_eta,
                             reactions=reactions, photoi_modes=3)
        m.photoi_species_index = 2   # photoionization produces O2+
        return m

    def seed_center(self):
        return (1.5e-2, 1.5e-2, 1.7e-2)


class Poisson3d(Workload):
    """3D Poisson + Helmholtz configuration: 2 cm cube, 8^3-cell boxes,
    uniform to level 5 plus 5 AMR levels (10 levels, ~41 M cells) from a
    seeded refinement map around a Gaussian seed of sigma = 0.3 mm at the
    centre: spheres whose radius shrinks per level, with a seeded
    modulation of their surface (uneven per-level box counts).  The
    Poisson right-hand side comes from the seed's charge, the applied field
    is 1.5e6 V/m; three Helmholtz modes (photoionization) share the source."""
    name = "poisson3d"
    voltage = -3e4
    seed_sigma = 0.3e-3
    positive_species = 1
    radii = (6.3e-3, 3.8e-3, 2.15e-3, 1.3e-3, 0.75e-3)

    def tree(self, reduced=False, coarsen=0):
        c = np.asarray(self.seed_center())
        radii = self.radii
        rng = np.random.default_rng(2026)
        a, b, ph = rng.uniform(20, 40, 3), rng.uniform(5, 15, 3), rng.uniform(0, 2 * np.pi, 3)

        def refine(lvl, cen, dr):
            if lvl < 5:
                return np.ones(len(cen), bool)
            R = radii[lvl - 5]
            d = np.sqrt(((cen - c) ** 2).sum(axis=1))
            mod = 1 + 0.25 * np.sin(a[0] * cen[:, 0] / R + b[0] * cen[:, 1] / R + ph[0]) * \
                np.cos(a[1] * cen[:, 2] / R + ph[1])
            return d < R * mod
        return at.build_tree(3, 8, [8, 8, 8], [2e-2] * 3, max_lvl=10 - coarsen, refine=refine)

    def model(self):
        return sm.StreamerModel(3, alpha=sm.baseline_alpha, eta=sm.baseline_eta, photoi_modes=3)

    def seed_center(self):
        return (1e-2, 1e-2, 1e-2)


class CylInstance(Workload):
    """One instance of the batched configuration: 2D axisymmetric,
    r in [0, 1 cm], z in [0, 1 cm], uniform grid of `side`^2 cells in 16^2
    boxes (coarse grid one box, log2(side/16)+1 levels), the cyl2d transport
    and chemistry without photoionization."""
    name = "cyl-instance"
    seed_sigma = 0.5e-3
    positive_species = 1
    use_photoi = False

    def __init__(self, side, voltage, amplitude):
        self.side, self.voltage, self.amplitude = int(side), float(voltage), float(amplitude)

    def tree(self, reduced=False, coarsen=0):
        levels = int(np.log2(self.side // 16)) + 1
        return at.build_tree(2, 16, [16, 16], [1e-2, 1e-2], coord=ag.AFG_CYL, max_lvl=levels)

    def model(self):
        return sm.StreamerModel(2, alpha=sm.baseline_alpha, eta=sm.baseline_eta)

    def seed_center(self):
        return (0.0, 0.8e-2)


class BatchCyl2d:
    """Batched uneven instances: n_inst independent 2D axisymmetric
    Poisson + transport instances; grid sides drawn uniformly from
    {64, 128, 256, 512}, applied voltages uniformly from 15-35 kV over 1 cm
    (negative, as the other workloads), seed amplitudes log-uniform in
    [1e13, 1e16] m^-3, all from one seed (expected 22.3 M leaf cells for 256
    instances)."""
    name = "batch"
    dt = 5e-12
    integrator = "heun"
    max_rel_residual = 1e-8
    domain_len = 1e-2

    def __init__(self, n_inst=256, seed=2024, sides=(64, 128, 256, 512)):
        rng = np.random.default_rng(seed)
        self.sides = rng.choice(np.asarray(sides), size=n_inst)
        self.voltages = -rng.uniform(15e3, 35e3, size=n_inst)
        self.amplitudes = 10 ** rng.uniform(13, 16, size=n_inst)
        self.instances = [CylInstance(s, v, a) for s, v, a in zip(self.sides, self.voltages, self.amplitudes)]

    def model(self):
        return self.instances[0].model()

    def run_kwargs(self):
        return dict(max_rel_residual=self.max_rel_residual, num_vcycles=30, integrator=self.integrator, photoi=None)

    def trees(self):
        return [w.tree() for w in self.instances]

    def forest(self, trees=None):
        """(forest tree, instance of each box, instance trees)"""
        trees = trees if trees is not None else self.trees()
        f, box_inst = at.forest(trees)
        return f, box_inst, trees

    def initial_host_state(self, trees, model):
        """Per-instance initial states stacked in forest box order (as
        Workload.initial_host_state)."""
        parts, ivs = [], None
        for q, (w, t) in enumerate(zip(self.instances, trees)):
            H, ivs = w.initial_host_state(t, model, seed=12345 + q)
            parts.append(H)
        return np.concatenate(parts), ivs


WORKLOADS = {"cart2d": Cart2d, "cyl2d": Cyl2d, "3d": Streamer3d, "poisson3d": Poisson3d}
