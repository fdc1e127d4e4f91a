"""Differentiable design problems on the GPU engine.

`DesignProblem2D` sets up a 2-D TM (Ez) problem through the C ABI: a cell with
PML, eps=12 waveguides entering on the left and leaving on the right, a design
block whose permittivity is the optimisation variable, a Gaussian Ez line
source in the input guide and DFT monitors of Ez on an output line.
`run()` advances it; with `grad=True` it keeps what the reverse-time adjoint
needs (design-point D per step, or full checkpoints every K steps) and
`backward()` returns dJ/deps over the design block for dJ/dDFT.

`DesignProblem3D` is the 3-D counterpart with a flux objective.

`DesignDFT` is the torch.autograd.Function mapping the design permittivity to
the complex DFT of the output line, so objectives can be written in torch.
"""
import numpy as np

from . import _lib


class DesignProblem2D:
    """Synthetic waveguide-and-design-block problem (2-D TM).

    Default sizes: 400x240 cells at resolution 20 (20 x 12 units), 16-cell PML
    (0.8 units) on every side, 8-cell eps=12 guides, 100x100 design block in
    the middle, Gaussian Ez line source (fcen 0.15, df 0.05) across the input
    guide, 10 frequencies on a 20-cell output line, 3000 steps.
    """

    def __init__(self, engine=None, nx=400, ny=240, res=20.0, dpml_cells=16, guide_cells=8, design=(100, 100),
                 fcen=0.15, df=0.05, nfreq=10, line_cells=20, steps=3000, precision=64):
        self.eng = engine or _lib.Engine()
        self.nx, self.ny, self.res = nx, ny, res
        self.dpml = dpml_cells / res
        self.guide = guide_cells
        self.design = design
        self.fcen, self.df, self.nfreq = fcen, df, nfreq
        self.line = line_cells
        self.steps = steps
        self.precision = precision
        self.comps = [_lib.comp(_lib.E, _lib.Z), _lib.comp(_lib.D, _lib.Z), _lib.comp(_lib.H, _lib.X),
                      _lib.comp(_lib.B, _lib.X), _lib.comp(_lib.H, _lib.Y), _lib.comp(_lib.B, _lib.Y)]
        self.ez = self.comps[0]
        ext = (nx + 1, ny + 1)
        jc = ny // 2
        self.guide_j = (jc - guide_cells // 2, jc + guide_cells // 2)
        self.lo = (nx // 2 - design[0] // 2, jc - design[1] // 2, 0)
        self.hi = (self.lo[0] + design[0] - 1, self.lo[1] + design[1] - 1, 0)
        eps = np.ones(ext)
        eps[:, self.guide_j[0]:self.guide_j[1]] = 12.0
        self.eps_bg = eps
        self.src_i = dpml_cells + 10
        self.out_i = nx - dpml_cells - 10
        self.line_j = (jc - line_cells // 2, jc - line_cells // 2 + line_cells - 1)
        self.freqs = np.linspace(fcen - df / 2, fcen + df / 2, nfreq)

    def _sim(self, eps_design, precision):
        pml = {(d, s): (self.dpml, 1e-15, 1.0) for d in (0, 1) for s in (0, 1)}
        sim = _lib.Sim(self.eng, dim=2, n=(self.nx, self.ny, 0), io=(-self.nx, -self.ny, 0), a=self.res,
                       courant=0.5, pml=pml, precision=precision, components=self.comps)
        eps = self.eps_bg.copy()
        eps[self.lo[0]:self.hi[0] + 1, self.lo[1]:self.hi[1] + 1] = eps_design
        sim.set_chi1inv(self.ez, _lib.Z, 1.0 / eps)
        src = sim.add_gaussian_src(self.fcen, self.df)
        ext1 = self.ny + 1
        idx = [self.src_i * ext1 + j for j in range(self.guide_j[0], self.guide_j[1] + 1)]
        sim.add_source_points(self.ez, src, idx, np.ones(len(idx)) * self.res)
        npt = self.line_j[1] - self.line_j[0] + 1
        mid = sim.add_dft(self.ez, (self.out_i, self.line_j[0], 0), (self.out_i, self.line_j[1], 0),
                          [np.ones(1), np.ones(npt), None], dV=1.0, include_weights=False, scale=1.0,
                          centered=False, freqs=self.freqs, decimation=1)
        return sim, mid

    def run(self, eps_design, grad=False, checkpoint_every=55, precision=None):
        """Forward run.  Returns (F, handle): F is the complex DFT of Ez on the
        output line, [npts, nfreq]; handle is passed to backward() (None when
        grad is False)."""
        prec = precision or self.precision
        sim, mid = self._sim(np.asarray(eps_design, dtype=np.float64), prec)
        if grad:
            sim.design([self.ez], self.lo, self.hi)
            sim.forward(self.steps, checkpoint_every)
        else:
            sim.step(self.steps)
        F = sim.get_dft(mid)
        if not grad:
            sim.close()
            return F, None
        return F, (sim, mid, np.asarray(eps_design, dtype=np.float64))

    @staticmethod
    def backward(handle, dJdF):
        """dJ/deps over the design block for dJdF = dJ/dRe F + i dJ/dIm F."""
        sim, mid, eps_design = handle
        gchi = sim.backward({mid: dJdF})[0, :, :, 0]
        sim.close()
        return -gchi / (eps_design * eps_design)  # chi1inv = 1/eps

    def grid_block(self):
        """(center, size) of the block that a material grid over the design
        takes: the design's Ez points with half a pixel around them, so a
        grid of design-sized nodes puts one node on every point."""
        h = 0.5 / self.res
        x0 = [(-n + 2 * l) * h for n, l in ((self.nx, self.lo[0]), (self.ny, self.lo[1]))]
        x1 = [(-n + 2 * l) * h for n, l in ((self.nx, self.hi[0]), (self.ny, self.hi[1]))]
        return ((0.5 * (x0[0] + x1[0]), 0.5 * (x0[1] + x1[1]), 0.0),
                (x1[0] - x0[0] + 2 * h, x1[1] - x0[1] + 2 * h, 0.0))

    def run_grid(self, weights, grid, grad=False, checkpoint_every=55, precision=None):
        """Forward run with the design block's permittivity from a material
        grid: weights u of shape grid['n'], eps = eps1 + p (eps2 - eps1) with
        p the (beta, eta) projection of u interpolated to each Ez point,
        evaluated by the engine (mfd_add_material_grid).  Returns (F, handle)
        as run() does."""
        prec = precision or self.precision
        sim, mid = self._sim(np.full(self.design, float(grid["eps1"])), prec)
        center, size = self.grid_block()
        gid = sim.add_material_grid(center, size, np.asarray(weights, dtype=np.float64).reshape(grid["n"]),
                                    grid["eps1"], grid["eps2"], beta=grid.get("beta", 0.0),
                                    eta=grid.get("eta", 0.5))
        if grad:
            sim.design([self.ez], self.lo, self.hi)
            sim.forward(self.steps, checkpoint_every)
        else:
            sim.step(self.steps)
        F = sim.get_dft(mid)
        if not grad:
            sim.close()
            return F, None
        return F, (sim, mid, gid, tuple(grid["n"]))

    @staticmethod
    def backward_grid(handle, dJdF):
        """dJ/du of the material grid's weights for dJdF (run_grid handle):
        the reverse-time dJ/dchi1inv through the projection and the
        interpolation (mfd_material_grid_vjp)."""
        sim, mid, gid, n = handle
        gchi = sim.backward({mid: dJdF})
        gu = sim.material_grid_vjp(gid, gchi)
        sim.close()
        return gu.reshape(n)

    @staticmethod
    def objective(F):
        """sum over frequencies of the mean over the line of |F|^2, and dJ/dF."""
        n = F.shape[0]
        return float(np.sum(np.abs(F) ** 2) / n), 2.0 * F / n


class DesignProblem3D:
    """Synthetic 3-D design problem: an eps block on a slab under a dipole,
    objective = flux through a plane above it, summed over frequencies.

    Default sizes: 192x192x128 cells at resolution 20, 16-cell PML (0.8
    units) on every face, an eps=2.1 slab 10 cells thick across the cell, a
    64x64x16-voxel design block (eps per voxel) on top of it, a Gaussian Ex
    dipole (fcen 0.25, df 0.1) below the slab, and Ex, Ey, Hx, Hy DFT
    monitors at 20 frequencies on a 128x128 z-normal plane above the block;
    2000 steps.  The objective is J = sum_w Flux_z(w), Flux_z = sum over the
    plane of Re(Ex conj Hy - Ey conj Hx).  The design variable is eps of each
    voxel, applied to the inverse permittivity of Ex, Ey and Ez at the point
    of the same index.
    """

    def __init__(self, engine=None, n=(192, 192, 128), res=20.0, dpml_cells=16, slab=(40, 50), design=(64, 64, 16),
                 plane_z=90, plane=128, src_z=30, fcen=0.25, df=0.1, nfreq=20, steps=2000, precision=32):
        self.eng = engine or _lib.Engine()
        self.n, self.res = tuple(n), res
        self.dpml = dpml_cells / res
        self.steps, self.precision = steps, precision
        self.fcen, self.df = fcen, df
        self.freqs = np.linspace(fcen - df / 2, fcen + df / 2, nfreq)
        self.comps = [_lib.comp(t, d) for t in range(4) for d in range(3)]
        self.ecomps = [_lib.comp(_lib.E, d) for d in range(3)]
        self.ext = tuple(x + 1 for x in self.n)
        cx, cy = self.n[0] // 2, self.n[1] // 2
        self.lo = (cx - design[0] // 2, cy - design[1] // 2, slab[1])
        self.hi = (self.lo[0] + design[0] - 1, self.lo[1] + design[1] - 1, slab[1] + design[2] - 1)
        eps = np.ones(self.ext)
        eps[:, :, slab[0]:slab[1]] = 2.1
        self.eps_bg = eps
        self.src = (cx, cy, src_z)
        self.plane_lo = (cx - plane // 2, cy - plane // 2, plane_z)
        self.plane_hi = (self.plane_lo[0] + plane - 1, self.plane_lo[1] + plane - 1, plane_z)
        self.design_shape = design

    def _sim(self, eps_design, precision):
        pml = {(d, s): (self.dpml, 1e-15, 1.0) for d in range(3) for s in (0, 1)}
        sim = _lib.Sim(self.eng, dim=3, n=self.n, io=tuple(-x for x in self.n), a=self.res, courant=0.5, pml=pml,
                       precision=precision, components=self.comps)
        eps = self.eps_bg.copy()
        eps[self.lo[0]:self.hi[0] + 1, self.lo[1]:self.hi[1] + 1, self.lo[2]:self.hi[2] + 1] = eps_design
        inv = 1.0 / eps
        for d, c in enumerate(self.ecomps):
            sim.set_chi1inv(c, d, inv)
        src = sim.add_gaussian_src(self.fcen, self.df)
        e1, e2 = self.ext[1], self.ext[2]
        sim.add_source_points(self.ecomps[0], src, [(self.src[0] * e1 + self.src[1]) * e2 + self.src[2]], [1.0])
        npl = self.plane_hi[0] - self.plane_lo[0] + 1
        w = [np.ones(npl), np.ones(npl), np.ones(1)]
        mons = {}
        for name, c, sc in (("ex", _lib.comp(_lib.E, _lib.X), 1.0), ("ey", _lib.comp(_lib.E, _lib.Y), -1.0),
                            ("hx", _lib.comp(_lib.H, _lib.X), 1.0), ("hy", _lib.comp(_lib.H, _lib.Y), 1.0)):
            mons[name] = sim.add_dft(c, self.plane_lo, self.plane_hi, w, dV=1.0, include_weights=False, scale=sc,
                                     centered=False, freqs=self.freqs, decimation=1)
        return sim, mons

    @staticmethod
    def objective(F):
        """J = sum_w Flux(w) and dJ/dF for F = {ex, ey, hx, hy} DFT arrays (the
        Ey monitor carries the flux sign in its scale)."""
        J = float(np.sum((F["ex"] * np.conj(F["hy"])).real + (F["ey"] * np.conj(F["hx"])).real))
        return J, {"ex": F["hy"], "hy": F["ex"], "ey": F["hx"], "hx": F["ey"]}

    def run(self, eps_design, grad=False, checkpoint_every=-1, precision=None):
        """Forward run.  Returns (J, F, handle); handle goes to backward()."""
        prec = precision or self.precision
        eps_design = np.asarray(eps_design, dtype=np.float64)
        sim, mons = self._sim(eps_design, prec)
        if grad:
            sim.design(self.ecomps, self.lo, self.hi)
            sim.forward(self.steps, checkpoint_every)
        else:
            sim.step(self.steps)
        F = {k: sim.get_dft(m) for k, m in mons.items()}
        J, _ = self.objective(F)
        if not grad:
            sim.close()
            return J, F, None
        return J, F, (sim, mons, eps_design)

    def backward(self, handle, F):
        """dJ/deps over the design block for the flux objective."""
        sim, mons, eps_design = handle
        _, g = self.objective(F)
        gchi = sim.backward({mons[k]: g[k] for k in g})
        sim.close()
        return -gchi.sum(axis=0) / (eps_design * eps_design)  # chi1inv = 1/eps on Ex, Ey, Ez


try:
    import torch

    class DesignDFT(torch.autograd.Function):
        """eps over the design block (float64 tensor) -> complex DFT of the
        output line (complex128 tensor [npts, nfreq]); backward runs the
        reverse-time adjoint on the GPU engine."""

        @staticmethod
        def forward(ctx, eps, problem, checkpoint_every=55):
            F, handle = problem.run(eps.detach().cpu().numpy(), grad=True, checkpoint_every=checkpoint_every)
            ctx.handle = handle
            return torch.from_numpy(F)

        @staticmethod
        def backward(ctx, grad_F):
            # torch passes dJ/dRe F + i dJ/dIm F for a real objective
            g = DesignProblem2D.backward(ctx.handle, grad_F.detach().cpu().numpy())
            ctx.handle = None
            return torch.from_numpy(g), None, None

except ImportError:  # torch is optional for the C ABI and the C++ drop-in
    DesignDFT = None
