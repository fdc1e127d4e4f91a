"""Differentiable design problems on the GPU engine.

`DesignProblem2D` sets up a 2-D TM (Ez) problem through the C ABI: a cell with
PML, eps=12 waveguides entering on the left and leaving on the right, a design
block whose permittivity is the optimisation variable, a Gaussian Ez line
source in the input guide and DFT monitors of Ez on an output line.
`run()` advances it; with `grad=True` it keeps what the reverse-time adjoint
needs (design-point D per step, or full checkpoints every K steps) and
`backward()` returns dJ/deps over the design block for dJ/dDFT.

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

    @staticmethod
    def objective(F):
        """sum over frequencies of the mean over the line of |F|^2, and dJ/dF."""
        n = F.shape[0]
        return float(np.sum(np.abs(F) ** 2) / n), 2.0 * F / n


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
