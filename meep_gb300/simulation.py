"""Meep's Python Simulation interface over the GB300 engine.

The names, arguments and defaults follow the reference's Python layer
(python/simulation.py, python/geom.py, python/source.py) for the stepping
path: a cell with PML layers, geometry of blocks / spheres / cylinders with
media (epsilon or index, diagonal anisotropy, D conductivity, Lorentzian and
Drude susceptibilities), Gaussian and continuous sources on points or
volumes, DFT flux regions and DFT field monitors, `run(until=...)` and
`run(until_after_sources=...)` with step functions.  The calls land on the
C++ drop-in (include/meep_gb300/meep.hpp) through its C interface
(include/meep_gb300/mgb.h), which runs the CUDA engine.

Subpixel averaging (`eps_averaging=True`, the default) runs on the GPU with
the reference's default material-function method (sphere-quadrature normal,
sampled means of eps and 1/eps, `subpixel_tol`, `subpixel_maxeval`): the
reference's Python layer averages through libctl's analytic overlaps instead,
so interface pixels differ from it at the level of the averaging tolerance.
Averaging needs isotropic media.  Fields are double precision unless the
environment sets MEEP_GB300_PRECISION=32 (the reference's single-precision
build).  Differences from the reference, raised as
errors where they would change results: no symmetries, no material functions
(per-point Python callables).  `k_point` gives Bloch-periodic walls (complex
fields when it is nonzero), as in the reference.

    import meep_gb300 as mp
    sim = mp.Simulation(cell_size=mp.Vector3(16, 8), resolution=10,
                        boundary_layers=[mp.PML(1.0)], eps_averaging=False,
                        geometry=[mp.Block(mp.Vector3(mp.inf, 1, mp.inf),
                                           material=mp.Medium(epsilon=12))],
                        sources=[mp.Source(mp.GaussianSource(0.15, fwidth=0.1),
                                           component=mp.Ez, center=mp.Vector3(-7))])
    flux = sim.add_flux(0.15, 0.1, 50, mp.FluxRegion(center=mp.Vector3(6), size=mp.Vector3(y=2)))
    sim.run(until_after_sources=200)
    print(mp.get_fluxes(flux))
"""
import collections
import ctypes as C
import math
import numbers
import os
import warnings

import numpy as np

# meep::component values
Ex, Ey, Er, Ep, Ez, Hx, Hy, Hr, Hp, Hz, Dx, Dy, Dr, Dp, Dz, Bx, By, Br, Bp, Bz = range(20)
X, Y, Z = 0, 1, 2
ALL = -1
AUTOMATIC = -1
High, Low = 0, 1
inf = 1.0e20

_HERE = os.path.dirname(os.path.abspath(__file__))
# The reference picks its floating-point type when it is built (realnum is
# float with --enable-single); both builds ship here and MEEP_GB300_PRECISION
# (64, the default, or 32) picks the one Simulation runs on.
DOUBLE_LIB = os.path.join(_HERE, "lib", "libmeep_gb300.so")
SINGLE_LIB = os.path.join(_HERE, "lib", "libmeep_gb300_single.so")


def _product_lib():
    prec = os.environ.get("MEEP_GB300_PRECISION", "64").strip()
    if prec not in ("32", "64"):
        raise ValueError("MEEP_GB300_PRECISION must be 32 or 64, not %r" % prec)
    return SINGLE_LIB if prec == "32" else DOUBLE_LIB


PRODUCT_LIB = DOUBLE_LIB


class Vector3:
    """3-vector with the reference's constructor (missing components are 0)."""

    def __init__(self, x=0.0, y=0.0, z=0.0):
        self.x, self.y, self.z = float(x), float(y), float(z)

    def __iter__(self):
        return iter((self.x, self.y, self.z))

    def __getitem__(self, i):
        return (self.x, self.y, self.z)[i]

    def __add__(self, o):
        return Vector3(self.x + o.x, self.y + o.y, self.z + o.z)

    def __sub__(self, o):
        return Vector3(self.x - o.x, self.y - o.y, self.z - o.z)

    def __mul__(self, s):
        return Vector3(self.x * s, self.y * s, self.z * s)

    __rmul__ = __mul__

    def __neg__(self):
        return Vector3(-self.x, -self.y, -self.z)

    def __eq__(self, o):
        return isinstance(o, Vector3) and tuple(self) == tuple(o)

    def __hash__(self):
        return hash(tuple(self))

    def norm(self):
        return math.sqrt(self.x * self.x + self.y * self.y + self.z * self.z)

    def unit(self):
        n = self.norm()
        return Vector3(self.x / n, self.y / n, self.z / n)

    def __repr__(self):
        return "Vector3<%g, %g, %g>" % (self.x, self.y, self.z)


def _v3(v):
    if v is None:
        return Vector3()
    if isinstance(v, Vector3):
        return v
    return Vector3(*v)


class Volume:
    def __init__(self, center=Vector3(), size=Vector3(), dims=3, is_cylindrical=False):
        self.center, self.size, self.dims = _v3(center), _v3(size), dims


# ------------------------------------------------------------- materials
class Susceptibility:
    def __init__(self, sigma_diag=Vector3(), sigma_offdiag=Vector3(), sigma=None):
        self.sigma_diag = Vector3(sigma, sigma, sigma) if sigma else _v3(sigma_diag)
        if any(_v3(sigma_offdiag)):
            raise NotImplementedError("meep: off-diagonal susceptibility sigma is not supported by the GB300 engine")


class LorentzianSusceptibility(Susceptibility):
    """sigma * frequency^2 / (frequency^2 - omega^2 - i gamma omega), frequencies
    in units of 2 pi c / a (python/geom.py)."""

    def __init__(self, frequency=0.0, gamma=0.0, **kwargs):
        super().__init__(**kwargs)
        self.frequency, self.gamma = float(frequency), float(gamma)

    def _key(self):
        return (float(self.frequency), float(self.gamma), 0)


class DrudeSusceptibility(Susceptibility):
    """sigma * frequency^2 / (-omega^2 - i gamma omega)."""

    def __init__(self, frequency=0.0, gamma=0.0, **kwargs):
        super().__init__(**kwargs)
        self.frequency, self.gamma = float(frequency), float(gamma)

    def _key(self):
        return (float(self.frequency), float(self.gamma), 1)


class Medium:
    """Electric medium: epsilon (or index), diagonal anisotropy, D
    conductivity, Lorentzian/Drude susceptibilities (python/geom.py Medium)."""

    def __init__(self, epsilon_diag=Vector3(1, 1, 1), epsilon_offdiag=Vector3(), mu_diag=Vector3(1, 1, 1),
                 E_susceptibilities=(), H_susceptibilities=(), D_conductivity_diag=Vector3(),
                 B_conductivity_diag=Vector3(), epsilon=None, index=None, mu=None, D_conductivity=None,
                 B_conductivity=None, chi2=None, chi3=None, **kwargs):
        if epsilon:
            epsilon_diag = Vector3(epsilon, epsilon, epsilon)
        elif index:
            epsilon_diag = Vector3(index * index, index * index, index * index)
        if D_conductivity:
            D_conductivity_diag = Vector3(D_conductivity, D_conductivity, D_conductivity)
        self.epsilon_diag = _v3(epsilon_diag)
        self.D_conductivity_diag = _v3(D_conductivity_diag)
        self.E_susceptibilities = list(E_susceptibilities)
        unsupported = []
        if any(_v3(epsilon_offdiag)):
            unsupported.append("off-diagonal epsilon")
        if (mu and mu != 1) or tuple(_v3(mu_diag)) != (1, 1, 1) or H_susceptibilities:
            unsupported.append("magnetic materials")
        if (B_conductivity and B_conductivity != 0) or any(_v3(B_conductivity_diag)):
            unsupported.append("B conductivity")
        if chi2 or chi3:
            unsupported.append("nonlinear materials")
        if unsupported:
            raise NotImplementedError("meep: %s not supported by the GB300 engine" % ", ".join(unsupported))


vacuum = air = Medium(epsilon=1.0)


class MaterialGrid:
    """Material on a rectilinear grid of design weights u in [0, 1] over a
    Block (python/geom.py MaterialGrid): u is interpolated linearly to each
    point (nodes at cell centres, mirror faces), optionally projected by
    (tanh(beta eta) + tanh(beta (u - eta))) / (tanh(beta eta) + tanh(beta (1 -
    eta))), and eps = eps1 + u (eps2 - eps1) with eps1, eps2 the diagonal
    permittivities of medium1 and medium2 (src/meepgeom.cpp:489-581).  The
    engine evaluates it on the device.  Covered: the default grid type, no
    subpixel smoothing of the grid (do_averaging=False, the reference's
    default), no damping, media without susceptibilities or conductivity; a
    grid is the material of a Block.  With eps_averaging=True the pixels
    straddling the block's faces are averaged against medium1 (the reference
    evaluates the grid there)."""

    def __init__(self, grid_size, medium1, medium2, weights=None, grid_type="U_DEFAULT", do_averaging=False,
                 beta=0, eta=0.5, damping=0):
        gs = _v3(grid_size)
        self.grid_size = Vector3(*(1 if math.isclose(v, 0, abs_tol=1e-9) else int(round(v)) for v in gs))
        self.medium1, self.medium2 = medium1, medium2
        self.num_params = int(self.grid_size.x * self.grid_size.y * self.grid_size.z)
        self.do_averaging, self.beta, self.eta, self.damping = do_averaging, float(beta), float(eta), damping
        unsupported = []
        if grid_type != "U_DEFAULT":
            unsupported.append("material grid type %s" % grid_type)
        if do_averaging:
            unsupported.append("subpixel smoothing of material grids")
        if damping:
            unsupported.append("material grid damping")
        for m in (medium1, medium2):
            if m.E_susceptibilities or any(m.D_conductivity_diag):
                unsupported.append("dispersive or conductive material grid media")
                break
        if unsupported:
            raise NotImplementedError("meep: %s not supported by the GB300 engine" % ", ".join(unsupported))
        if weights is None:
            self.weights = np.zeros(self.num_params)
        elif np.asarray(weights).size != self.num_params:
            raise ValueError("weights of shape {} do not match user specified grid dimension: {}".format(
                np.asarray(weights).shape, self.grid_size))
        else:
            self.weights = self.check_weights(np.asarray(weights, dtype=np.float64).flatten())

    def check_weights(self, w):
        if np.amin(w) >= 0.0 and np.amax(w) <= 1.0:
            return w
        warnings.warn("The weights parameter of MaterialGrid must be in the range [0,1].")
        return np.clip(w, 0.0, 1.0)

    def update_weights(self, x):
        x = np.asarray(x, dtype=np.float64)
        if x.size != self.num_params:
            raise ValueError("weights of size {} do not match user specified grid dimension: {}".format(
                x.size, self.grid_size))
        self.weights[:] = self.check_weights(x).flatten()


# -------------------------------------------------------------- geometry
class GeometricObject:
    def __init__(self, material=Medium(), center=Vector3(), epsilon_func=None, label=None):
        if callable(material) and not isinstance(material, (Medium, MaterialGrid)):
            raise NotImplementedError("meep: material functions are not supported by the GB300 engine")
        self.material = material
        self.center = _v3(center)


class Block(GeometricObject):
    def __init__(self, size, e1=Vector3(1, 0, 0), e2=Vector3(0, 1, 0), e3=Vector3(0, 0, 1), **kwargs):
        super().__init__(**kwargs)
        self.size = _v3(size)
        if (tuple(_v3(e1)), tuple(_v3(e2)), tuple(_v3(e3))) != ((1, 0, 0), (0, 1, 0), (0, 0, 1)):
            raise NotImplementedError("meep: only axis-aligned blocks are supported")


class Sphere(GeometricObject):
    def __init__(self, radius, **kwargs):
        super().__init__(**kwargs)
        self.radius = float(radius)


class Cylinder(GeometricObject):
    def __init__(self, radius, axis=Vector3(0, 0, 1), height=1e20, **kwargs):
        super().__init__(**kwargs)
        self.radius, self.height, self.axis = float(radius), float(height), _v3(axis).unit()


class PML:
    def __init__(self, thickness, direction=ALL, side=ALL, R_asymptotic=1e-15, mean_stretch=1.0, pml_profile=None):
        if pml_profile is not None:
            raise NotImplementedError("meep: custom PML profiles are not supported by the GB300 engine")
        self.thickness, self.direction, self.side = float(thickness), direction, side
        self.R_asymptotic, self.mean_stretch = float(R_asymptotic), float(mean_stretch)


# --------------------------------------------------------------- sources
class SourceTime:
    def __init__(self, is_integrated=False):
        self.is_integrated = is_integrated


class GaussianSource(SourceTime):
    """gaussian_src_time(frequency, width, start_time, start_time + 2 width
    cutoff) with width = max(width, 1/fwidth) (python/source.py)."""

    def __init__(self, frequency=None, width=0, fwidth=float("inf"), start_time=0, cutoff=5.0, is_integrated=False,
                 wavelength=None, **kwargs):
        if frequency is None and wavelength is None:
            raise ValueError("Must set either frequency or wavelength in GaussianSource.")
        super().__init__(is_integrated=is_integrated)
        self.frequency = 1 / wavelength if wavelength else float(frequency)
        self.width = max(width, 1 / fwidth)
        self.start_time, self.cutoff = start_time, cutoff
        self.fwidth = 1 / self.width

    def _params(self):
        return 0, [self.frequency, self.width, self.start_time, self.start_time + 2 * self.width * self.cutoff, 0, 0]


class ContinuousSource(SourceTime):
    """continuous_src_time(frequency, width, start_time, end_time, slowness)."""

    def __init__(self, frequency=None, start_time=0, end_time=1.0e20, width=0, fwidth=float("inf"), cutoff=None,
                 slowness=3.0, is_integrated=False, wavelength=None, **kwargs):
        if frequency is None and wavelength is None:
            raise ValueError("Must set either frequency or wavelength in ContinuousSource.")
        super().__init__(is_integrated=is_integrated)
        self.frequency = 1 / wavelength if wavelength else float(frequency)
        self.start_time, self.end_time = start_time, end_time
        self.width = max(width, 1 / fwidth)
        self.slowness = cutoff if cutoff is not None else slowness

    def _params(self):
        return 1, [self.frequency, self.width, self.start_time, self.end_time, self.slowness, 0]


class Source:
    def __init__(self, src, component, center=None, volume=None, size=Vector3(), amplitude=1.0, amp_func=None,
                 **kwargs):
        if center is None and volume is None:
            raise ValueError("Source requires either center or volume")
        if amp_func is not None:
            raise NotImplementedError("meep: amp_func sources are not supported by the GB300 engine")
        self.center = volume.center if volume else _v3(center)
        self.size = volume.size if volume else _v3(size)
        self.src, self.component, self.amplitude = src, component, complex(amplitude)


class FluxRegion:
    def __init__(self, center=None, size=Vector3(), direction=AUTOMATIC, weight=1.0, volume=None):
        if center is None and volume is None:
            raise ValueError("Either center or volume required")
        self.center = volume.center if volume else _v3(center)
        self.size = volume.size if volume else _v3(size)
        self.direction, self.weight = direction, complex(weight)


# near-to-far and force surfaces are flux regions (python/simulation.py:
# Near2FarRegion = FluxRegion; a ForceRegion's direction is the force's)
Near2FarRegion = FluxRegion
ForceRegion = FluxRegion
EnergyRegion = FluxRegion


# ------------------------------------------------------------ step funcs
def _num_args(f):
    import inspect
    try:
        return len(inspect.signature(f).parameters)
    except (TypeError, ValueError):
        return 1


# Step functions (the reference's python/simulation.py:5049-5160 semantics):
# run() calls each with todo = "step" before every step and once with
# todo = "finish" after the last.  A one-argument function f(sim) only sees
# the steps; a two-argument f(sim, todo) sees both phases.  The combinators
# below are small stateful callables that decide when to pass a phase on.
def _eval_step_func(sim, func, todo):
    arity = _num_args(func)
    if arity not in (1, 2):
        raise ValueError("Step function requires 1 or 2 arguments")
    if arity == 2:
        func(sim, todo)
    elif todo == "step":
        func(sim)


class _Combinator:
    """Base of the step-function combinators: forwards a phase to the
    wrapped functions when `_due` says so."""

    def __init__(self, funcs):
        self.funcs = funcs

    def _forward(self, sim, todo):
        for func in self.funcs:
            _eval_step_func(sim, func, todo)

    def __call__(self, sim, todo):
        raise NotImplementedError


class _AtEvery(_Combinator):
    # due once `interval` has passed since the last call that ran (half a
    # time step of slack), and always at "finish"
    def __init__(self, interval, funcs):
        super().__init__(funcs)
        self.interval = interval
        self.last_run = 0.0

    def __call__(self, sim, todo):
        now = sim.round_time()
        if todo != "finish" and now < self.last_run + self.interval - 0.5 * sim.fields_dt:
            return
        self._forward(sim, todo)
        self.last_run = now


class _AtEnd(_Combinator):
    # only at "finish": one "step" call, then the "finish" call
    def __call__(self, sim, todo):
        if todo == "finish":
            self._forward(sim, "step")
            self._forward(sim, "finish")


class _AtBeginning(_Combinator):
    # only the first phase it sees
    def __init__(self, funcs):
        super().__init__(funcs)
        self.done = False

    def __call__(self, sim, todo):
        if not self.done:
            self._forward(sim, todo)
            self.done = True


class _AfterTime(_Combinator):
    # every phase from `delay` after the first call on
    def __init__(self, delay, funcs):
        super().__init__(funcs)
        self.delay = delay
        self.start = None

    def __call__(self, sim, todo):
        if self.start is None:
            self.start = sim.round_time()
        if todo == "finish" or sim.round_time() >= self.start + self.delay:
            self._forward(sim, todo)


def at_every(dt, *step_funcs):
    return _AtEvery(dt, step_funcs)


def at_end(*step_funcs):
    return _AtEnd(step_funcs)


def at_beginning(*step_funcs):
    return _AtBeginning(step_funcs)


def after_time(t, *step_funcs):
    return _AfterTime(t, step_funcs)


# ---------------------------------------------------------------- binding
class _Obj(C.Structure):
    _fields_ = [("kind", C.c_int), ("center", C.c_double * 3), ("size", C.c_double * 3), ("radius", C.c_double),
                ("height", C.c_double), ("axis", C.c_double * 3), ("material", C.c_int)]


MGB_MAX_SUS = 8


class _Med(C.Structure):
    _fields_ = [("eps", C.c_double * 3), ("d_cond", C.c_double * 3), ("nsus", C.c_int),
                ("sus", C.c_int * MGB_MAX_SUS), ("sigma", (C.c_double * 3) * MGB_MAX_SUS)]


class _Sus(C.Structure):
    _fields_ = [("frequency", C.c_double), ("gamma", C.c_double), ("drude", C.c_int)]


_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_SIGS = [
    ("mgb_create", C.c_int, [C.c_int, _DP, C.c_double, C.c_double, C.c_int, _DP, C.c_int, C.POINTER(_Med), C.c_int,
                             C.c_int, C.POINTER(_Obj), C.c_int, C.POINTER(_Sus), C.c_int, C.c_double, C.c_int,
                             C.POINTER(_P)]),
    ("mgb_destroy", None, [_P]),
    ("mgb_last_error", C.c_char_p, []),
    ("mgb_add_source", C.c_int, [_P, C.c_int, C.c_int, _DP, C.c_int, _DP, _DP, C.c_double, C.c_double]),
    ("mgb_last_source_time", C.c_double, [_P]),
    ("mgb_add_flux", C.c_int, [_P, C.c_int, _DP, C.c_int, _DP, C.c_int, C.POINTER(C.c_int)]),
    ("mgb_flux", C.c_int, [_P, C.c_int, _DP]),
    ("mgb_add_dft_fields", C.c_int, [_P, C.c_int, C.POINTER(C.c_int), _DP, _DP, C.c_int, _DP, C.c_int, C.c_int,
                                     C.POINTER(C.c_int)]),
    ("mgb_dft_fields_array", C.c_int, [_P, C.c_int, C.c_int, C.c_int, _DP, C.POINTER(C.c_int)]),
    ("mgb_step", C.c_int, [_P, C.c_int]),
    ("mgb_time", C.c_int, [_P, _DP, _DP, _DP, C.POINTER(C.c_int)]),
    ("mgb_get_field_points", C.c_int, [_P, C.c_int, C.c_int, _DP, _DP, _DP]),
    ("mgb_get_epsilon_points", C.c_int, [_P, C.c_int, _DP, _DP]),
    ("mgb_yee_array", C.c_int, [_P, C.c_int, C.c_int, _DP, C.POINTER(C.c_longlong)]),
    ("mgb_use_bloch", C.c_int, [_P, _DP]),
    ("mgb_add_material_grid", C.c_int, [_P, _DP, _DP, C.POINTER(C.c_int), _DP, C.c_double, C.c_double, _DP, _DP]),
    ("mgb_flux_data", C.c_int, [_P, C.c_int, C.c_int, _DP, C.POINTER(C.c_size_t)]),
    ("mgb_load_flux_data", C.c_int, [_P, C.c_int, C.c_int, _DP, C.c_size_t]),
    ("mgb_flux_scale", C.c_int, [_P, C.c_int, C.c_double, C.c_double]),
    ("mgb_dft_data", C.c_int, [_P, C.c_int, C.c_int, C.c_int, _DP, C.POINTER(C.c_size_t)]),
    ("mgb_load_dft_data", C.c_int, [_P, C.c_int, C.c_int, C.c_int, _DP, C.c_size_t]),
    ("mgb_scale_dft_data", C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double]),
    ("mgb_ldos_create", C.c_int, [_P, C.c_int, _DP, C.POINTER(C.c_int)]),
    ("mgb_ldos_update", C.c_int, [_P, C.c_int]),
    ("mgb_ldos_results", C.c_int, [_P, C.c_int, _DP, _DP, _DP]),
    ("mgb_add_energy", C.c_int, [_P, C.c_int, _DP, C.c_int, _DP, C.c_int, C.POINTER(C.c_int)]),
    ("mgb_energy", C.c_int, [_P, C.c_int, C.c_int, _DP]),
    ("mgb_add_force", C.c_int, [_P, C.c_int, _DP, C.c_int, _DP, C.c_int, C.POINTER(C.c_int)]),
    ("mgb_force", C.c_int, [_P, C.c_int, _DP]),
    ("mgb_add_near2far", C.c_int, [_P, C.c_int, _DP, C.c_int, _DP, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    ("mgb_near2far_points", C.c_int, [_P, C.c_int, C.c_int, _DP, _DP]),
    ("mgb_near2far_array", C.c_int, [_P, C.c_int, _DP, _DP, C.c_double, _DP, C.POINTER(C.c_int),
                                     C.POINTER(C.c_int)]),
    ("mgb_near2far_flux", C.c_int, [_P, C.c_int, C.c_int, _DP, _DP, C.c_double, _DP]),
    ("mgb_near2far_scale", C.c_int, [_P, C.c_int, C.c_double, C.c_double]),
    ("mgb_near2far_medium", C.c_int, [_P, C.c_int, _DP, _DP]),
]

_LIBS = {}


def _load(path):
    path = os.path.abspath(path)
    if path not in _LIBS:
        if not os.path.exists(path):
            raise RuntimeError("meep: native library %s is missing; run __graft_entry__.build()" % path)
        lib = C.CDLL(path, mode=C.RTLD_LOCAL)
        for name, res, args in _SIGS:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIBS[path] = lib
    return _LIBS[path]


def _arr(vals):
    a = np.ascontiguousarray(np.asarray(vals, dtype=np.float64))
    return a, a.ctypes.data_as(_DP)


class DftFlux:
    def __init__(self, sim, handle, freq):
        self.sim, self.handle, self.freq = sim, handle, list(freq)


class DftFields:
    def __init__(self, sim, handle, freq, components):
        self.sim, self.handle, self.freq, self.components = sim, handle, list(freq), list(components)


# python/simulation.py FluxData: the E and H DFT sums of a flux object
FluxData = collections.namedtuple("FluxData", ["E", "H"])
ForceData = collections.namedtuple("ForceData", ["offdiag1", "offdiag2", "diag"])
NearToFarData = collections.namedtuple("NearToFarData", ["F"])


class DftEnergy:
    def __init__(self, sim, handle, freq):
        self.sim, self.handle, self.freq = sim, handle, list(freq)

    def _get(self, which):
        out = np.zeros(len(self.freq))
        self.sim._check(self.sim._lib.mgb_energy(self.sim._h, self.handle, which, out.ctypes.data_as(_DP)))
        return list(out)


class DftForce:
    def __init__(self, sim, handle, freq):
        self.sim, self.handle, self.freq = sim, handle, list(freq)


class DftNear2Far:
    """Near-to-far transform object (python/simulation.py DftNear2Far): the
    DFTs of the tangential fields on its regions, far fields by the
    homogeneous-medium Green's function, evaluated on the GPU."""

    def __init__(self, sim, handle, freq, nperiods, regions):
        self.sim, self.handle, self.freq = sim, handle, list(freq)
        self.nfreqs, self.nperiods, self.regions = len(self.freq), nperiods, list(regions)

    def _medium(self):
        e, m = C.c_double(), C.c_double()
        self.sim._check(self.sim._lib.mgb_near2far_medium(self.sim._h, self.handle, C.byref(e), C.byref(m)))
        return e.value, m.value

    @property
    def eps(self):
        return self._medium()[0]

    @property
    def mu(self):
        return self._medium()[1]

    def flux(self, direction=None, where=None, resolution=None):
        """Poynting flux in `direction` of the far fields on a grid over the
        Volume `where` at `resolution` (a list of nfreq values)."""
        out = np.zeros(self.nfreqs)
        c_a, c_p = _arr(list(where.center))
        z_a, z_p = _arr(list(where.size))
        self.sim._check(self.sim._lib.mgb_near2far_flux(self.sim._h, self.handle, int(direction), c_p, z_p,
                                                        float(resolution), out.ctypes.data_as(_DP)))
        return list(out)

    def scale_dfts(self, s):
        s = complex(s)
        self.sim._check(self.sim._lib.mgb_near2far_scale(self.sim._h, self.handle, s.real, s.imag))


def _fix_dft_args(args, i):
    """fcen, df, nfreq (3 numbers) or a frequency array (python/simulation.py
    fix_dft_args)."""
    if (len(args) > i + 2 and isinstance(args[i], (int, float)) and isinstance(args[i + 1], (int, float))
            and isinstance(args[i + 2], int)):
        fcen, df, nfreq = args[i], args[i + 1], args[i + 2]
        freq = [fcen] if nfreq == 1 else np.linspace(fcen - 0.5 * df, fcen + 0.5 * df, nfreq)
        return args[:i] + (freq,) + args[i + 3:]
    if not isinstance(args[i], (np.ndarray, list)):
        raise TypeError("add_dft functions only accept fcen,df,nfreq (3 numbers) or freq (array/list)")
    return args


_IGNORED_KWARGS = {"progress_interval", "split_chunks_evenly", "num_chunks", "chunk_layout", "filename_prefix",
                   "output_volume", "output_single_precision", "collect_stats", "ensure_periodicity",
                   "accurate_fields_near_cylorigin", "loop_tile_base_db", "loop_tile_base_eh"}


class Simulation:
    """The reference's `meep.Simulation` for the stepping path (see the module
    docstring for what is supported)."""

    def __init__(self, cell_size, resolution, geometry=None, sources=None, eps_averaging=True, dimensions=3,
                 boundary_layers=None, symmetries=None, force_complex_fields=False, default_material=Medium(),
                 k_point=False, Courant=0.5, geometry_center=Vector3(), subpixel_tol=1e-4,
                 subpixel_maxeval=100000, _library=None, **kwargs):
        bad = set(kwargs) - _IGNORED_KWARGS
        if bad:
            raise TypeError("Simulation got unexpected keyword arguments %s" % sorted(bad))
        self.eps_averaging = bool(eps_averaging)
        self.subpixel_tol = float(subpixel_tol)
        self.subpixel_maxeval = int(subpixel_maxeval)
        if self.eps_averaging:
            for g in geometry or []:
                m = getattr(g, "material", None)
                if isinstance(m, Medium) and len(set(m.epsilon_diag)) > 1:
                    raise NotImplementedError("meep: subpixel averaging of anisotropic media is not supported by "
                                              "the GB300 engine; pass eps_averaging=False")
        if symmetries:
            raise NotImplementedError("meep: symmetries are not supported by the GB300 engine")
        if force_complex_fields:
            raise NotImplementedError("meep: complex fields are not supported by the GB300 engine")
        if any(_v3(geometry_center)):
            raise NotImplementedError("meep: geometry_center must be the origin")
        self.cell_size = _v3(cell_size)
        self.resolution = float(resolution)
        self.dimensions = dimensions
        if dimensions == 3 and self.cell_size.z == 0:
            self.dimensions = 2
        self.geometry = list(geometry or [])
        self.sources = list(sources or [])
        self.boundary_layers = list(boundary_layers or [])
        self.default_material = default_material
        self.k_point = _v3(k_point) if k_point not in (False, None) else False
        self.Courant = float(Courant)
        self.dft_objects = []
        self._lib = _load(_library or _product_lib())
        self._h = None

    # -------------------------------------------------------------- setup
    def init_sim(self):
        if self._h is not None:
            return
        if isinstance(self.default_material, MaterialGrid):
            raise NotImplementedError("meep: a material grid as the default material is not supported by the "
                                      "GB300 engine; put it in a Block")
        media = [self.default_material]
        index = {id(self.default_material): 0}
        grids = []
        for g in self.geometry:
            mat = g.material
            if isinstance(mat, MaterialGrid):
                if not isinstance(g, Block):
                    raise NotImplementedError("meep: a material grid must be the material of a Block")
                grids.append(g)
                mat = mat.medium1  # the block's faces average against medium1
            if id(mat) not in index:
                index[id(mat)] = len(media)
                media.append(mat)
        sus_keys = []
        for m in media:
            for s in m.E_susceptibilities:
                if s._key() not in sus_keys:
                    sus_keys.append(s._key())
        med = (_Med * len(media))()
        for q, m in enumerate(media):
            med[q].eps[:] = list(m.epsilon_diag)
            med[q].d_cond[:] = list(m.D_conductivity_diag)
            if len(m.E_susceptibilities) > MGB_MAX_SUS:
                raise NotImplementedError("meep: at most %d susceptibilities per medium" % MGB_MAX_SUS)
            med[q].nsus = len(m.E_susceptibilities)
            for k, s in enumerate(m.E_susceptibilities):
                med[q].sus[k] = sus_keys.index(s._key())
                med[q].sigma[k][:] = list(s.sigma_diag)
        objs = (_Obj * max(1, len(self.geometry)))()
        for q, g in enumerate(self.geometry):
            o = objs[q]
            o.center[:] = list(g.center)
            o.material = index[id(g.material.medium1 if isinstance(g.material, MaterialGrid) else g.material)]
            if isinstance(g, Block):
                o.kind = 0
                o.size[:] = list(g.size)
            elif isinstance(g, Sphere):
                o.kind, o.radius = 1, g.radius
            elif isinstance(g, Cylinder):
                o.kind, o.radius, o.height = 2, g.radius, g.height
                o.axis[:] = list(g.axis)
            else:
                raise NotImplementedError("meep: geometric object %s is not supported" % type(g).__name__)
        sus = (_Sus * max(1, len(sus_keys)))()
        for q, (f, g, dr) in enumerate(sus_keys):
            sus[q].frequency, sus[q].gamma, sus[q].drude = f, g, dr
        rows = []
        for layer in self.boundary_layers:
            if not isinstance(layer, PML):
                raise NotImplementedError("meep: only PML boundary layers are supported")
            rows.append([layer.thickness, layer.direction, layer.side, layer.R_asymptotic, layer.mean_stretch])
        pml_a, pml_p = _arr(np.array(rows, dtype=np.float64).reshape(-1) if rows else [0.0])
        cell_a, cell_p = _arr(list(self.cell_size))
        h = _P()
        self._check(self._lib.mgb_create(self.dimensions, cell_p, self.resolution, self.Courant, len(rows), pml_p,
                                         len(media), med, 0, len(self.geometry), objs, len(sus_keys), sus,
                                         int(self.eps_averaging), self.subpixel_tol, self.subpixel_maxeval,
                                         C.byref(h)))
        self._h = h
        for g in grids:
            m = g.material
            n = (C.c_int * 3)(*(int(v) for v in m.grid_size))
            c_a, c_p = _arr(list(g.center))
            z_a, z_p = _arr(list(g.size))
            w_a, w_p = _arr(m.weights)
            e1_a, e1_p = _arr(list(m.medium1.epsilon_diag))
            e2_a, e2_p = _arr(list(m.medium2.epsilon_diag))
            self._check(self._lib.mgb_add_material_grid(self._h, c_p, z_p, n, w_p, m.beta, m.eta, e1_p, e2_p))
        if self.k_point is not False:
            # Bloch-periodic walls in every direction (Simulation._init_fields);
            # complex fields when k != 0
            k_a, k_p = _arr(list(self.k_point))
            self._check(self._lib.mgb_use_bloch(self._h, k_p))
        for s in self.sources:
            kind, params = s.src._params()
            p_a, p_p = _arr(params)
            c_a, c_p = _arr(list(s.center))
            z_a, z_p = _arr(list(s.size))
            self._check(self._lib.mgb_add_source(self._h, s.component, kind, p_p, int(bool(s.src.is_integrated)), c_p,
                                                 z_p, s.amplitude.real, s.amplitude.imag))

    def _check(self, status):
        if status != 0:
            raise RuntimeError(self._lib.mgb_last_error().decode())

    def __del__(self):
        if getattr(self, "_h", None) is not None:
            self._lib.mgb_destroy(self._h)
            self._h = None

    # ----------------------------------------------------------- monitors
    def add_flux(self, *args, **kwargs):
        args = _fix_dft_args(args, 0)
        freq, regions = list(np.asarray(args[0], dtype=np.float64)), args[1:]
        decimation = int(kwargs.get("decimation_factor", 0))
        self.init_sim()
        rows = []
        for r in regions:
            if r.weight.imag != 0:
                raise NotImplementedError("meep: complex flux weights are not supported")
            rows += list(r.center) + list(r.size) + [r.direction, r.weight.real]
        r_a, r_p = _arr(rows)
        f_a, f_p = _arr(freq)
        h = C.c_int()
        self._check(self._lib.mgb_add_flux(self._h, len(regions), r_p, len(freq), f_p, decimation, C.byref(h)))
        flux = DftFlux(self, h.value, freq)
        self.dft_objects.append(flux)
        return flux

    def _flux_part(self, flux, part):
        n = C.c_size_t()
        self._check(self._lib.mgb_flux_data(self._h, flux.handle, part, None, C.byref(n)))
        out = np.zeros(2 * n.value)
        self._check(self._lib.mgb_flux_data(self._h, flux.handle, part, out.ctypes.data_as(_DP), C.byref(n)))
        return out[0::2] + 1j * out[1::2]

    def get_flux_data(self, flux):
        """The flux object's DFT sums as FluxData(E, H) (complex arrays, chunk
        after chunk), for load_flux_data / load_minus_flux_data."""
        return FluxData(E=self._flux_part(flux, 0), H=self._flux_part(flux, 1))

    def load_flux_data(self, flux, fdata):
        """Replace the flux object's DFT sums by fdata (from get_flux_data of a
        simulation with the same cell and regions); later steps add to them."""
        for part, arr in ((0, fdata.E), (1, fdata.H)):
            arr = np.asarray(arr, dtype=np.complex128)
            ri = np.ascontiguousarray(np.stack([arr.real, arr.imag], axis=-1).reshape(-1))
            self._check(self._lib.mgb_load_flux_data(self._h, flux.handle, part, ri.ctypes.data_as(_DP), arr.size))

    def load_minus_flux_data(self, flux, fdata):
        """As load_flux_data, then negate: the loaded fields are subtracted
        from what the run accumulates (the reflected-flux normalisation)."""
        self.load_flux_data(flux, fdata)
        scale_flux_fields(-1.0, flux)

    def add_energy(self, *args, **kwargs):
        """add_energy(fcen, df, nfreq | freq, *EnergyRegions, decimation_factor=0):
        electric and magnetic energy spectra in the regions
        (python/simulation.py Simulation.add_energy)."""
        args = _fix_dft_args(args, 0)
        freq, regions = list(np.asarray(args[0], dtype=np.float64)), args[1:]
        decimation = int(kwargs.get("decimation_factor", 0))
        self.init_sim()
        rows = []
        for r in regions:
            rows += list(r.center) + list(r.size) + [r.direction, r.weight.real]
        r_a, r_p = _arr(rows)
        f_a, f_p = _arr(freq)
        h = C.c_int()
        self._check(self._lib.mgb_add_energy(self._h, len(regions), r_p, len(freq), f_p, decimation, C.byref(h)))
        energy = DftEnergy(self, h.value, freq)
        self.dft_objects.append(energy)
        return energy

    # force and near2far data (python/simulation.py get_force_data,
    # load_force_data, load_minus_force_data, get_near2far_data, ...)
    def _dft_parts(self, kind, obj, nparts):
        out = []
        for part in range(nparts):
            n = C.c_size_t()
            self._check(self._lib.mgb_dft_data(self._h, kind, obj.handle, part, None, C.byref(n)))
            a = np.zeros(2 * n.value)
            self._check(self._lib.mgb_dft_data(self._h, kind, obj.handle, part, a.ctypes.data_as(_DP), C.byref(n)))
            out.append(a[0::2] + 1j * a[1::2])
        return out

    def _load_parts(self, kind, obj, arrays, minus):
        for part, arr in enumerate(arrays):
            arr = np.asarray(arr, dtype=np.complex128)
            ri = np.ascontiguousarray(np.stack([arr.real, arr.imag], axis=-1).reshape(-1))
            self._check(self._lib.mgb_load_dft_data(self._h, kind, obj.handle, part, ri.ctypes.data_as(_DP),
                                                    arr.size))
            if minus:
                self._check(self._lib.mgb_scale_dft_data(self._h, kind, obj.handle, part, -1.0, 0.0))

    def get_force_data(self, force):
        return ForceData(*self._dft_parts(1, force, 3))

    def load_force_data(self, force, fdata):
        self._load_parts(1, force, [fdata.offdiag1, fdata.offdiag2, fdata.diag], False)

    def load_minus_force_data(self, force, fdata):
        self._load_parts(1, force, [fdata.offdiag1, fdata.offdiag2, fdata.diag], True)

    def get_near2far_data(self, near2far):
        return NearToFarData(*self._dft_parts(2, near2far, 1))

    def load_near2far_data(self, near2far, n2fdata):
        self._load_parts(2, near2far, [n2fdata.F], False)

    def load_minus_near2far_data(self, near2far, n2fdata):
        self._load_parts(2, near2far, [n2fdata.F], True)

    def add_force(self, *args, **kwargs):
        """add_force(fcen, df, nfreq | freq, *ForceRegions, decimation_factor=0):
        the Maxwell-stress force along each region's direction
        (python/simulation.py Simulation.add_force)."""
        args = _fix_dft_args(args, 0)
        freq, regions = list(np.asarray(args[0], dtype=np.float64)), args[1:]
        decimation = int(kwargs.get("decimation_factor", 0))
        self.init_sim()
        rows = []
        for r in regions:
            if r.weight.imag != 0:
                raise NotImplementedError("meep: complex force weights are not supported")
            rows += list(r.center) + list(r.size) + [r.direction, r.weight.real]
        r_a, r_p = _arr(rows)
        f_a, f_p = _arr(freq)
        h = C.c_int()
        self._check(self._lib.mgb_add_force(self._h, len(regions), r_p, len(freq), f_p, decimation, C.byref(h)))
        force = DftForce(self, h.value, freq)
        self.dft_objects.append(force)
        return force

    def add_near2far(self, *args, **kwargs):
        """add_near2far(fcen, df, nfreq | freq, *Near2FarRegions, nperiods=1,
        decimation_factor=0): the DFTs of the tangential fields on the regions
        (python/simulation.py Simulation.add_near2far)."""
        args = _fix_dft_args(args, 0)
        freq, regions = list(np.asarray(args[0], dtype=np.float64)), args[1:]
        nperiods = int(kwargs.get("nperiods", 1))
        decimation = int(kwargs.get("decimation_factor", 0))
        self.init_sim()
        rows = []
        for r in regions:
            if r.weight.imag != 0:
                raise NotImplementedError("meep: complex near2far weights are not supported")
            rows += list(r.center) + list(r.size) + [r.direction, r.weight.real]
        r_a, r_p = _arr(rows)
        f_a, f_p = _arr(freq)
        h = C.c_int()
        self._check(self._lib.mgb_add_near2far(self._h, len(regions), r_p, len(freq), f_p, decimation, nperiods,
                                               C.byref(h)))
        n2f = DftNear2Far(self, h.value, freq, nperiods, regions)
        self.dft_objects.append(n2f)
        return n2f

    def _farfields_at(self, near2far, points):
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
        out = np.zeros((pts.shape[0], near2far.nfreqs, 6, 2))
        self._check(self._lib.mgb_near2far_points(self._h, near2far.handle, pts.shape[0], pts.ctypes.data_as(_DP),
                                                  out.ctypes.data_as(_DP)))
        return out[..., 0] + 1j * out[..., 1]

    def get_farfield(self, near2far, x, greencyl_tol=1e-3):
        """Far fields at the Vector3 x: a list of 6 nfreq complex values
        (Ex, Ey, Ez, Hx, Hy, Hz for each frequency in turn)."""
        self.init_sim()
        return list(self._farfields_at(near2far, [list(_v3(x))]).ravel())

    def get_farfields_at(self, near2far, points):
        """Far fields at many points (an n x 3 array) in one GPU call: an
        array (n, nfreq, 6) of complex Ex..Hz (an extension of get_farfield)."""
        self.init_sim()
        return self._farfields_at(near2far, points)

    def get_farfields(self, near2far, resolution=None, where=None, center=None, size=None, greencyl_tol=1e-3):
        """Far fields on a grid over a volume at `resolution`: a dict of
        arrays Ex..Hz shaped (points per non-singleton direction..., nfreq),
        the frequency axis only when nfreq > 1 (python/simulation.py
        get_farfields)."""
        self.init_sim()
        if where is not None:
            center, size = where.center, where.size
        c_a, c_p = _arr(list(_v3(center)))
        z_a, z_p = _arr(list(_v3(size)))
        dims = (C.c_int * 3)()
        rank = C.c_int()
        self._check(self._lib.mgb_near2far_array(self._h, near2far.handle, c_p, z_p, float(resolution), None, dims,
                                                 C.byref(rank)))
        npts = int(np.prod([dims[i] for i in range(3)]))
        out = np.zeros(12 * npts * near2far.nfreqs)
        self._check(self._lib.mgb_near2far_array(self._h, near2far.handle, c_p, z_p, float(resolution),
                                                 out.ctypes.data_as(_DP), dims, C.byref(rank)))
        shape = [dims[i] for i in range(rank.value) if dims[i] > 1]
        if near2far.nfreqs > 1:
            shape.append(near2far.nfreqs)
        arr = out.reshape(12, -1)
        names = ["Ex", "Ey", "Ez", "Hx", "Hy", "Hz"]
        return {n: (arr[2 * k] + 1j * arr[2 * k + 1]).reshape(shape) for k, n in enumerate(names)}

    def add_dft_fields(self, components, *args, where=None, center=None, size=None, yee_grid=False,
                       decimation_factor=0, persist=False):
        if persist:
            raise NotImplementedError("meep: persistent DFT fields are not supported by the GB300 engine")
        args = _fix_dft_args(args, 0)
        freq = list(np.asarray(args[0], dtype=np.float64))
        if where is not None:
            center, size = where.center, where.size
        center = _v3(center) if center is not None else Vector3()
        size = _v3(size) if size is not None else self.cell_size
        self.init_sim()
        comps = (C.c_int * len(components))(*components)
        c_a, c_p = _arr(list(center))
        z_a, z_p = _arr(list(size))
        f_a, f_p = _arr(freq)
        h = C.c_int()
        self._check(self._lib.mgb_add_dft_fields(self._h, len(components), comps, c_p, z_p, len(freq), f_p,
                                                 int(bool(yee_grid)), int(decimation_factor), C.byref(h)))
        d = DftFields(self, h.value, freq, components)
        self.dft_objects.append(d)
        return d

    def get_dft_array(self, dft_obj, component, num_freq):
        shape = (C.c_int * 3)()
        self._check(self._lib.mgb_dft_fields_array(self._h, dft_obj.handle, component, num_freq, None, shape))
        n = shape[0] * shape[1] * shape[2]
        out = np.zeros(2 * n)
        self._check(self._lib.mgb_dft_fields_array(self._h, dft_obj.handle, component, num_freq,
                                                   out.ctypes.data_as(_DP), shape))
        arr = (out[0::2] + 1j * out[1::2]).reshape(tuple(shape))
        return np.squeeze(arr)

    # ------------------------------------------------------------ stepping
    def _time(self):
        t, rt, dt, it = C.c_double(), C.c_double(), C.c_double(), C.c_int()
        self._lib.mgb_time(self._h, C.byref(t), C.byref(rt), C.byref(dt), C.byref(it))
        return t.value, rt.value, dt.value, it.value

    def round_time(self):
        self.init_sim()
        return self._time()[1]

    def meep_time(self):
        self.init_sim()
        return self._time()[0]

    def timestep(self):
        self.init_sim()
        return self._time()[3]

    @property
    def fields_dt(self):
        self.init_sim()
        return self._time()[2]

    def _steps_until(self, stop):
        """Number of steps until round_time() >= stop (float(t * dt), the
        reference's round_time)."""
        _, _, dt, t0 = self._time()
        n = 0
        while float(np.float32((t0 + n) * dt)) < stop:
            n += 1
        return n

    def _run_until(self, cond, step_funcs):
        self.init_sim()
        conds = cond if isinstance(cond, list) else [cond]
        t0 = self.round_time()
        stops, funcs = [], []
        for c in conds:
            if isinstance(c, numbers.Number):
                stops.append(t0 + c)
            else:
                funcs.append(c)
        if not funcs and not step_funcs:
            # numeric stopping times only: one batched engine call
            n = self._steps_until(min(stops))
            self._check(self._lib.mgb_step(self._h, n))
        else:
            # every condition is evaluated on every step, as the reference's
            # list comprehension does (stateful conditions sample each step)
            while not any([self.round_time() >= s for s in stops] + [f(self) for f in funcs]):
                for func in step_funcs:
                    _eval_step_func(self, func, "step")
                self._check(self._lib.mgb_step(self._h, 1))
        for func in step_funcs:
            _eval_step_func(self, func, "step")
        for func in step_funcs:
            _eval_step_func(self, func, "finish")

    def _run_sources_until(self, cond, step_funcs):
        self.init_sim()
        conds = cond if isinstance(cond, list) else [cond]
        ts = self._lib.mgb_last_source_time(self._h)
        new = []
        for c in conds:
            if isinstance(c, numbers.Number):
                new.append((ts - self.round_time()) + c)
            else:
                new.append(lambda sim, c=c: c(sim) and sim.round_time() >= ts)
        self._run_until(new, step_funcs)

    def run(self, *step_funcs, until=None, until_after_sources=None):
        self.init_sim()
        if until_after_sources is not None:
            self._run_sources_until(until_after_sources, step_funcs)
        elif until is not None:
            self._run_until(until, step_funcs)
        else:
            raise ValueError("Invalid run configuration")

    # ------------------------------------------------------------- fields
    def get_field_point(self, c, pt):
        self.init_sim()
        p_a, p_p = _arr(list(_v3(pt)))
        re, im = np.zeros(1), np.zeros(1)
        self._check(self._lib.mgb_get_field_points(self._h, c, 1, p_p, re.ctypes.data_as(_DP), im.ctypes.data_as(_DP)))
        return complex(re[0], im[0])

    def get_epsilon_point(self, pt, frequency=0.0):
        self.init_sim()
        p_a, p_p = _arr(list(_v3(pt)))
        e = np.zeros(1)
        self._check(self._lib.mgb_get_epsilon_points(self._h, 1, p_p, e.ctypes.data_as(_DP)))
        return float(e[0])

    def get_array(self, component=None, center=None, size=None, cmplx=False):
        """Field values on the grid points x = center - size/2 + i/resolution
        covering the volume (one point along zero-size directions),
        interpolated from the Yee grid as fields::get_field does."""
        self.init_sim()
        center = _v3(center) if center is not None else Vector3()
        size = _v3(size) if size is not None else self.cell_size
        axes = []
        for d in range(3):
            present = (self.dimensions == 3) or (self.dimensions == 2 and d < 2) or (self.dimensions == 1 and d == 2)
            if not present or size[d] == 0:
                axes.append(np.array([center[d]]))
            else:
                n = int(round(size[d] * self.resolution))
                axes.append(center[d] - 0.5 * size[d] + np.arange(n + 1) / self.resolution)
        grid = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1).reshape(-1, 3)
        g_a = np.ascontiguousarray(grid)
        re, im = np.zeros(len(grid)), np.zeros(len(grid))
        self._check(self._lib.mgb_get_field_points(self._h, component, len(grid), g_a.ctypes.data_as(_DP),
                                                   re.ctypes.data_as(_DP), im.ctypes.data_as(_DP)))
        shape = tuple(len(a) for a in axes)
        out = (re + 1j * im) if cmplx else re
        return np.squeeze(out.reshape(shape))


    def get_yee_array(self, component, cmplx=False):
        """Component `component` at every point of its own Yee grid over the
        whole cell (N_d + 1 points per direction, x slowest): the values the
        engine stores, without interpolation (an addition to the reference's
        interface)."""
        self.init_sim()
        n = C.c_longlong()
        self._check(self._lib.mgb_yee_array(self._h, component, 0, None, C.byref(n)))
        out = np.zeros(n.value)
        self._check(self._lib.mgb_yee_array(self._h, component, 0, out.ctypes.data_as(_DP), C.byref(n)))
        if cmplx:
            im = np.zeros(n.value)
            self._check(self._lib.mgb_yee_array(self._h, component, 1, im.ctypes.data_as(_DP), C.byref(n)))
            out = out + 1j * im
        dims = [d for d in range(3) if (self.dimensions == 3 or (self.dimensions == 2 and d < 2)
                                         or (self.dimensions == 1 and d == 2))]
        shape = tuple(int(round(self.cell_size[d] * self.resolution)) + 1 for d in dims)
        return out.reshape(shape) if int(np.prod(shape)) == out.size else out


def get_fluxes(f):
    sim = f.sim
    out = np.zeros(len(f.freq))
    sim._check(sim._lib.mgb_flux(sim._h, f.handle, out.ctypes.data_as(_DP)))
    return list(out)


def get_flux_freqs(f):
    return list(f.freq)


def get_near2far_freqs(f):
    return list(f.freq)


def scale_near2far_fields(s, near2far):
    near2far.scale_dfts(s)


def stop_when_fields_decayed(dt=None, c=None, pt=None, decay_by=None, sampling_interval=1):
    """Condition for Simulation.run: keep running in windows of dt time units
    until the largest |c(pt)|^2 of the last window is below decay_by times
    the largest of all earlier windows (python/simulation.py
    stop_when_fields_decayed); the field is sampled every sampling_interval
    steps."""
    if dt is None or c is None or pt is None or decay_by is None:
        raise ValueError("dt, c, pt, and decay_by are all required.")
    if not isinstance(sampling_interval, numbers.Integral) or sampling_interval < 1:
        raise ValueError("sampling_interval must be a positive integer.")
    state = {"max_abs": 0, "cur_max": 0, "t0": 0}

    def _stop(sim):
        if sim.timestep() % sampling_interval == 0:
            state["cur_max"] = max(state["cur_max"], abs(sim.get_field_point(c, pt)) ** 2)
        if sim.round_time() <= dt + state["t0"]:
            return False
        old = state["cur_max"]
        state["cur_max"] = 0
        state["t0"] = sim.round_time()
        state["max_abs"] = max(state["max_abs"], old)
        return old <= state["max_abs"] * decay_by

    return _stop


def get_forces(f):
    sim = f.sim
    out = np.zeros(len(f.freq))
    sim._check(sim._lib.mgb_force(sim._h, f.handle, out.ctypes.data_as(_DP)))
    return list(out)


def get_force_freqs(f):
    return list(f.freq)


def scale_flux_fields(s, flux):
    """Multiply the flux object's DFT sums by the complex number s."""
    s = complex(s)
    flux.sim._check(flux.sim._lib.mgb_flux_scale(flux.sim._h, flux.handle, s.real, s.imag))


def get_electric_energy(f):
    return f._get(0)


def get_magnetic_energy(f):
    return f._get(1)


def get_total_energy(f):
    return f._get(2)


def get_energy_freqs(f):
    return list(f.freq)


class Ldos:
    """Frequencies of a local-density-of-states spectrum (python/simulation.py
    Ldos(fcen, df, nfreq) or Ldos(freq)); pass it to dft_ldos(ldos=...)."""

    def __init__(self, *args):
        self.freq = list(np.asarray(_fix_dft_args(args, 0)[0], dtype=np.float64))
        self.handle = None


def get_ldos_freqs(l):
    return list(l.freq)


def dft_ldos(*args, **kwargs):
    """Step function: the power spectrum of the sources normalised to the
    LDOS (python/simulation.py dft_ldos).  After the run, sim.ldos_data holds
    the spectrum and sim.ldos_Fdata / sim.ldos_Jdata the DFTs of E.J* and of
    the source current."""
    ldos = kwargs.get("ldos", None)
    if ldos is None:
        if not args and "freq" in kwargs:
            args = (kwargs["freq"],)
        elif not args:
            args = (kwargs.get("fcen"), kwargs.get("df"), kwargs.get("nfreq"))
        ldos = Ldos(*args)

    def _ldos(sim, todo):
        if ldos.handle is None:
            h = C.c_int()
            f_a, f_p = _arr(ldos.freq)
            sim._check(sim._lib.mgb_ldos_create(sim._h, len(ldos.freq), f_p, C.byref(h)))
            ldos.handle = h.value
        if todo == "step":
            sim._check(sim._lib.mgb_ldos_update(sim._h, ldos.handle))
        else:
            nf = len(ldos.freq)
            out, F, J = np.zeros(nf), np.zeros(2 * nf), np.zeros(2 * nf)
            sim._check(sim._lib.mgb_ldos_results(sim._h, ldos.handle, out.ctypes.data_as(_DP),
                                                 F.ctypes.data_as(_DP), J.ctypes.data_as(_DP)))
            sim.ldos_data = list(out)
            sim.ldos_Fdata = list(F[0::2] + 1j * F[1::2])
            sim.ldos_Jdata = list(J[0::2] + 1j * J[1::2])

    return _ldos
