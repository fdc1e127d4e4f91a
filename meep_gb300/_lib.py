"""ctypes binding of the C ABI declared in include/mfd.h.

`Engine(path)` loads a library that exports the C ABI: the CUDA engine
meep_gb300/lib/libmfd.so (the product) or, in the tests, the CPU oracle
oracle/_build/liboracle_mfd.so.  `Sim` wraps one simulation handle with numpy
arrays in and out.  Errors raise MeepError with the library's message, as the
reference's Python layer raises on meep::abort.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PRODUCT_LIB = os.path.join(HERE, "lib", "libmfd.so")

E, H, D, B = 0, 1, 2, 3
X, Y, Z = 0, 1, 2


def comp(ftype, d):
    return 3 * ftype + d


class MeepError(RuntimeError):
    pass


class mfd_grid(C.Structure):
    _fields_ = [
        ("dim", C.c_int),
        ("n", C.c_int * 3),
        ("io", C.c_int * 3),
        ("a", C.c_double),
        ("courant", C.c_double),
        ("pml_thickness", (C.c_double * 2) * 3),
        ("pml_R", (C.c_double * 2) * 3),
        ("pml_stretch", (C.c_double * 2) * 3),
        ("precision", C.c_int),
        ("components", C.c_int),
    ]


class mfd_object(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("center", C.c_double * 3),
        ("size", C.c_double * 3),
        ("radius", C.c_double),
        ("height", C.c_double),
        ("axis", C.c_double * 3),
        ("eps", C.c_double),
    ]


# (name, restype, argtypes) of every entry point in include/mfd.h
_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
SIGNATURES = [
    ("mfd_create", C.c_int, [C.POINTER(mfd_grid), C.POINTER(_P)]),
    ("mfd_destroy", None, [_P]),
    ("mfd_last_error", C.c_char_p, []),
    ("mfd_set_chi1inv", C.c_int, [_P, C.c_int, C.c_int, _DP]),
    ("mfd_set_conductivity", C.c_int, [_P, C.c_int, _DP]),
    ("mfd_add_lorentzian", C.c_int, [_P, C.c_int, C.c_double, C.c_double, C.c_int, C.POINTER(_DP)]),
    ("mfd_add_gaussian_src", C.c_int,
     [_P, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, _IP]),
    ("mfd_add_continuous_src", C.c_int,
     [_P, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, _IP]),
    ("mfd_add_source_points", C.c_int, [_P, C.c_int, C.c_int, C.c_size_t, C.POINTER(C.c_int64), _DP]),
    ("mfd_add_dft", C.c_int,
     [_P, C.c_int, _IP, _IP, C.POINTER(_DP), C.c_double, C.c_int, C.c_double, C.c_double, C.c_int,
      C.c_size_t, _DP, C.c_int, _IP]),
    ("mfd_step", C.c_int, [_P, C.c_int]),
    ("mfd_get_time", C.c_int, [_P, C.POINTER(C.c_int64), _DP]),
    ("mfd_get_field", C.c_int, [_P, C.c_int, _DP]),
    ("mfd_get_dft", C.c_int, [_P, C.c_int, _DP, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    ("mfd_flux", C.c_int, [_P, C.c_int, _IP, _IP, _DP]),
    ("mfd_design", C.c_int, [_P, C.c_int, _IP, _IP, _IP]),
    ("mfd_forward", C.c_int, [_P, C.c_int, C.c_int]),
    ("mfd_backward", C.c_int, [_P, C.c_int, _IP, C.POINTER(_DP), _DP]),
    ("mfd_add_material_grid", C.c_int, [_P, _DP, _DP, _IP, _DP, C.c_double, C.c_double, _DP, _DP, _IP]),
    ("mfd_material_grid_vjp", C.c_int, [_P, C.c_int, C.c_int, _IP, _IP, _IP, _DP, _DP]),
    ("mfd_set_bloch", C.c_int, [_P, C.POINTER(C.c_int), _DP]),
    ("mfd_get_field_im", C.c_int, [_P, C.c_int, _DP]),
    ("mfd_subpixel_rows", C.c_int, [C.c_int, C.c_int, C.c_int64, _DP, _DP, C.c_double, C.c_int, C.c_int,
                                    C.POINTER(mfd_object), C.c_double, _DP]),
    ("mfd_scale_dft", C.c_int, [_P, C.c_int, C.c_double, C.c_double]),
    ("mfd_set_dft", C.c_int, [_P, C.c_int, _DP]),
    ("mfd_src_current", C.c_int, [_P, C.c_int, C.c_double, _DP]),
    ("mfd_farfield", C.c_int, [_P, C.c_int, _IP, _IP, _DP, _DP, C.c_double, C.c_double, _IP, _IP, _DP, _DP,
                               C.c_int64, _DP, _DP]),
    ("mfd_green", C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                            C.c_int64, _DP, _DP, _DP]),
    ("mfd_flux_noalloc", C.c_int, [_P, _P, C.c_int64, C.c_int, _P, _P]),
    ("mfd_noalloc_last_error", C.c_char_p, []),
    ("mfd_kernel_launches", C.c_int64, [_P]),
    ("mfd_last_step_ms", C.c_double, [_P]),
]


# entry points that take device pointers; only the CUDA library exports them
DEVICE_ONLY = ("mfd_flux_noalloc", "mfd_noalloc_last_error")


class Engine:
    """One loaded library exporting the C ABI."""

    _cache = {}

    def __new__(cls, path=PRODUCT_LIB):
        path = os.path.abspath(path)
        if path in cls._cache:
            return cls._cache[path]
        if not os.path.exists(path):
            raise MeepError("native library %s is missing; run __graft_entry__.build()" % path)
        self = super().__new__(cls)
        self.path = path
        self.lib = C.CDLL(path, mode=C.RTLD_LOCAL)
        for name, res, args in SIGNATURES:
            if name in DEVICE_ONLY and not hasattr(self.lib, name):
                continue  # the CPU oracle library has no device-pointer entries
            fn = getattr(self.lib, name)
            fn.restype = res
            fn.argtypes = args
        cls._cache[path] = self
        return self

    def check(self, status):
        if status != 0:
            raise MeepError(self.lib.mfd_last_error().decode())

    def subpixel_rows(self, dim, cdir, lo, hi, objects, eps_default=1.0, tol=1e-4, maxeval=100000):
        """Averaged inverse-permittivity rows (mfd_subpixel_rows) of the pixels
        [lo[i], hi[i]] (arrays n x 3); objects: list of dicts with kind (0
        block, 1 sphere, 2 cylinder), center, size, radius, height, axis, eps."""
        lo = np.ascontiguousarray(lo, dtype=np.float64).reshape(-1, 3)
        hi = np.ascontiguousarray(hi, dtype=np.float64).reshape(-1, 3)
        objs = (mfd_object * max(1, len(objects)))()
        for q, o in enumerate(objects):
            objs[q].kind = int(o["kind"])
            objs[q].center[:] = list(o.get("center", (0, 0, 0)))
            objs[q].size[:] = list(o.get("size", (0, 0, 0)))
            objs[q].radius = float(o.get("radius", 0.0))
            objs[q].height = float(o.get("height", 0.0))
            objs[q].axis[:] = list(o.get("axis", (0, 0, 1)))
            objs[q].eps = float(o["eps"])
        rows = np.zeros((lo.shape[0], 3))
        self.check(self.lib.mfd_subpixel_rows(dim, cdir, lo.shape[0], _dptr(lo), _dptr(hi), tol, maxeval,
                                              len(objects), objs, eps_default, _dptr(rows)))
        return rows


    def green(self, dim, c0, freq, eps, mu, x, x0, f0=1.0 + 0.0j):
        """Homogeneous-medium Green's function (mfd_green) for the point pairs
        x[i], x0[i] (arrays n x 3) of a current f0 of component c0 (0..2 Ex..Ez,
        3..5 Hx..Hz): (n, 6) complex fields Ex, Ey, Ez, Hx, Hy, Hz."""
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        x0 = np.ascontiguousarray(x0, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((x.shape[0], 6, 2))
        self.check(self.lib.mfd_green(dim, c0, freq, eps, mu, complex(f0).real, complex(f0).imag, x.shape[0],
                                      _dptr(x), _dptr(x0), _dptr(out)))
        return out[..., 0] + 1j * out[..., 1]


def _dptr(a):
    return a.ctypes.data_as(_DP)


class Sim:
    """A simulation handle on one engine: dense numpy arrays in and out."""

    def __init__(self, engine, dim, n, io, a, courant=0.5, pml=None, precision=64, components=None):
        self.eng = engine
        g = mfd_grid()
        g.dim = dim
        for d in range(3):
            g.n[d] = int(n[d])
            g.io[d] = int(io[d])
        g.a = a
        g.courant = courant
        for (d, side), (thick, R, stretch) in (pml or {}).items():
            g.pml_thickness[d][side] = thick
            g.pml_R[d][side] = R
            g.pml_stretch[d][side] = stretch
        g.precision = precision
        mask = 0
        for c in components or []:
            mask |= 1 << c
        g.components = mask
        self.dim = dim
        self.ext = [int(n[d]) + 1 if self._present(d) else 1 for d in range(3)]
        self.ndense = int(np.prod(self.ext))
        h = _P()
        engine.check(engine.lib.mfd_create(C.byref(g), C.byref(h)))
        self.h = h

    def _present(self, d):
        return (self.dim == 1 and d == 2) or (self.dim == 2 and d < 2) or self.dim == 3

    def close(self):
        if self.h:
            self.eng.lib.mfd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _dense(self, arr):
        arr = np.ascontiguousarray(np.asarray(arr, dtype=np.float64).reshape(-1))
        if arr.size != self.ndense:
            raise MeepError("array has %d points, grid has %d" % (arr.size, self.ndense))
        return arr

    def set_chi1inv(self, c, d, arr):
        arr = self._dense(arr)
        self.eng.check(self.eng.lib.mfd_set_chi1inv(self.h, c, d, _dptr(arr)))

    def set_conductivity(self, c, arr):
        arr = self._dense(arr)
        self.eng.check(self.eng.lib.mfd_set_conductivity(self.h, c, _dptr(arr)))

    def add_lorentzian(self, omega0, gamma, drude, sigma):
        keep = [self._dense(s) if s is not None else None for s in sigma]
        ptrs = (_DP * 3)(*[_dptr(s) if s is not None else _DP() for s in keep])
        self.eng.check(self.eng.lib.mfd_add_lorentzian(self.h, E, omega0, gamma, int(drude), ptrs))

    def add_gaussian_src(self, freq, fwidth, integrated=True, s=5.0, window=None):
        i = C.c_int()
        if window is None:
            self.eng.check(self.eng.lib.mfd_add_gaussian_src(self.h, freq, fwidth, s, 0.0, 0, int(integrated),
                                                             C.byref(i)))
        else:
            self.eng.check(self.eng.lib.mfd_add_gaussian_src(self.h, freq, fwidth, window[0], window[1], 1,
                                                             int(integrated), C.byref(i)))
        return i.value

    def add_continuous_src(self, freq, width=0.0, start=0.0, end=1e300, slowness=3.0, integrated=True):
        i = C.c_int()
        f = complex(freq)
        self.eng.check(self.eng.lib.mfd_add_continuous_src(self.h, f.real, f.imag, width, start, end, slowness,
                                                           int(integrated), C.byref(i)))
        return i.value

    def add_source_points(self, c, src, idx, amp):
        idx = np.ascontiguousarray(np.asarray(idx, dtype=np.int64))
        amp = np.asarray(amp, dtype=np.complex128)
        ri = np.ascontiguousarray(np.stack([amp.real, amp.imag], axis=-1).reshape(-1))
        self.eng.check(self.eng.lib.mfd_add_source_points(self.h, c, src, idx.size,
                                                          idx.ctypes.data_as(C.POINTER(C.c_int64)), _dptr(ri)))

    def add_dft(self, c, lo, hi, weights, dV=1.0, include_weights=True, scale=1.0, centered=True,
                freqs=(0.1,), decimation=1):
        lo_a = (C.c_int * 3)(*lo)
        hi_a = (C.c_int * 3)(*hi)
        keep = [np.ascontiguousarray(np.asarray(w, dtype=np.float64)) if w is not None else None
                for w in weights]
        wp = (_DP * 3)(*[_dptr(w) if w is not None else _DP() for w in keep])
        fr = np.ascontiguousarray(np.asarray(freqs, dtype=np.float64))
        i = C.c_int()
        sc = complex(scale)
        self.eng.check(self.eng.lib.mfd_add_dft(self.h, c, lo_a, hi_a, wp, dV, int(include_weights), sc.real,
                                                sc.imag, int(centered), fr.size, _dptr(fr), decimation,
                                                C.byref(i)))
        return i.value

    def step(self, n=1):
        self.eng.check(self.eng.lib.mfd_step(self.h, int(n)))

    def time(self):
        t = C.c_int64()
        dt = C.c_double()
        self.eng.check(self.eng.lib.mfd_get_time(self.h, C.byref(t), C.byref(dt)))
        return t.value, dt.value

    def get_field(self, c):
        out = np.zeros(self.ndense)
        self.eng.check(self.eng.lib.mfd_get_field(self.h, c, _dptr(out)))
        return out.reshape(self.ext)

    def set_bloch(self, periodic, k):
        """Bloch-periodic boundaries: periodic[d] != 0 with wavevector k[d]
        (units of 2 pi / a); a nonzero k makes the fields complex."""
        per = (C.c_int * 3)(*[int(bool(x)) for x in periodic])
        kk = np.ascontiguousarray(np.asarray(k, dtype=np.float64))
        self.eng.check(self.eng.lib.mfd_set_bloch(self.h, per, _dptr(kk)))

    def get_field_im(self, c):
        out = np.zeros(self.ndense)
        self.eng.check(self.eng.lib.mfd_get_field_im(self.h, c, _dptr(out)))
        return out.reshape(self.ext)

    def get_dft(self, mid):
        npts = C.c_size_t()
        nf = C.c_size_t()
        self.eng.check(self.eng.lib.mfd_get_dft(self.h, mid, None, C.byref(npts), C.byref(nf)))
        out = np.zeros(2 * npts.value * nf.value)
        self.eng.check(self.eng.lib.mfd_get_dft(self.h, mid, _dptr(out), C.byref(npts), C.byref(nf)))
        return (out[0::2] + 1j * out[1::2]).reshape(npts.value, nf.value)

    def flux(self, idE, idH, nfreq):
        idE = (C.c_int * len(idE))(*idE)
        idH = (C.c_int * len(idH))(*idH)
        out = np.zeros(nfreq)
        self.eng.check(self.eng.lib.mfd_flux(self.h, len(idE), idE, idH, _dptr(out)))
        return out

    def scale_dft(self, mid, s):
        s = complex(s)
        self.eng.check(self.eng.lib.mfd_scale_dft(self.h, mid, s.real, s.imag))

    def farfield(self, sheets, x, eps=1.0, mu=1.0, periodic=None):
        """Near-to-far transform (mfd_farfield).  sheets: list of (monitor id,
        equivalent current component 0..5, is_half[3], rshift[3]); x: far points
        (n x 3); periodic: up to two (direction, images per side, phase per
        image, period).  Returns (n, nfreq, 6) complex Ex..Hz."""
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1, 3))
        ids = (C.c_int * len(sheets))(*[int(s[0]) for s in sheets])
        c0 = (C.c_int * len(sheets))(*[int(s[1]) for s in sheets])
        ish = np.ascontiguousarray([v for s in sheets for v in s[2]], dtype=np.float64)
        rsh = np.ascontiguousarray([v for s in sheets for v in s[3]], dtype=np.float64)
        per = list(periodic or []) + [(-1, 0, 0.0, 0.0)] * 2
        pd = (C.c_int * 2)(*[int(per[i][0]) for i in range(2)])
        pn = (C.c_int * 2)(*[int(per[i][1]) for i in range(2)])
        pk = np.ascontiguousarray([per[i][2] for i in range(2)], dtype=np.float64)
        pp = np.ascontiguousarray([per[i][3] for i in range(2)], dtype=np.float64)
        npts = C.c_size_t()
        nf = C.c_size_t()
        self.eng.check(self.eng.lib.mfd_get_dft(self.h, int(sheets[0][0]), None, C.byref(npts), C.byref(nf)))
        out = np.zeros((x.shape[0], nf.value, 6, 2))
        self.eng.check(self.eng.lib.mfd_farfield(self.h, len(sheets), ids, c0, _dptr(ish), _dptr(rsh), eps, mu, pd,
                                                 pn, _dptr(pk), _dptr(pp), x.shape[0], _dptr(x), _dptr(out)))
        return out[..., 0] + 1j * out[..., 1]

    def design(self, comps, lo, hi):
        """Declare the design: chi1inv of E components `comps` over the point
        box lo..hi (inclusive)."""
        self.design_comps = list(comps)
        self.design_lo, self.design_hi = tuple(int(x) for x in lo), tuple(int(x) for x in hi)
        self.design_shape = tuple(int(hi[d]) - int(lo[d]) + 1 for d in range(3))
        ca = (C.c_int * len(comps))(*comps)
        self.eng.check(self.eng.lib.mfd_design(self.h, len(comps), ca, (C.c_int * 3)(*lo), (C.c_int * 3)(*hi)))

    def add_material_grid(self, center, size, weights, eps1, eps2, beta=0.0, eta=0.5):
        """Material grid over the axis-aligned block (center, size): weights
        u of shape (n0, n1, n2) (fewer axes are padded with 1), projected with
        (beta, eta), eps = eps1 + p (eps2 - eps1) per direction (scalars or
        3-vectors).  Returns the grid's id."""
        u = np.asarray(weights, dtype=np.float64)
        u = u.reshape(u.shape + (1,) * (3 - u.ndim))
        n = (C.c_int * 3)(*u.shape)
        e1 = np.broadcast_to(np.asarray(eps1, dtype=np.float64), (3,)).copy()
        e2 = np.broadcast_to(np.asarray(eps2, dtype=np.float64), (3,)).copy()
        c = np.asarray(center, dtype=np.float64).reshape(3).copy()
        z = np.asarray(size, dtype=np.float64).reshape(3).copy()
        uu = np.ascontiguousarray(u.reshape(-1))
        i = C.c_int()
        self.eng.check(self.eng.lib.mfd_add_material_grid(self.h, _dptr(c), _dptr(z), n, _dptr(uu), float(beta),
                                                          float(eta), _dptr(e1), _dptr(e2), C.byref(i)))
        self.matgrid_shapes = getattr(self, "matgrid_shapes", {})
        self.matgrid_shapes[i.value] = u.shape
        return i.value

    def material_grid_vjp(self, grid, grad_chi1inv, comps=None, lo=None, hi=None):
        """dJ/du of a material grid from dJ/dchi1inv over a point box (by
        default the design's components and box: backward()'s output)."""
        comps = list(self.design_comps if comps is None else comps)
        lo = self.design_lo if lo is None else lo
        hi = self.design_hi if hi is None else hi
        g = np.ascontiguousarray(np.asarray(grad_chi1inv, dtype=np.float64).reshape(-1))
        shapes = getattr(self, "matgrid_shapes", {})
        if grid not in shapes:
            raise MeepError("meep: material grid id out of range")
        out = np.zeros(int(np.prod(shapes[grid])))
        self.eng.check(self.eng.lib.mfd_material_grid_vjp(self.h, int(grid), len(comps), (C.c_int * len(comps))(*comps),
                                                          (C.c_int * 3)(*lo), (C.c_int * 3)(*hi), _dptr(g),
                                                          _dptr(out)))
        return out.reshape(self.matgrid_shapes[grid])

    def forward(self, n, checkpoint_every=0):
        self.eng.check(self.eng.lib.mfd_forward(self.h, int(n), int(checkpoint_every)))

    def backward(self, dft_grads):
        """dft_grads: {monitor id: complex array [npts, nfreq] of dJ/dRe F +
        i dJ/dIm F}.  Returns dJ/dchi1inv, shape (ncomp, *design box)."""
        ids = list(dft_grads)
        keep = []
        for m in ids:
            g = np.asarray(dft_grads[m], dtype=np.complex128).reshape(-1)
            keep.append(np.ascontiguousarray(np.stack([g.real, g.imag], axis=-1).reshape(-1)))
        ida = (C.c_int * max(1, len(ids)))(*ids)
        gp = (_DP * max(1, len(ids)))(*[_dptr(k) for k in keep])
        out = np.zeros(len(self.design_comps) * int(np.prod(self.design_shape)))
        self.eng.check(self.eng.lib.mfd_backward(self.h, len(ids), ida, gp, _dptr(out)))
        return out.reshape((len(self.design_comps),) + self.design_shape)

    def launches(self):
        return self.eng.lib.mfd_kernel_launches(self.h)

    def last_step_ms(self):
        return self.eng.lib.mfd_last_step_ms(self.h)
