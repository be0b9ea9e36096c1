"""ctypes front end of the CPU oracle (test infrastructure only).

Loads oracle/_build/liboracle.so, building it with oracle/Makefile when it is
missing.  Only the test suite, __graft_entry__.smoke() and bench.py's CPU
baseline use this module; the library itself never imports it.
"""
import ctypes as C
import os
import subprocess
import threading

import numpy as np

from alps_gb300 import _abi
from alps_gb300._abi import alps_complex, AlpsError

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_lib = None
_lock = threading.Lock()


def build(force=False):
    """Compiles the oracle with its Makefile (g++, no GPU needed)."""
    if force or not os.path.exists(LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _stale():
    src = [os.path.join(HERE, f) for f in ("alps_oracle.cpp", "alps_oracle.h")]
    src.append(os.path.join(HERE, "..", "include", "alps_gb300.h"))
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(s) > t for s in src)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB_PATH)
            P = C.POINTER
            dp = P(C.c_double)
            cp = P(alps_complex)
            L.oracle_create.argtypes = [P(_abi.alps_system), P(C.c_void_p)]
            L.oracle_destroy.argtypes = [C.c_void_p]
            L.oracle_destroy.restype = None
            L.oracle_set_species.argtypes = [C.c_void_p, C.c_int, P(_abi.alps_species), dp, dp, dp]
            L.oracle_prepare.argtypes = [C.c_void_p]
            L.oracle_get_fit.argtypes = [C.c_void_p, C.c_int, dp]
            L.oracle_set_fit.argtypes = [C.c_void_p, C.c_int, dp]
            L.oracle_get_df0.argtypes = [C.c_void_p, C.c_int, dp, dp]
            L.oracle_get_f0_rel.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp, dp]
            L.oracle_set_f0_rel.argtypes = [C.c_void_p, C.c_int, dp]
            L.oracle_set_k.argtypes = [C.c_void_p, C.c_double, C.c_double]
            L.oracle_get_nmax.argtypes = [C.c_void_p, P(C.c_int)]
            L.oracle_get_bessel.argtypes = [C.c_void_p, C.c_int, dp]
            L.oracle_disp.argtypes = [C.c_void_p, alps_complex, cp, cp, cp, cp]
            L.oracle_disp_mag.argtypes = [C.c_void_p, alps_complex, dp]
            L.oracle_disp_batch.argtypes = [C.c_void_p, C.c_int, cp, cp, C.c_int]
            L.oracle_full_integrate.argtypes = [C.c_void_p, C.c_int, alps_complex, C.c_int, C.c_int, cp, P(C.c_int)]
            L.oracle_int_ee.argtypes = [C.c_void_p, C.c_int, alps_complex, cp]
            L.oracle_secant.argtypes = [C.c_void_p, C.c_int, cp, P(C.c_int), cp]
            L.oracle_map.argtypes = [C.c_void_p, P(_abi.alps_map_params), cp, cp, dp, C.c_int]
            L.oracle_find_minima.argtypes = [dp, C.c_int, C.c_int, C.c_int, P(C.c_int), P(C.c_int)]
            L.oracle_scan.argtypes = [C.c_void_p, C.c_void_p, C.c_int, cp, dp, C.c_void_p]
            L.oracle_calc_eigen.argtypes = [C.c_void_p, alps_complex, C.c_int, C.c_int, P(_abi.alps_eigen)]
            L.oracle_set_threads.argtypes = [C.c_int]
            L.oracle_set_threads.restype = None
            L.oracle_bessj.argtypes = [C.c_int, C.c_double]
            L.oracle_bessj.restype = C.c_double
            L.oracle_bessi_scaled.argtypes = [C.c_int, C.c_double]
            L.oracle_bessi_scaled.restype = C.c_double
            L.oracle_wofz.argtypes = [C.c_double, C.c_double, P(C.c_double), P(C.c_double)]
            L.oracle_generate_f0.argtypes = [P(_abi.alps_dist_params), C.c_int, C.c_int, dp, dp, dp, dp]
            L.oracle_interpolate.argtypes = [dp, dp, dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                             C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, dp]
            _lib = L
    return _lib


class ScanDef(C.Structure):
    _fields_ = [("type_s", C.c_int), ("swi", C.c_double), ("swf", C.c_double),
                ("log_scan", C.c_int), ("n_out", C.c_int), ("n_res", C.c_int),
                ("eigen", C.c_int), ("heat", C.c_int)]


def _chk(st, where):
    if st != 0:
        raise AlpsError(st, where)


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _cptr(a):
    return a.ctypes.data_as(C.POINTER(alps_complex))


def bessi_scaled(n, x):
    """exp(-x) I_n(x) of the NHDS branch."""
    return lib().oracle_bessi_scaled(int(n), float(x))


def interpolate(pperp_c, ppar_c, f_c, nperp, npar, smoothing, pperp_range, ppar_range, normalize,
                mult_f=1.0):
    """interpolation/interpolation.f90: the spline of log f through the
    samples on the fine grid; returns f [(nperp+1), (npar+1)]."""
    pp = np.ascontiguousarray(pperp_c, dtype=np.float64)
    pl = np.ascontiguousarray(ppar_c, dtype=np.float64)
    ff = np.ascontiguousarray(f_c, dtype=np.float64)
    out = np.zeros((nperp + 1) * (npar + 1))
    _chk(lib().oracle_interpolate(_dptr(pp), _dptr(pl), _dptr(ff), len(ff), int(nperp), int(npar),
                                  float(smoothing), float(pperp_range[0]), float(pperp_range[1]),
                                  float(ppar_range[0]), float(ppar_range[1]), int(bool(normalize)),
                                  float(mult_f), _dptr(out)), "oracle_interpolate")
    return out.reshape(nperp + 1, npar + 1)


def wofz(z):
    """Faddeeva function w(z) of the NHDS branch (algorithm 680)."""
    u, v = C.c_double(), C.c_double()
    lib().oracle_wofz(z.real, z.imag, C.byref(u), C.byref(v))
    return complex(u.value, v.value)


def set_threads(n):
    lib().oracle_set_threads(int(n))


def bessj(n, x):
    return lib().oracle_bessj(int(n), float(x))


def generate_f0(dist, nperp, npar):
    """Restated generate_distribution: returns (pperp, ppar, f0, ideal)."""
    n = (nperp + 1) * (npar + 1)
    pperp = np.zeros(n)
    ppar = np.zeros(n)
    f0 = np.zeros(n)
    ideal = np.zeros(6)
    _chk(lib().oracle_generate_f0(C.byref(dist), nperp, npar, _dptr(pperp), _dptr(ppar), _dptr(f0), _dptr(ideal)),
         "oracle_generate_f0")
    return pperp, ppar, f0, ideal


class OraclePlasma:
    """One plasma (context) in the oracle.  species: list of (alps_species,
    pperp, ppar, f0) with arrays of length (nperp+1)*(npar+1)."""

    def __init__(self, system, species, prepare=True, fits=None, f0_rel=None):
        """f0_rel: optional {species index: f0_rel table [(ngamma+1),
        (npparbar+1)]} used in place of the oracle's own spline remap (for
        input grids whose dense spline system is beyond a CPU)."""
        L = lib()
        self.sys = system
        self.nspec = system.nspec
        self._h = C.c_void_p()
        _chk(L.oracle_create(C.byref(system), C.byref(self._h)), "oracle_create")
        self._keep = []
        for i, (sp, pperp, ppar, f0) in enumerate(species):
            if pperp is None:  # NHDS species: no table
                ptrs = [None, None, None]
            else:
                a = [np.ascontiguousarray(x, dtype=np.float64) for x in (pperp, ppar, f0)]
                self._keep.append(a)
                ptrs = [_dptr(x) for x in a]
            _chk(L.oracle_set_species(self._h, i, C.byref(sp), *ptrs), "oracle_set_species")
        self.species = [s[0] for s in species]
        for i, tab in (f0_rel or {}).items():
            tab = np.ascontiguousarray(tab, dtype=np.float64).ravel()
            self._keep.append(tab)
            _chk(L.oracle_set_f0_rel(self._h, i, _dptr(tab)), "oracle_set_f0_rel")
        if prepare:
            _chk(L.oracle_prepare(self._h), "oracle_prepare")
        if fits is not None:
            for i, f in enumerate(fits):
                self.set_fit(i, f)

    def __del__(self):
        try:
            if self._h:
                lib().oracle_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def fit_size(self, i):
        sp = self.species[i]
        if sp.ac_method == 2 and not sp.use_bM:
            return (self.sys.nperp + 1) * (sp.poly_order + 1)
        rows = max(self.sys.nperp, self.sys.ngamma) if sp.relat else self.sys.nperp
        return (rows + 1) * 5 * (max(1, sp.n_fits) if sp.ac_method == 1 else 1)

    def get_fit(self, i):
        out = np.zeros(self.fit_size(i))
        _chk(lib().oracle_get_fit(self._h, i, _dptr(out)), "oracle_get_fit")
        return out

    def set_fit(self, i, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        _chk(lib().oracle_set_fit(self._h, i, _dptr(arr)), "oracle_set_fit")

    def get_df0(self, i):
        n = (self.sys.nperp + 1) * (self.sys.npar + 1)
        a, b = np.zeros(n), np.zeros(n)
        _chk(lib().oracle_get_df0(self._h, i, _dptr(a), _dptr(b)), "oracle_get_df0")
        return a, b

    def get_f0_rel(self, i):
        """(gamma, pparbar, f0_rel, df/dGamma, df/dpparbar) of a relativistic species."""
        ng, npb = self.sys.ngamma, self.sys.npparbar
        g, p = np.zeros(ng + 1), np.zeros(npb + 1)
        f, a, b = (np.zeros((ng + 1) * (npb + 1)) for _ in range(3))
        _chk(lib().oracle_get_f0_rel(self._h, i, _dptr(g), _dptr(p), _dptr(f), _dptr(a), _dptr(b)),
             "oracle_get_f0_rel")
        shape = (ng + 1, npb + 1)
        return g, p, f.reshape(shape), a.reshape(shape), b.reshape(shape)

    def set_k(self, kperp, kpar):
        _chk(lib().oracle_set_k(self._h, kperp, kpar), "oracle_set_k")

    def nmax(self):
        out = (C.c_int * self.nspec)()
        _chk(lib().oracle_get_nmax(self._h, out), "oracle_get_nmax")
        return list(out)

    def bessel(self, i):
        nm = self.nmax()[i]
        out = np.zeros((nm + 3) * (self.sys.nperp + 1))
        _chk(lib().oracle_get_bessel(self._h, i, _dptr(out)), "oracle_get_bessel")
        return out.reshape(nm + 3, self.sys.nperp + 1)

    def disp(self, om):
        D = alps_complex()
        chi0 = np.zeros(self.nspec * 9, dtype=np.complex128)
        chil = np.zeros(self.nspec * 27, dtype=np.complex128)
        wave = np.zeros(9, dtype=np.complex128)
        _chk(lib().oracle_disp(self._h, alps_complex(om.real, om.imag), C.byref(D), _cptr(chi0), _cptr(chil),
                               _cptr(wave)), "oracle_disp")
        return complex(D.re, D.im), chi0.reshape(self.nspec, 3, 3), chil.reshape(self.nspec, 3, 3, 3), \
            wave.reshape(3, 3)

    def disp_mag(self, om):
        """Sum over orders of |chi_ij contributions| per species [s,i,j]."""
        out = np.zeros(self.nspec * 9)
        _chk(lib().oracle_disp_mag(self._h, alps_complex(om.real, om.imag), _dptr(out)), "oracle_disp_mag")
        return out.reshape(self.nspec, 3, 3)

    def disp_batch(self, oms, nthreads=1):
        oms = np.ascontiguousarray(oms, dtype=np.complex128)
        out = np.zeros_like(oms)
        _chk(lib().oracle_disp_batch(self._h, len(oms), _cptr(oms), _cptr(out), nthreads), "oracle_disp_batch")
        return out

    def full_integrate(self, is_, om, nn, mode):
        out = alps_complex()
        res = C.c_int()
        _chk(lib().oracle_full_integrate(self._h, is_, alps_complex(om.real, om.imag), nn, mode, C.byref(out),
                                         C.byref(res)), "oracle_full_integrate")
        return complex(out.re, out.im), bool(res.value)

    def int_ee(self, is_):
        out = alps_complex()
        _chk(lib().oracle_int_ee(self._h, is_, alps_complex(0, 0), C.byref(out)), "oracle_int_ee")
        return complex(out.re, out.im)

    def secant(self, om, method=None):
        if method is None:
            method = self.sys.secant_method
        o = alps_complex(om.real, om.imag)
        it = C.c_int()
        Df = alps_complex()
        _chk(lib().oracle_secant(self._h, method, C.byref(o), C.byref(it), C.byref(Df)), "oracle_secant")
        return complex(o.re, o.im), it.value, complex(Df.re, Df.im)

    def map(self, mp, nthreads=1):
        n = mp.nr * mp.ni
        om = np.zeros(n, dtype=np.complex128)
        cal = np.zeros(n, dtype=np.complex128)
        val = np.zeros(n)
        _chk(lib().oracle_map(self._h, C.byref(mp), _cptr(om), _cptr(cal), _dptr(val), nthreads), "oracle_map")
        return om, cal, val

    def scan(self, type_s, swi, swf, log_scan, n_out, n_res, wroots, eigen=False, heat=False):
        """om_scan: rows [it, root, (kperp, kpar, re, im)] and the updated
        roots; with eigen/heat also a list [it][root] of alps_eigen."""
        sd = ScanDef(type_s, swi, swf, int(log_scan), n_out, n_res, int(eigen), int(heat))
        wr = np.ascontiguousarray(wroots, dtype=np.complex128)
        rows = np.zeros((n_out + 1) * len(wr) * 4)
        eig = (_abi.alps_eigen * ((n_out + 1) * len(wr)))() if (eigen or heat) else None
        _chk(lib().oracle_scan(self._h, C.byref(sd), len(wr), _cptr(wr), _dptr(rows),
                               C.cast(eig, C.c_void_p) if eig is not None else None), "oracle_scan")
        rows = rows.reshape(n_out + 1, len(wr), 4)
        if eig is None:
            return rows, wr
        return rows, wr, [[eig[it * len(wr) + r] for r in range(len(wr))] for it in range(n_out + 1)]

    def calc_eigen(self, om, eigen=True, heat=True):
        out = _abi.alps_eigen()
        _chk(lib().oracle_calc_eigen(self._h, alps_complex(om.real, om.imag), int(eigen), int(heat), C.byref(out)),
             "oracle_calc_eigen")
        return out


def find_minima(val, nr, ni, numroots=100):
    val = np.ascontiguousarray(val, dtype=np.float64)
    iroots = (C.c_int * (2 * numroots))()
    nf = C.c_int()
    _chk(lib().oracle_find_minima(_dptr(val), nr, ni, numroots, iroots, C.byref(nf)), "oracle_find_minima")
    return [(iroots[2 * k], iroots[2 * k + 1]) for k in range(nf.value)]
