"""Python front end of the GB300 library, mirroring the reference's call
surface (src/ALPS_fns.f90): disp, secant / secant_osc / rtsec, refine_guess,
map_search, find_minima, om_scan.  Every evaluation goes through the native
library (alps_gb300/lib/libalps_gb300.so); nothing here computes det D.
"""
import ctypes as C
import math

import numpy as np

from . import _abi
from ._native import check, lib

alps_complex = _abi.alps_complex


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _cptr(a):
    return a.ctypes.data_as(C.POINTER(alps_complex))


def generate_f0(dist, nperp, npar):
    """f0 table of generate_distribution: (pperp, ppar, f0, ideal[6])."""
    n = (nperp + 1) * (npar + 1)
    pperp, ppar, f0, ideal = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(6)
    check(lib().alps_generate_f0(C.byref(dist), nperp, npar, _dptr(pperp), _dptr(ppar), _dptr(f0), _dptr(ideal)),
          "alps_generate_f0")
    return pperp, ppar, f0, ideal


def find_minima(val, nr, ni, numroots=100):
    """find_minima (src/ALPS_fns.f90:3860-3966); val[ir*ni+ii]; returns
    0-based (ir, ii) pairs in the reference's scan order."""
    val = np.ascontiguousarray(val, dtype=np.float64)
    iroots = (C.c_int * (2 * max(1, numroots)))()
    nf = C.c_int()
    check(lib().alps_find_minima(_dptr(val), nr, ni, numroots, iroots, C.byref(nf)), "alps_find_minima")
    return [(iroots[2 * k], iroots[2 * k + 1]) for k in range(nf.value)]


def read_input(path):
    """Parses an ALPS input file (init_param + scan_read) into alps_input."""
    inp = _abi.alps_input()
    check(lib().alps_read_input(path.encode(), C.byref(inp)), "alps_read_input")
    return inp


def read_f0(path, nperp, npar):
    """Reads an f0 table file (read_f0): (pperp, ppar, f0)."""
    n = (nperp + 1) * (npar + 1)
    a, b, c = np.zeros(n), np.zeros(n), np.zeros(n)
    check(lib().alps_read_f0(path.encode(), nperp, npar, _dptr(a), _dptr(b), _dptr(c)), "alps_read_f0")
    return a, b, c


def write_f0(path, pperp, ppar, f0):
    """Writes an f0 table in the list-directed layout generate_distribution
    produces (one "pperp ppar f0" line per node, 17 significant digits)."""
    with open(path, "w") as fh:
        for x, y, z in zip(pperp, ppar, f0):
            fh.write("%25.17E %25.17E %25.17E\n" % (x, y, z))


def run_input(input_path, workdir):
    """Runs an ALPS input file end to end (map or guesses, refine_guess,
    scans), writing the reference's output files under workdir/solution."""
    check(lib().alps_run_input(input_path.encode(), workdir.encode()), "alps_run_input")


class Plasma:
    """One plasma (an alps_ctx on the current CUDA device).

    species: list of (alps_species, pperp, ppar, f0), arrays of length
    (nperp+1)*(npar+1) in f0-file order.  prepare() runs derivative_f0 and
    the continuation fits on the device; set_k() runs determine_nmax, the
    Bessel table and the p_perp contraction.
    """

    def __init__(self, system, species, prepare=True, precision="fp64"):
        L = lib()
        self.sys = system
        self.nspec = system.nspec
        self._h = C.c_void_p()
        check(L.alps_create(C.byref(system), C.byref(self._h)), "alps_create")
        self.species = []
        for i, (sp, pperp, ppar, f0) in enumerate(species):
            if pperp is None:  # bi-Maxwellian / cold species (use_bM): no table
                ptrs = [None, None, None]
            else:
                a = [np.ascontiguousarray(x, dtype=np.float64) for x in (pperp, ppar, f0)]
                ptrs = [_dptr(x) for x in a]
            check(L.alps_set_species(self._h, i, C.byref(sp), *ptrs), "alps_set_species")
            self.species.append(sp)
        self.set_precision(precision)
        if prepare:
            self.prepare()
        self.kperp, self.kpar = system.kperp, system.kpar

    def close(self):
        if getattr(self, "_h", None):
            lib().alps_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_precision(self, precision):
        p = {"fp64": 0, "mixed": 1}[precision]
        check(lib().alps_set_precision(self._h, p), "alps_set_precision")
        self.precision = precision

    def prepare(self):
        check(lib().alps_prepare(self._h), "alps_prepare")

    def fit_size(self, i):
        sp = self.species[i]
        if sp.ac_method == 2 and not sp.use_bM:
            return (self.sys.nperp + 1) * (sp.poly_order + 1)
        nf = sp.n_fits if sp.ac_method == 1 else 1
        rows = max(self.sys.nperp, self.sys.ngamma) if sp.relat else self.sys.nperp
        return (rows + 1) * 5 * nf

    def get_fit(self, i):
        out = np.zeros(self.fit_size(i))
        check(lib().alps_get_fit(self._h, i, _dptr(out)), "alps_get_fit")
        return out

    def set_fit(self, i, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        check(lib().alps_set_fit(self._h, i, _dptr(arr)), "alps_set_fit")

    def get_f0_rel(self, i):
        """(gamma, pparbar, f0_rel, df/dGamma, df/dpparbar) of a relativistic
        species: the tables derivative_f0_rel writes."""
        ng, npb = self.sys.ngamma, self.sys.npparbar
        g, p = np.zeros(ng + 1), np.zeros(npb + 1)
        f, a, b = (np.zeros((ng + 1) * (npb + 1)) for _ in range(3))
        check(lib().alps_get_f0_rel(self._h, i, _dptr(g), _dptr(p), _dptr(f), _dptr(a), _dptr(b)),
              "alps_get_f0_rel")
        shape = (ng + 1, npb + 1)
        return g, p, f.reshape(shape), a.reshape(shape), b.reshape(shape)

    def set_k(self, kperp, kpar):
        check(lib().alps_set_k(self._h, float(kperp), float(kpar)), "alps_set_k")
        self.kperp, self.kpar = kperp, kpar

    def nmax(self):
        out = (C.c_int * self.nspec)()
        check(lib().alps_get_nmax(self._h, out), "alps_get_nmax")
        return list(out)

    def disp(self, om):
        """det D(om) with chi0 [s,i,j], chi0_low [s,n+1,i,j] (n = -1,0,1) and
        the wave tensor [i,j] (the side results of disp)."""
        D = alps_complex()
        chi0 = np.zeros(self.nspec * 9, dtype=np.complex128)
        chil = np.zeros(self.nspec * 27, dtype=np.complex128)
        wave = np.zeros(9, dtype=np.complex128)
        check(lib().alps_disp(self._h, alps_complex(om.real, om.imag), C.byref(D), _cptr(chi0), _cptr(chil),
                              _cptr(wave)), "alps_disp")
        return complex(D.re, D.im), chi0.reshape(self.nspec, 3, 3), chil.reshape(self.nspec, 3, 3, 3), \
            wave.reshape(3, 3)

    def disp_batch(self, oms):
        oms = np.ascontiguousarray(oms, dtype=np.complex128)
        out = np.zeros_like(oms)
        check(lib().alps_disp_batch(self._h, len(oms), _cptr(oms), _cptr(out)), "alps_disp_batch")
        return out

    def disp_batch_device(self, n, d_om_ptr, d_D_ptr, stream_ptr=None):
        check(lib().alps_disp_batch_device(self._h, n, C.c_void_p(d_om_ptr), C.c_void_p(d_D_ptr),
                                           C.c_void_p(stream_ptr or 0)), "alps_disp_batch_device")

    def batch_status(self, stream_ptr=None):
        """Status code of the last asynchronous batch (alps_batch_status):
        0, or the ALPS_E_* code of a device error; waits for the stream."""
        return lib().alps_batch_status(self._h, C.c_void_p(stream_ptr or 0))

    def secant(self, oms, method=None):
        """Polishes roots in place; returns (roots, iterations, det at root)."""
        if method is None:
            method = self.sys.secant_method
        oms = np.atleast_1d(np.ascontiguousarray(oms, dtype=np.complex128)).copy()
        it = (C.c_int * len(oms))()
        Df = np.zeros_like(oms)
        check(lib().alps_secant(self._h, method, len(oms), _cptr(oms), it, _cptr(Df)), "alps_secant")
        return oms, list(it), Df

    def polish(self, oms, om_rtol=1e-12, method=None):
        """Secant polish with the relative-step stop (alps_secant_ex):
        returns (roots, iterations, det at root, converged mask)."""
        if method is None:
            method = self.sys.secant_method
        oms = np.atleast_1d(np.ascontiguousarray(oms, dtype=np.complex128)).copy()
        it = (C.c_int * len(oms))()
        cv = (C.c_int * len(oms))()
        Df = np.zeros_like(oms)
        check(lib().alps_secant_ex(self._h, method, len(oms), _cptr(oms), float(om_rtol), it, _cptr(Df), cv),
              "alps_secant_ex")
        return oms, list(it), Df, np.array(list(cv), dtype=bool)

    def calc_eigen(self, oms, eigen=True, heat=True):
        """calc_eigen for each root in oms: a list of alps_eigen (fields
        relative to E_x, U_s, delta n_s, heating rates and their split)."""
        oms = np.atleast_1d(np.ascontiguousarray(oms, dtype=np.complex128))
        out = (_abi.alps_eigen * len(oms))()
        check(lib().alps_calc_eigen(self._h, len(oms), _cptr(oms), int(eigen), int(heat), out), "alps_calc_eigen")
        return list(out)

    def map_search(self, mp):
        """(om, cal, val) of map_search (src/ALPS_fns.f90:3595-3788)."""
        n = mp.nr * mp.ni
        om = np.zeros(n, dtype=np.complex128)
        cal = np.zeros(n, dtype=np.complex128)
        val = np.zeros(n)
        check(lib().alps_map(self._h, C.byref(mp), _cptr(om), _cptr(cal), _dptr(val)), "alps_map")
        return om, cal, val

    def set_profiling(self, on):
        check(lib().alps_set_profiling(self._h, int(bool(on))), "alps_set_profiling")

    def profile(self):
        """Summed device ms of (classify, pole sums, resonant, finalize) and
        the number of batches since profiling was switched on."""
        ms = np.zeros(4)
        nb = C.c_int64()
        check(lib().alps_get_profile(self._h, _dptr(ms), C.byref(nb)), "alps_get_profile")
        return ms, nb.value

    def autotune(self, n, om_device_ptr=None):
        """alps_autotune: times the launch shapes of a batch of n
        frequencies on this plasma and keeps the fastest for its bucket;
        returns {js, blocks_per_sm, warps_per_sm, tuned, candidates,
        ms_default, ms_best}."""
        r = _abi.alps_tune_result()
        check(lib().alps_autotune(self._h, int(n), C.c_void_p(om_device_ptr) if om_device_ptr else None,
                                  C.byref(r)), "alps_autotune")
        return {f: getattr(r, f) for f, _ in r._fields_}

    def stats(self):
        s = _abi.alps_stats()
        check(lib().alps_get_stats(self._h, C.byref(s)), "alps_get_stats")
        return s

    def om_scan(self, type_s, swi, swf, log_scan, n_out, n_res, wroots, eigen=False, heat=False, om_rtol=None):
        """k-scan with root following (om_scan, src/ALPS_fns.f90:2198-2600,
        step sizes of scan_read, src/ALPS_io.f90:426-552).  Returns
        rows[it, root, (kperp, kpar, Re, Im)] and the final roots; with eigen
        or heat also eig[it][root] (alps_eigen of calc_eigen at that row).
        om_rtol: None follows each root with the reference's secant rule;
        a number adds the relative-step stop of alps_secant_ex."""
        sy = self.sys
        wr = np.array(wroots, dtype=np.complex128)
        nroots = len(wr)
        kperp_last, kpar_last = self.kperp, self.kpar
        ns, nres = n_out, n_res
        theta_0 = math.atan(kperp_last / kpar_last)
        k_0 = math.sqrt(kperp_last ** 2 + kpar_last ** 2)
        d = 1.0 * ns * nres
        lg = math.log10
        diff = diff2 = 0.0
        if type_s == 0:
            diff = (lg(swi) - lg(kperp_last)) / d if log_scan else (swi - kperp_last) / d
            diff2 = (lg(swf) - lg(kpar_last)) / d if log_scan else (swf - kpar_last) / d
        elif type_s == 1:
            tf = swf * 4.0 * math.atan(1.0) / 180.0
            diff = (lg(tf) - lg(theta_0)) / d if log_scan else (tf - theta_0) / d
        elif type_s == 2:
            diff = (lg(swf) - lg(k_0)) / d if log_scan else (swf - k_0) / d
        elif type_s == 3:
            diff = (lg(swf) - lg(kperp_last)) / d if log_scan else (swf - kperp_last) / d
        elif type_s == 4:
            diff = (lg(swf) - lg(kpar_last)) / d if log_scan else (swf - kpar_last) / d
        else:
            raise ValueError("scan_type must be 0..4")
        rows = np.zeros((ns + 1, nroots, 4))
        rows[0, :, 0] = self.kperp
        rows[0, :, 1] = self.kpar
        rows[0, :, 2] = wr.real
        rows[0, :, 3] = wr.imag
        jump = np.ones(nroots, dtype=bool)
        want = eigen or heat
        eig = [[None] * nroots for _ in range(ns + 1)] if want else None
        if want:
            eig[0] = self.calc_eigen(wr, eigen, heat)
        out_row = 1
        for it in range(1, ns * nres + 1):
            kperp, kpar = self.kperp, self.kpar
            if type_s == 0:
                if log_scan:
                    kperp = 10.0 ** (lg(kperp_last) + diff * it)
                    kpar = 10.0 ** (lg(kpar_last) + diff2 * it)
                else:
                    kperp = kperp_last + diff * it
                    kpar = kpar_last + diff2 * it
            elif type_s == 1:
                th = 10.0 ** (lg(theta_0) + diff * it) if log_scan else theta_0 + diff * it
                kperp, kpar = k_0 * math.sin(th), k_0 * math.cos(th)
            elif type_s == 2:
                kt = 10.0 ** (lg(k_0) + diff * it) if log_scan else k_0 + diff * it
                kperp, kpar = kt * math.sin(theta_0), kt * math.cos(theta_0)
            elif type_s == 3:
                kperp = 10.0 ** (lg(kperp_last) + diff * it) if log_scan else kperp_last + diff * it
            else:
                kpar = 10.0 ** (lg(kpar_last) + diff * it) if log_scan else kpar_last + diff * it
            self.set_k(kperp, kpar)
            if not jump.any():
                raise _abi.AlpsError(9, "om_scan")
            idx = [i for i in range(nroots) if jump[i]]
            if om_rtol is None:
                new, _, _ = self.secant(wr[idx], sy.secant_method)
            else:
                new = self.polish(wr[idx], om_rtol, sy.secant_method)[0]
            ev = self.calc_eigen(new, eigen, heat) if (want and it % nres == 0) else None
            for q, i in enumerate(idx):
                wr[i] = new[q]
                if ev is not None:
                    eig[out_row][i] = ev[q]
                if not math.isfinite(wr[i].real):
                    jump[i] = False
                for imm in range(i):
                    if abs(wr[i] - wr[imm]) < sy.D_gap:
                        wr[i] = 0.0
                        jump[i] = False
                if it % nres == 0:
                    rows[out_row, i] = (kperp, kpar, wr[i].real, wr[i].imag)
            if it % nres == 0:
                out_row += 1
        if want:
            return rows, wr, eig
        return rows, wr


class Request:
    """A request submitted to a Server; its buffers live here until done."""

    def __init__(self, server, kind, plasma, **kw):
        self._server = server
        self.plasma = plasma
        self.kind = kind
        rq = _abi.alps_request()
        rq.kind = kind
        rq.ctx = plasma.handle.value if isinstance(plasma.handle, C.c_void_p) else plasma.handle
        rq.om_rtol = float(kw.get("om_rtol", 0.0))
        self._bufs = []
        if kind in (_abi.REQ_POLISH, _abi.REQ_SCAN):
            om = np.ascontiguousarray(np.atleast_1d(kw["guesses"]), dtype=np.complex128).copy()
            self.om = om
            rq.n = len(om)
            rq.om = _cptr(om)
            self.iters = (C.c_int * max(1, len(om)))()
            rq.iters = C.cast(self.iters, C.POINTER(C.c_int))
            self._conv = (C.c_int * max(1, len(om)))()
            rq.converged = C.cast(self._conv, C.POINTER(C.c_int))
        if kind == _abi.REQ_MAP:
            mp = kw["map"]
            rq.map = mp
            n = mp.nr * mp.ni
            self.cal = np.zeros(n, dtype=np.complex128)
            self.val = np.zeros(n)
            rq.map_cal = _cptr(self.cal)
            rq.map_val = _dptr(self.val)
        if kind == _abi.REQ_SCAN:
            sc = kw["scan"]
            rq.scan = sc
            self.rows = np.zeros((sc.n_out + 1) * len(self.om) * 4)
            rq.scan_rows = _dptr(self.rows)
        self._rq = rq
        self.id = C.c_int64()
        check(lib().alps_server_submit(server._h, C.byref(rq), C.byref(self.id)), "alps_server_submit")

    def done(self):
        d = C.c_int()
        check(lib().alps_server_poll(self._server._h, self.id, C.byref(d)), "alps_server_poll")
        return bool(d.value)

    def wait(self):
        """Blocks until done; returns the result (roots; (cal, val) of a map;
        the scan rows [it, root, (kperp, kpar, Re, Im)] and final roots)."""
        check(lib().alps_server_wait(self._server._h, self.id), "alps_server_wait")
        if self.kind == _abi.REQ_POLISH:
            return self.om.copy()
        if self.kind == _abi.REQ_MAP:
            return self.cal.copy(), self.val.copy()
        n = len(self.om)
        return self.rows.reshape(-1, n, 4).copy(), self.om.copy()

    @property
    def latency_ms(self):
        return self._rq.latency_ms

    @property
    def converged(self):
        """Polish: per root, whether it met a stopping rule before numiter."""
        return np.array(list(self._conv)[:len(self.om)], dtype=bool)

    @property
    def rounds(self):
        return self._rq.rounds


class Server:
    """Continuous batching of root polishes, k scans and maps over many
    plasmas (alps_server_*): requests run as they arrive, their batches
    overlap on the GPU, each result equals the request's result alone.
    A plasma serves one request at a time and must not be used elsewhere
    while it does."""

    def __init__(self, hbm_budget=0, max_active=0):
        self._h = C.c_void_p()
        check(lib().alps_server_create(int(hbm_budget), int(max_active), C.byref(self._h)), "alps_server_create")

    def polish(self, plasma, guesses, om_rtol=0.0):
        """om_rtol > 0 adds the relative-step stop of alps_secant_ex."""
        return Request(self, _abi.REQ_POLISH, plasma, guesses=guesses, om_rtol=om_rtol)

    def map(self, plasma, mp):
        return Request(self, _abi.REQ_MAP, plasma, map=mp)

    def scan(self, plasma, scan_def, roots, om_rtol=0.0):
        """scan_def: alps_scan_def with the step sizes of scan_read (diff,
        diff2), e.g. from scan_def(); roots: the refined roots at the
        plasma's current k."""
        return Request(self, _abi.REQ_SCAN, plasma, scan=scan_def, guesses=roots, om_rtol=om_rtol)

    def stats(self):
        r, a, b = C.c_int64(), C.c_int(), C.c_size_t()
        check(lib().alps_server_stats(self._h, C.byref(r), C.byref(a), C.byref(b)), "alps_server_stats")
        return {"batches": r.value, "peak_active": a.value, "peak_bytes": b.value}

    def profile(self):
        """alps_server_get_profile: rounds, jobs, device time of the rounds,
        scan k-step batches and host loop time since creation."""
        p = _abi.alps_server_profile()
        check(lib().alps_server_get_profile(self._h, C.byref(p)), "alps_server_get_profile")
        return {f: getattr(p, f) for f, _ in p._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().alps_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _handles(plasmas):
    return (C.c_void_p * len(plasmas))(*[p.handle.value if isinstance(p.handle, C.c_void_p) else p.handle
                                         for p in plasmas])


def make_many(systems_species, precision="fp64", ks=None):
    """Plasmas for many (system, species) pairs, prepared together
    (alps_prepare_many) and, with ks = [(kperp, kpar), ...], set to their k
    together (alps_set_k_many)."""
    plasmas = [Plasma(s, sp, prepare=False, precision=precision) for s, sp in systems_species]
    n = len(plasmas)
    st = (C.c_int * max(1, n))()
    check(lib().alps_prepare_many(_handles(plasmas), n, st), "alps_prepare_many")
    if ks is not None:
        set_k_many(plasmas, ks)
    return plasmas


def tune_clear():
    """alps_tune_clear: every bucket back to the default launch shapes."""
    check(lib().alps_tune_clear(), "alps_tune_clear")


def set_k_many(plasmas, ks):
    """alps_set_k_many: plasmas[i] to ks[i] = (kperp, kpar), all together;
    plasmas whose kperp stays keep their k tables."""
    n = len(plasmas)
    st = (C.c_int * max(1, n))()
    kp = np.ascontiguousarray([k[0] for k in ks], dtype=np.float64)
    kz = np.ascontiguousarray([k[1] for k in ks], dtype=np.float64)
    check(lib().alps_set_k_many(_handles(plasmas), n, _dptr(kp), _dptr(kz), st), "alps_set_k_many")
    for p, k in zip(plasmas, ks):
        p.kperp, p.kpar = k


def solve_many(plasmas, guesses, om_rtol=1e-12, method=2):
    """alps_solve_many: guesses[r] polished on plasmas[r] (each a Plasma at
    its own k), all on the device in one graph launch.  Returns (roots,
    iterations, det at root, converged mask)."""
    n = len(plasmas)
    oms = np.ascontiguousarray(np.asarray(guesses, dtype=np.complex128)).copy()
    handles = _handles(plasmas)
    it = (C.c_int * n)()
    cv = (C.c_int * n)()
    Df = np.zeros_like(oms)
    check(lib().alps_solve_many(handles, n, int(method), _cptr(oms), float(om_rtol), it, _cptr(Df), cv),
          "alps_solve_many")
    return oms, np.array(list(it)), Df, np.array(list(cv), dtype=bool)


def scan_def(type_s, swi, swf, log_scan, n_out, n_res, kperp, kpar):
    """alps_scan_def with scan_read's step sizes (src/ALPS_io.f90:426-552)
    for a scan starting at (kperp, kpar)."""
    lg = math.log10
    sc = _abi.alps_scan_def()
    sc.type_s, sc.swi, sc.swf, sc.log_scan, sc.n_out, sc.n_res = type_s, swi, swf, int(log_scan), n_out, n_res
    d = 1.0 * n_out * n_res
    theta_0 = math.atan(kperp / kpar)
    k_0 = math.sqrt(kperp ** 2 + kpar ** 2)
    if type_s == 0:
        sc.diff = (lg(swi) - lg(kperp)) / d if log_scan else (swi - kperp) / d
        sc.diff2 = (lg(swf) - lg(kpar)) / d if log_scan else (swf - kpar) / d
    elif type_s == 1:
        tf = swf * 4.0 * math.atan(1.0) / 180.0
        sc.diff = (lg(tf) - lg(theta_0)) / d if log_scan else (tf - theta_0) / d
    elif type_s == 2:
        sc.diff = (lg(swf) - lg(k_0)) / d if log_scan else (swf - k_0) / d
    elif type_s == 3:
        sc.diff = (lg(swf) - lg(kperp)) / d if log_scan else (swf - kperp) / d
    else:
        sc.diff = (lg(swf) - lg(kpar)) / d if log_scan else (swf - kpar) / d
    return sc
