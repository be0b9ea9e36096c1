"""ctypes mirrors of the structs declared in include/alps_gb300.h.

Pure data definitions; loading the native library happens in
:mod:`alps_gb300._native`.
"""
import ctypes as C

MAX_FITS = 4

STATUS = {
    0: "ALPS_OK", 1: "ALPS_E_NAMELIST", 2: "ALPS_E_FIT_POINTS",
    3: "ALPS_E_SCAN_OPTION", 4: "ALPS_E_NSCAN", 5: "ALPS_E_SCAN_SAME_TYPE",
    6: "ALPS_E_SCAN_TYPE0", 7: "ALPS_E_FIT_FAILED", 8: "ALPS_E_SUBLUMINAL",
    9: "ALPS_E_ROOTS_DIVERGED", 10: "ALPS_E_POLY_KIND", 11: "ALPS_E_NPROC",
    20: "ALPS_E_INVALID", 21: "ALPS_E_CUDA", 22: "ALPS_E_OOM",
    23: "ALPS_E_TIMEOUT", 24: "ALPS_E_UNSUPPORTED", 25: "ALPS_E_GRID",
    26: "ALPS_E_SINGULAR", 27: "ALPS_E_IO", 28: "ALPS_E_NO_DEVICE",
}


class AlpsError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)} ({status})")


class alps_complex(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class alps_system(C.Structure):
    _fields_ = [
        ("nspec", C.c_int), ("nperp", C.c_int), ("npar", C.c_int),
        ("kperp", C.c_double), ("kpar", C.c_double), ("vA", C.c_double),
        ("Bessel_zero", C.c_double), ("kperp_norm", C.c_int),
        ("positions_principal", C.c_int), ("n_resonance_interval", C.c_int),
        ("Tlim", C.c_double), ("secant_method", C.c_int), ("numiter", C.c_int),
        ("D_threshold", C.c_double), ("D_prec", C.c_double),
        ("D_gap", C.c_double), ("D_tol", C.c_double),
        ("maxsteps_fit", C.c_int), ("lambda_initial_fit", C.c_double),
        ("lambdafac_fit", C.c_double), ("epsilon_fit", C.c_double),
        ("nproc", C.c_int), ("ngamma", C.c_int), ("npparbar", C.c_int),
    ]


class alps_species(C.Structure):
    _fields_ = [
        ("ns", C.c_double), ("qs", C.c_double), ("ms", C.c_double),
        ("ac_method", C.c_int), ("n_fits", C.c_int), ("relat", C.c_int),
        ("log_fit", C.c_int), ("use_bM", C.c_int),
        ("fit_type", C.c_int * MAX_FITS),
        ("fit_init", (C.c_double * 5) * MAX_FITS),
        ("perp_correction", C.c_double * MAX_FITS),
        ("poly_kind", C.c_int), ("poly_order", C.c_int),
        ("poly_log_max", C.c_double), ("bM_nmaxs", C.c_int),
        ("bM_Bessel_zeros", C.c_double), ("bM_betas", C.c_double),
        ("bM_alphas", C.c_double), ("bM_pdrifts", C.c_double),
    ]


class alps_map_params(C.Structure):
    _fields_ = [
        ("omi", C.c_double), ("omf", C.c_double), ("gami", C.c_double),
        ("gamf", C.c_double), ("nr", C.c_int), ("ni", C.c_int),
        ("loggridw", C.c_int), ("loggridg", C.c_int),
    ]


class alps_interp_params(C.Structure):
    _fields_ = [
        ("nperp", C.c_int), ("npar", C.c_int), ("smoothing", C.c_double),
        ("pperp_min", C.c_double), ("pperp_max", C.c_double),
        ("ppar_min", C.c_double), ("ppar_max", C.c_double),
        ("do_normalize", C.c_int), ("mult_f", C.c_double),
    ]


class alps_dist_params(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("ms", C.c_double), ("tau", C.c_double),
        ("alph", C.c_double), ("p_drift", C.c_double), ("kappa", C.c_double),
        ("beta", C.c_double), ("vA", C.c_double), ("maxP", C.c_double),
        ("autoscale", C.c_int), ("maxPperp", C.c_double),
        ("maxPpar", C.c_double), ("kappa1", C.c_double), ("species", C.c_int),
    ]


MAX_ROOTS = 100
MAX_SCANS = 8
MAX_INPUT_SPECIES = 8


class alps_scan_def(C.Structure):
    _fields_ = [
        ("type_s", C.c_int), ("swi", C.c_double), ("swf", C.c_double), ("log_scan", C.c_int),
        ("n_out", C.c_int), ("n_res", C.c_int), ("heating", C.c_int), ("eigen", C.c_int),
        ("diff", C.c_double), ("diff2", C.c_double),
    ]


class alps_input(C.Structure):
    _fields_ = [
        ("sys", alps_system), ("species", alps_species * MAX_INPUT_SPECIES),
        ("runname", C.c_char * 256), ("arrayName", C.c_char * 256),
        ("nroots", C.c_int), ("use_map", C.c_int), ("determine_minima", C.c_int),
        ("scan_option", C.c_int), ("n_scan", C.c_int), ("ngamma", C.c_int), ("npparbar", C.c_int),
        ("writeOut", C.c_int), ("guess", alps_complex * MAX_ROOTS), ("map", alps_map_params),
        ("scan", alps_scan_def * MAX_SCANS),
    ]


EIGEN_MAX_SPECIES = 8


class alps_eigen(C.Structure):
    _fields_ = [
        ("electric", alps_complex * 3), ("magnetic", alps_complex * 3),
        ("vmean", (alps_complex * 3) * EIGEN_MAX_SPECIES), ("ds", alps_complex * EIGEN_MAX_SPECIES),
        ("Ps", C.c_double * EIGEN_MAX_SPECIES), ("Ps_split", (C.c_double * 4) * EIGEN_MAX_SPECIES),
        ("ewave", C.c_double),
    ]


def eigen_columns(e, nspec):
    """Values of one output row after (kperp, kpar, Re om, Im om), in the
    order om_scan writes them (src/ALPS_fns.f90:2361-2381):
    eigen (ef, bf, Us(1:3,1:nspec), ds), heat (Ps, W_EM), heat_mech
    (Ps_split(1:4,1:nspec))."""
    def cx(z):
        return [z.re, z.im]
    eig = []
    for z in list(e.electric) + list(e.magnetic):
        eig += cx(z)
    for s in range(nspec):
        for j in range(3):
            eig += cx(e.vmean[s][j])
    for s in range(nspec):
        eig += cx(e.ds[s])
    heat = [e.Ps[s] for s in range(nspec)] + [e.ewave]
    mech = [e.Ps_split[s][q] for s in range(nspec) for q in range(4)]
    return eig, heat, mech


REQ_POLISH, REQ_MAP, REQ_SCAN = 0, 1, 2


class alps_request(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("ctx", C.c_void_p), ("n", C.c_int), ("om", C.POINTER(alps_complex)),
        ("iters", C.POINTER(C.c_int)), ("map", alps_map_params), ("map_cal", C.POINTER(alps_complex)),
        ("map_val", C.POINTER(C.c_double)), ("scan", alps_scan_def), ("scan_rows", C.POINTER(C.c_double)),
        ("status", C.c_int), ("latency_ms", C.c_double), ("rounds", C.c_int), ("om_rtol", C.c_double),
        ("converged", C.POINTER(C.c_int)),
    ]


class alps_server_profile(C.Structure):
    _fields_ = [
        ("rounds", C.c_int64), ("round_jobs", C.c_int64), ("group_batches", C.c_int64),
        ("scan_step_batches", C.c_int64), ("scan_steps", C.c_int64), ("round_gpu_ms", C.c_double),
        ("step_ms", C.c_double), ("loop_busy_ms", C.c_double), ("admit_ms", C.c_double),
        ("land_ms", C.c_double), ("groups_ms", C.c_double), ("round_launch_ms", C.c_double),
    ]


class alps_tune_result(C.Structure):
    _fields_ = [
        ("js", C.c_int), ("blocks_per_sm", C.c_int), ("warps_per_sm", C.c_int), ("tuned", C.c_int),
        ("candidates", C.c_int), ("ms_default", C.c_double), ("ms_best", C.c_double),
    ]


class alps_stats(C.Structure):
    _fields_ = [
        ("n_eval", C.c_int64), ("n_pole_terms", C.c_int64),
        ("n_resonant", C.c_int64), ("n_landau", C.c_int64),
        ("kernels_launched", C.c_int), ("graph_replays", C.c_int64), ("graph_captures", C.c_int64),
        ("tc_contractions", C.c_int), ("tc_fixed_entries", C.c_int64), ("tc_entries", C.c_int64),
        ("n_eval_total", C.c_int64), ("k_reused", C.c_int64),
    ]


def system_defaults(**kw):
    """&system defaults of the reference (src/ALPS_var.f90:83-314)."""
    s = alps_system()
    s.nspec = 1
    s.nperp = 0
    s.npar = 0
    s.kperp = 0.0
    s.kpar = 0.0
    s.vA = 0.0
    s.Bessel_zero = 1.0e-45
    s.kperp_norm = 1
    s.positions_principal = 5
    s.n_resonance_interval = 100
    s.Tlim = 0.01
    s.secant_method = 2
    s.numiter = 50
    s.D_threshold = 1.0e-5
    s.D_prec = 1.0e-5
    s.D_gap = 1.0e-5
    s.D_tol = 1.0e-7
    s.maxsteps_fit = 500
    s.lambda_initial_fit = 1.0
    s.lambdafac_fit = 10.0
    s.epsilon_fit = 1.0e-8
    s.nproc = 0
    s.ngamma = 100
    s.npparbar = 200
    for k, v in kw.items():
        if not hasattr(s, k):
            raise KeyError(k)
        setattr(s, k, v)
    return s


def species_defaults(**kw):
    """&spec_i defaults (src/ALPS_io.f90:302-345)."""
    sp = alps_species()
    sp.ns = 1.0
    sp.qs = 1.0
    sp.ms = 1.0
    sp.ac_method = 1
    sp.n_fits = 1
    sp.relat = 0
    sp.log_fit = 1
    sp.use_bM = 0
    sp.poly_kind = 0
    sp.poly_order = 0
    sp.poly_log_max = 0.0
    sp.bM_nmaxs = 500
    sp.bM_Bessel_zeros = 1.0e-50
    sp.bM_betas = 1.0
    sp.bM_alphas = 1.0
    sp.bM_pdrifts = 0.0
    fits = kw.pop("fits", None)
    for k, v in kw.items():
        if not hasattr(sp, k):
            raise KeyError(k)
        setattr(sp, k, v)
    if fits is not None:
        sp.n_fits = len(fits)
        for i, (ftype, init, pc) in enumerate(fits):
            sp.fit_type[i] = ftype
            for j in range(5):
                sp.fit_init[i][j] = init[j] if j < len(init) else 0.0
            sp.perp_correction[i] = pc
    return sp
