"""Synthetic plasmas used by the tests and the benchmark.

Every f0 table is produced by a restatement of the reference's
generate_distribution formulas (distribution/generate_distribution.f90:
176-300); no dataset is involved.  A workload is a dict with

  system   -- alps_system (the &system namelist)
  dists    -- list of alps_dist_params, one per species
  species  -- list of alps_species (the &spec_i / &ffit_i_j namelists)
  k        -- (kperp, kpar) of the first evaluation
  extra    -- scan / map / guess settings of the workload

``build(workload, generate)`` turns it into the (system, [(species, pperp,
ppar, f0)]) pair both the library and the oracle take; ``generate`` is a
generator with the signature of alps_generate_f0.
"""
from . import _abi

M_E_KPAR_FAST = 5.44662e-4   # m_e/m_p of the reference's quick test inputs


def _dist(kind=1, ms=1.0, tau=1.0, alph=1.0, p_drift=0.0, kappa=8.0, beta=1.0, vA=1e-4, maxP=6.0,
          autoscale=1, kappa1=8.0):
    d = _abi.alps_dist_params()
    d.kind = kind
    d.ms = ms
    d.tau = tau
    d.alph = alph
    d.p_drift = p_drift
    d.kappa = kappa
    d.beta = beta
    d.vA = vA
    d.maxP = maxP
    d.autoscale = autoscale
    d.maxPperp = 1.0
    d.maxPpar = 1.0
    d.kappa1 = kappa1
    return d


def kpar_fast(nproc=4):
    """The reference's CI input tests/test_kpar_fast.in with the f0 tables of
    distribution/test_kpar_fast_dist.in (2 species, 120x240, k_par scan)."""
    sysd = _abi.system_defaults(
        nspec=2, nperp=120, npar=240, kperp=1e-2, kpar=1e-2, vA=1e-4, Bessel_zero=1e-50,
        secant_method=2, numiter=50, kperp_norm=1, D_threshold=1e-15, D_prec=1e-5, D_gap=1e-5,
        D_tol=1e-7, positions_principal=3, n_resonance_interval=100, Tlim=0.01, maxsteps_fit=500,
        lambda_initial_fit=1.0, lambdafac_fit=10.0, epsilon_fit=1e-8, nproc=nproc)
    sp1 = _abi.species_defaults(ns=1.0, qs=1.0, ms=1.0, fits=[(1, [1.7959e-1, 1.0, 0, 0, 0], 1.0)])
    sp2 = _abi.species_defaults(ns=1.0, qs=-1.0, ms=M_E_KPAR_FAST,
                                fits=[(1, [1.4128e4, 1.836e3, 0, 0, 0], 1.836e3)])
    return dict(system=sysd, dists=[_dist(ms=1.0), _dist(ms=M_E_KPAR_FAST)], species=[sp1, sp2],
                k=(1e-2, 1e-2),
                extra=dict(guess=[9.9e-3 - 5.5e-6j],
                           scan=dict(type_s=4, swi=1e-3, swf=1e-1, log_scan=True, n_out=32, n_res=1)))


def proton_electron(nperp, npar, kperp, kpar, Bessel_zero, me=1.0 / 1836.0, nproc=0, ideal_fits=True,
                    gen=None):
    """Two bi-Maxwellian species, protons (m=1,q=1,n=1) and electrons
    (m=me,q=-1,n=1), beta_par=1, T_perp/T_par=1, no drift, maxP=6, vA/c=1e-4:
    the plasma of the benchmark configurations."""
    sysd = _abi.system_defaults(
        nspec=2, nperp=nperp, npar=npar, kperp=kperp, kpar=kpar, vA=1e-4, Bessel_zero=Bessel_zero,
        secant_method=2, numiter=50, kperp_norm=1, D_threshold=1e-15, D_prec=1e-5, D_gap=1e-5,
        D_tol=1e-7, positions_principal=3, n_resonance_interval=100, Tlim=0.01, nproc=nproc)
    dists = [_dist(ms=1.0), _dist(ms=me)]
    species = []
    for d, q in zip(dists, (1.0, -1.0)):
        # The ideal fit parameters of generate_distribution seed the LM fit.
        import math
        norm = math.pi ** -1.5 / ((d.ms * d.beta * d.tau) ** 1.5 * d.alph)
        species.append(_abi.species_defaults(
            ns=1.0, qs=q, ms=d.ms,
            fits=[(1, [norm, 1.0 / (d.beta * d.ms * d.tau), d.p_drift, 0, 0],
                   1.0 / (d.tau * d.beta * d.ms * d.alph))]))
    return dict(system=sysd, dists=dists, species=species, k=(kperp, kpar), extra={})


def config_kscan():
    """Plain-FP64 k-scan: 60x120 grid, k_perp d_p = 1, k_par d_p from 0.05 to
    1 (log, 32 steps), Bessel cutoff 1e-50, guess 0.05-0.01i."""
    w = proton_electron(60, 120, 1.0, 0.05, 1e-50)
    w["extra"] = dict(guess=[0.05 - 0.01j],
                      scan=dict(type_s=4, swi=0.05, swf=1.0, log_scan=True, n_out=32, n_res=1))
    return w


def config_map(nr=512, ni=512, Bessel_zero=1e-9):
    """Complex-frequency map: 128x256 grid, k_perp d_p = 2, k_par d_p = 0.3,
    det D on an nr x ni lattice Re(omega) in [0,3], Im(omega) in [-0.5,0.1];
    the Bessel cutoff 1e-9 gives the stated nmax ~30 for protons."""
    w = proton_electron(128, 256, 2.0, 0.3, Bessel_zero)
    mp = _abi.alps_map_params()
    mp.omi, mp.omf, mp.gami, mp.gamf = 0.0, 3.0, -0.5, 0.1
    mp.nr, mp.ni = nr, ni
    mp.loggridw = mp.loggridg = 0
    w["extra"] = dict(map=mp, n_polish=8)
    return w


M_E = 1.0 / 1836.0
VA_REL = 1e-2  # v_A/c of the relativistic configuration


def config_relativistic(theta_e, nperp=128, npar=256, ngamma=100, npparbar=200, kpar_de=0.1, vA=VA_REL,
                        Bessel_zero=1e-20):
    """Relativistic electrons: a Juettner f0 (generator kind 3) with
    Theta = kT_e/(m_e c^2) = theta_e on an nperp x npar (p_perp, p_par) grid,
    remapped to an ngamma x npparbar (Gamma, pparbar) grid (relat = T,
    fit type 4, the Gamma-only Juettner continuation with perp_correction
    1/Theta in Gamma), beside a bi-Maxwellian proton background (beta_p = 1)
    in the closed form (use_bM).  v_A/c = vA; the generator's exponent
    2 m_e/(v_A^2 beta tau_e) equals 1/Theta for tau_e = 2 m_e Theta/(v_A^2
    beta); the grid spans |p| <= m_e c sqrt((1 + 18 Theta)^2 - 1).  k at
    propagation angle 30 degrees with k_par d_e = kpar_de
    (d_e = d_p sqrt(m_e/m_p)), the whistler branch's start; guess from the
    cold whistler omega = Omega_e k^2 d_e^2 cos(theta)/(1 + k^2 d_e^2)."""
    import math
    beta = 1.0
    tau_e = 2.0 * M_E * theta_e / (vA * vA * beta)
    # the generator's autoscale is written for species of the reference
    # mass; the electron grid spans Gamma - 1 <= 18 Theta instead (f0 down to
    # e^-18, as maxP = 6 does for a Maxwellian), in units of m_p v_A
    pmax = (M_E / vA) * math.sqrt((1.0 + 18.0 * theta_e) ** 2 - 1.0)
    de = _dist(kind=3, ms=M_E, tau=tau_e, beta=beta, vA=vA, autoscale=0)
    de.maxPperp = de.maxPpar = pmax
    sysd = _abi.system_defaults(
        nspec=2, nperp=nperp, npar=npar, kperp=0.0, kpar=0.0, vA=vA, Bessel_zero=Bessel_zero,
        secant_method=2, numiter=50, kperp_norm=1, D_threshold=1e-30, D_prec=1e-5, D_gap=1e-5, D_tol=1e-7,
        positions_principal=5, n_resonance_interval=100, Tlim=0.01, ngamma=ngamma, npparbar=npparbar)
    spE = _abi.species_defaults(ns=1.0, qs=-1.0, ms=M_E, relat=1, fits=[(4, [1.0, 0, 0, 0, 0], 1.0 / theta_e)])
    spP = _abi.species_defaults(ns=1.0, qs=1.0, ms=1.0, use_bM=1, bM_nmaxs=500, bM_Bessel_zeros=1e-50,
                                bM_betas=beta, bM_alphas=1.0, bM_pdrifts=0.0)
    th = math.radians(30.0)
    sq = math.sqrt(1.0 / M_E)                    # d_p / d_e
    kpar = kpar_de * sq
    kperp = kpar * math.tan(th)
    kde = kpar_de / math.cos(th)
    guess = (1.0 / M_E) * kde * kde * math.cos(th) / (1.0 + kde * kde)
    return dict(system=sysd, dists=[de, None], species=[spE, spP], k=(kperp, kpar),
                extra=dict(theta_e=theta_e, tau_e=tau_e, guess=[guess - 1e-3j * guess],
                           scan=dict(type_s=2, swi=0.0, swf=2.0 * sq / math.cos(th), log_scan=True, n_out=64,
                                     n_res=1)))


def build_relativistic(w, generate):
    """(system, [(species, pperp, ppar, f0)]) of config_relativistic: the
    electron table from the generator, the closed-form protons without one."""
    s = w["system"]
    pperp, ppar, f0, _ = generate(w["dists"][0], s.nperp, s.npar)
    return s, [(w["species"][0], pperp, ppar, f0), (w["species"][1], None, None, None)]


def uneven_plasma(rng, grid=None, Bessel_zero=1e-20):
    """One solve of the uneven-batch draw: 1-3 species from {bi-Maxwellian
    with T_perp/T_par in U[0.3,3] and beta in logU[0.01,10]; a drifting proton
    beam with n_b/n_p in U[0.02,0.2] and drift in U[0,2] v_A; bi-kappa with
    kappa in U[3,10] (fit type 2)}, grid N_perp in {64,96,128,192,256} with
    N_par = 2 N_perp (or ``grid``), k_perp rho_p in logU[0.01,10] and a
    propagation angle in U[20,88] degrees.  ``rng`` is a numpy Generator."""
    import math
    nspec = int(rng.integers(1, 4))
    N = int(rng.choice([64, 96, 128, 192, 256])) if grid is None else grid[0]
    M = 2 * N if grid is None else grid[1]
    beta_p = 10.0 ** rng.uniform(-2.0, 1.0)
    dists, species = [], []
    kinds = ["bimax"] + [str(rng.choice(["bimax", "beam", "kappa"])) for _ in range(nspec - 1)]
    for k, kind in enumerate(kinds):
        electron = (k == 1 and kind == "bimax")
        ms, qs = (1.0 / 1836.0, -1.0) if electron else (1.0, 1.0)
        ns = 1.0
        # the generator's autoscale spans maxP sqrt(m tau alpha) whatever the
        # beta, so maxP = 6 sqrt(beta) keeps six thermal momenta on the grid
        if kind == "bimax":
            beta = beta_p if k == 0 else 10.0 ** rng.uniform(-2, 1)
            d = _dist(kind=1, ms=ms, alph=rng.uniform(0.3, 3.0), beta=beta, maxP=6.0 * math.sqrt(beta))
        elif kind == "beam":
            ns = rng.uniform(0.02, 0.2)
            d = _dist(kind=1, ms=1.0, beta=beta_p, p_drift=rng.uniform(0.0, 2.0), maxP=6.0 * math.sqrt(beta_p))
        else:
            kap = rng.uniform(3.0, 10.0)
            d = _dist(kind=2, ms=ms, beta=beta_p, kappa=kap, kappa1=kap, maxP=6.0 * math.sqrt(beta_p))
        dists.append(d)
        species.append((kind, ns, qs, ms))
    krho = 10.0 ** rng.uniform(-2.0, 1.0)
    kperp = krho / math.sqrt(beta_p)
    theta = math.radians(rng.uniform(20.0, 88.0))
    # keep the largest Bessel argument k_perp pperp_max/|q| <= 60 (nmax up
    # to ~80, the stated range): species with their own larger beta would
    # otherwise push it into the thousands
    zmax = max(kperp * d.maxP * math.sqrt(d.ms * d.tau * d.alph) / abs(q)
               for d, (_, _, q, _) in zip(dists, species))
    if zmax > 60.0:
        kperp *= 60.0 / zmax
    kpar = kperp / math.tan(theta)
    sysd = _abi.system_defaults(
        nspec=nspec, nperp=N, npar=M, kperp=kperp, kpar=kpar, vA=1e-4, Bessel_zero=Bessel_zero,
        secant_method=2, numiter=50, kperp_norm=1, D_threshold=1e-15, positions_principal=3,
        n_resonance_interval=100, Tlim=0.01)
    return dict(system=sysd, dists=dists, species_kinds=species, k=(kperp, kpar),
                extra=dict(theta_deg=math.degrees(theta), krho=krho, beta_p=beta_p))


def build_uneven(w, generate):
    """(system, [(species, pperp, ppar, f0)]) of an uneven_plasma draw, the
    continuation seeded with generate_distribution's ideal parameters (fit
    type 1 for the Maxwellians and the beam, type 2 for bi-kappa)."""
    s = w["system"]
    out = []
    for d, (kind, ns, qs, ms) in zip(w["dists"], w["species_kinds"]):
        pperp, ppar, f0, ideal = generate(d, s.nperp, s.npar)
        ftype = 2 if kind == "kappa" else 1
        sp = _abi.species_defaults(ns=ns, qs=qs, ms=ms, fits=[(ftype, list(ideal[:5]), ideal[5])])
        out.append((sp, pperp, ppar, f0))
    return s, out


def build(w, generate):
    """Returns (system, [(species, pperp, ppar, f0), ...])."""
    s = w["system"]
    out = []
    for d, sp in zip(w["dists"], w["species"]):
        pperp, ppar, f0, _ = generate(d, s.nperp, s.npar)
        out.append((sp, pperp, ppar, f0))
    return s, out
