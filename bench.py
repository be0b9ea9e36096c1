"""Benchmark of the det D(omega, k) hot path on one GB300 (or N replicas).

Workload (one "step"): the complex-frequency map of the two-species plasma
(protons + electrons, bi-Maxwellian, beta=1) on a 128x256 (p_perp, p_par)
grid at k_perp d_p = 2, k_par d_p = 0.3, det D on a 512 x 512 lattice of
omega in [0,3] x [-0.5,0.1] Omega_p; after the timed steps the 8 deepest map
minima are polished by the secant method (roots/s, latency).  Inputs are
synthetic (f0 tables from the restated generate_distribution formulas).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU oracle (the restatement of the Fortran
reference, which cannot be built on this image) on the host cores, on a
bounded sample of the same lattice.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from alps_gb300 import _abi, workloads  # noqa: E402
from alps_gb300.sharding import shard_range  # noqa: E402

METRIC = "D(omega,k) evals/s & roots/s at <=1e-8 rel vs FP64, vs plain GPU; p50/p99 latency"
UNIT = "evals/s"
POLISH_RTOL = 1e-12
KSCAN_RTOL = 1e-12  # the k-scan's stop on |delta omega| / |omega|
SERVED_RTOL = 1e-10  # the served stream's stop: two orders below its 1e-8 root tolerance  # the map configuration's polish tolerance on |delta omega| / |omega|


def lattice(mp):
    dr = (mp.omf - mp.omi) / (mp.nr - 1)
    di = (mp.gamf - mp.gami) / (mp.ni - 1)
    wr = mp.omi + dr * np.arange(mp.nr)
    wi = mp.gami + di * np.arange(mp.ni)
    return (wr[:, None] + 1j * wi[None, :]).ravel()


def config_dict(w, nr, ni, world):
    s = w["system"]
    return {"workload": "map%dx%d_grid%dx%d_kperp%g_kpar%g" % (nr, ni, s.nperp, s.npar, s.kperp, s.kpar),
            "species": 2, "nperp": s.nperp, "npar": s.npar, "kperp": s.kperp, "kpar": s.kpar,
            "Bessel_zero": s.Bessel_zero, "lattice": [nr, ni], "omega_re": [0.0, 3.0], "omega_im": [-0.5, 0.1],
            "l2": "inputs < L2; a 256 MiB buffer is written between timed steps",
            "parallelism": "replicas%d" % world}


class Clocks:
    """nvidia-smi sampling (200 ms) during the timed region."""

    def __init__(self, idx):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(idx), "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def fp64_peak_tflops(torch):
    """Measured FP64 throughput of a cuBLAS DGEMM on this GPU (burst)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2.0 * n ** 3 / best / 1e12


def fp32_peak_tflops(torch):
    """Measured FP32 (FFMA) throughput of a cuBLAS SGEMM with TF32 off (burst)."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, dtype=torch.float32, device="cuda")
        b = torch.randn(n, n, dtype=torch.float32, device="cuda")
        for _ in range(2):
            torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e9
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return 2.0 * n ** 3 / best / 1e12


def pole_sum_flops(nmax, npar):
    """Algorithmic FP64 flops of the non-resonant pole sums per evaluation:
    150 per (order n >= 0, p_par node) covering +n and -n (2 complex
    reciprocals, 3 numerators, 12 entry MACs; complex mul 6, add 2,
    reciprocal 8)."""
    return sum(150.0 * (n + 1) * (npar - 1) for n in nmax)


def pole_sum_flops_issued(nmax, npar):
    """FP64 flops the pole-sum kernel issues per evaluation (FMA = 2): per
    (signed order, p_par node) 1 add, 1 FMA for |D|^2, reciprocal = rcp seed +
    2 Newton steps (4 FMA), 2 multiplies and 24 FMA: 61 flops."""
    return sum(61.0 * (2 * n + 1) * (npar - 1) for n in nmax)


# FP32-pipe flops (FMA = 2) of the fast path's pole sums, counted from the
# kernel's code (device_math.cuh, disp_kernels.cu pole_fused).  One
# double-float node: the pole distance d = A - k_par p_j (19), |d|^2 + D^2
# (19), its reciprocal (rcp and three FMA / one multiply of its series
# correction, 8), the two weights (22) and 12 double-float
# multiply-accumulates of the 6 base vectors (three Bessel families against
# g1 and g2) against them (15 each: product with its error term, two-sum
# into the accumulator)
DF_NODE_FLOPS = 19 + 19 + 8 + 22 + 12 * 15
# one double-float Laurent term (k >= 2): 12 multiply-accumulates of the
# base moments against the complex power and the power update (4 products,
# 2 sums)
DF_TERM_FLOPS = 12 * 15 + 4 * 9 + 2 * 10
# one FP32 Laurent tail term: 12 FMA and the complex power update
FP32_TERM_FLOPS = 12 * 2 + 6
# per (omega, signed order), the combination of the base sums into the six
# entries (double-float: complex product 62, omega-combination 104, real
# factor and accumulation 18 per component): a node sum's zeta products and
# range sums (about 1000), a series' k = 0, 1 terms, the Laurent T and U
# parts and the d, p_cen products (about 2100)
DF_ORDER_NODE_FLOPS = 1000
DF_ORDER_SERIES_FLOPS = 2100


def pole_sum_work_fast(system, species, kpar, oms, nmax):
    """Work of the fast path's pole sums over a lattice, with the kernel's own
    decisions per (omega, signed order): a pole far from the grid (not
    resonant, rho = prad/|p_res - pcen| with rho^2 < 0.58) takes K Laurent
    terms, rho^K <= 2^-53 (1 - rho), of which those from K32 on
    (rho^K32 <= 2^-33 (1 - rho)) run in FP32 and the ones before in
    double-float; any other order sums its nodes (a resonant one outside the
    principal-value window) in double-float.  The series' k = 0, 1 terms
    are part of the order's combination.  Returns counts: nodes (signed
    order x node pairs summed), series terms in double-float and in FP32,
    orders summed over nodes and by series, and resonant items (omega,
    species, signed order)."""
    ns, npar, M_I = system.nspec, system.npar, system.positions_principal
    M = npar
    kfar = min(128, int(0.8 * (M - 1)))
    out = {"nodes": 0.0, "series_df": 0.0, "series_fp32": 0.0, "node_orders": 0.0, "series_orders": 0.0,
           "items": 0.0}
    for si in range(ns):
        spc, pl = species[si][0], np.asarray(species[si][2])
        ppar = pl.reshape(-1, M + 1)[0]
        pcen, prad = 0.5 * (ppar[1] + ppar[M - 1]), 0.5 * (ppar[M - 1] - ppar[1])
        dpp = ppar[2] - ppar[1]
        for nn in range(-nmax[si], nmax[si] + 1):
            x = (spc.ms * oms.real - nn * spc.qs) / kpar
            y = spc.ms * oms.imag / kpar
            res = ((ppar[1] <= x) & (x < ppar[M])) | ((x < ppar[1]) & (x >= ppar[1] - M_I * dpp)) | \
                  ((x >= ppar[M - 1]) & (x < ppar[M - 1] + M_I * dpp))
            dd = (x - pcen) ** 2 + y ** 2
            far = (~res) & (prad * prad < 0.58 * dd)
            rho = np.where(far, prad / np.sqrt(np.where(far, dd, 1.0)), 0.5)
            # the kernel adds one term to each count for the rounding of its FP32 logarithms
            K = np.where(far, np.ceil((36.7368005696771 - np.log1p(-rho)) / -np.log(rho)) + 1, kfar + 1)
            K32 = np.where(far, np.ceil((22.8738569584782 - np.log1p(-rho)) / -np.log(rho)) + 1, kfar + 1)
            lau = K <= kfar
            out["series_df"] += np.maximum(np.minimum(K32, K) - 2, 0)[lau].sum()
            out["series_fp32"] += np.maximum(K - np.maximum(K32, 2), 0)[lau].sum()
            out["series_orders"] += lau.sum()
            nodes = np.where(res, (M - 1) - (2 * M_I + 2), M - 1)
            out["nodes"] += nodes[~lau].sum()
            out["node_orders"] += (~lau).sum()
            out["items"] += res.sum()
    return {k: float(v) for k, v in out.items()}


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the
    machine type)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def cpu_sample(P, oms, budget_s, nthreads, values=False):
    """Times the oracle on a bounded sample of the lattice; returns evals/s
    (and, with values, the sample's indices and det D)."""
    t0 = time.perf_counter()
    P.disp_batch(oms[:1], nthreads=1)
    t1 = time.perf_counter() - t0
    m = int(max(nthreads, min(len(oms), budget_s * nthreads / max(t1, 1e-6))))
    m = min(m, 512)
    idx = np.linspace(0, len(oms) - 1, m).astype(int)
    t0 = time.perf_counter()
    D = P.disp_batch(oms[idx], nthreads=nthreads)
    dt = time.perf_counter() - t0
    if values:
        return m / dt, m, dt, idx, D
    return m / dt, m, dt


def chi_errors(P, G, oms):
    """Per-entry chi0 error of the library against the oracle at oms: the
    largest |chi_gpu - chi_oracle| / max(|chi_oracle|, 1e-3 mag) (mag = the
    sum over Bessel orders of |order contribution|, as in the parity tests),
    over species and the nine entries, and the cofactor-normalised det D
    error |dD| / sum_ij |cof_ij| max(|w_ij|, 1e-3 mag_ij)."""
    sy = P.sys
    chi_err, det_err = 0.0, 0.0
    for om in oms:
        Do, co, _, wo = P.disp(om)
        Dg, cg, _, _ = G.disp(om)
        mag = P.disp_mag(om)
        denom = abs(om * om) * sy.vA ** 2 * (1.0 if sy.kperp_norm else sy.kperp ** 2)
        scale = np.maximum(np.abs(co), 1e-3 * mag / denom)
        chi_err = max(chi_err, float((np.abs(cg - co) / np.maximum(scale, 1e-300)).max()))
        cof = np.array([[np.linalg.det(np.delete(np.delete(wo, i, 0), j, 1)) for j in range(3)] for i in range(3)])
        norm = np.sum(np.abs(cof) * np.maximum(np.abs(wo), 1e-3 * mag.sum(axis=0)))
        det_err = max(det_err, float(abs(Dg - Do) / norm))
    return chi_err, det_err


def root_errors(P, roots, nthreads):
    """Distance of each root from the oracle's root, relative to |omega|: the
    oracle's Newton step |D(w) / D'(w)| / |w| at the library's root, D' from
    a central difference over 1e-7 |w|."""
    roots = np.asarray(roots)
    h = 1e-7 * np.abs(roots)
    pts = np.concatenate([roots, roots + h, roots - h])
    D = P.disp_batch(pts, nthreads=nthreads)
    n = len(roots)
    Dp = (D[n:2 * n] - D[2 * n:]) / (2 * h)
    return [float(abs(D[k] / Dp[k]) / abs(roots[k])) for k in range(n)]


def run_reference(args, w, mp, rank, world):
    if rank != 0:
        return
    from oracle import pyoracle as po
    nthreads = os.cpu_count() or 1
    system, species = workloads.build(w, po.generate_f0)
    P = po.OraclePlasma(system, species)
    P.set_k(system.kperp, system.kpar)
    oms = lattice(mp)
    # each step a bounded sample: about 8 s, less when many steps are asked
    # for, so that the whole run stays near two minutes
    budget = min(float(os.environ.get("ALPS_REF_STEP_S", "8")), max(0.5, 120.0 / max(1, args.steps)))
    for _ in range(args.warmup):
        cpu_sample(P, oms, min(budget, 2.0), nthreads)
    rates, ms = [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r, m, dt = cpu_sample(P, oms, budget, nthreads)
        rates.append(r)
        ms.append(dt * 1e3)
    wall = time.perf_counter() - t0
    value = float(np.mean(rates))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(ms)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference", "config": config_dict(w, mp.nr, mp.ni, world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": "per step %d lattice points of the map, oracle threads over points" % m},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line))


def kscan_leg(api, args):
    """The plain k-scan configuration: 2 species on a 60x120 grid, Bessel
    cutoff 1e-50 (nmax 58/24), k_perp d_p = 1, k_par d_p 0.05 -> 1 in 32 log
    steps, the Alfven / ion-cyclotron root followed from 0.05 - 0.01i by
    secant_osc (om_scan) until the secant update is at most KSCAN_RTOL of
    |omega|, on both precision paths; the oracle runs the same scan with
    the reference's stopping rule (|D| below D_threshold) on the host
    cores.  The absolute |D| rule sits at the mixed path's det D rounding
    level on this plasma, where it would run secant steps to numiter."""
    import torch
    w = workloads.config_kscan()
    system, species = workloads.build(w, api.generate_f0)
    sc = w["extra"]["scan"]
    scan_args = (sc["type_s"], sc["swi"], sc["swf"], sc["log_scan"], sc["n_out"], sc["n_res"])
    out = {"workload": "kscan32_grid60x120_kperp1_kpar0.05to1", "steps": sc["n_out"]}
    rows_p = None
    for precision in ("fp64", "mixed"):
        G = api.Plasma(system, species, precision=precision)
        G.set_k(*w["k"])
        root = G.polish([w["extra"]["guess"][0]], om_rtol=KSCAN_RTOL)[0]
        G.om_scan(*scan_args, root, om_rtol=KSCAN_RTOL)  # warm-up (graphs, tables)
        G.set_k(*w["k"])
        torch.cuda.synchronize()
        e0 = G.stats().n_eval_total
        t0 = time.perf_counter()
        rows, _ = G.om_scan(*scan_args, root, om_rtol=KSCAN_RTOL)
        dt = time.perf_counter() - t0
        ev = G.stats().n_eval_total - e0
        out[precision] = {"wall_s": dt, "evals": int(ev), "evals_per_s": ev / dt, "roots_per_s": sc["n_out"] / dt,
                          "final_root": [rows[-1, 0, 2], rows[-1, 0, 3]], "stop_rule": "secant update <= %g |omega|" % KSCAN_RTOL}
        if precision == "fp64":
            rows_p = rows
        else:
            wp = rows_p[:, 0, 2] + 1j * rows_p[:, 0, 3]
            wm = rows[:, 0, 2] + 1j * rows[:, 0, 3]
            out["max_rel_diff_roots_mixed_vs_fp64"] = float(np.max(np.abs(wm - wp) / np.abs(wp)))
        G.close()
    if not args.no_cpu_baseline:
        from oracle import pyoracle as po
        po.set_threads(os.cpu_count() or 1)
        O = po.OraclePlasma(system, species)
        O.set_k(*w["k"])
        ro = O.secant(w["extra"]["guess"][0])[0]
        t0 = time.perf_counter()
        rows_o, _ = O.scan(*scan_args, np.array([ro]))
        dt = time.perf_counter() - t0
        wo = rows_o[:, 0, 2] + 1j * rows_o[:, 0, 3]
        wp = rows_p[:, 0, 2] + 1j * rows_p[:, 0, 3]
        out["oracle"] = {"wall_s": dt, "roots_per_s": sc["n_out"] / dt, "cores": os.cpu_count(),
                         "kind": "port", "threads": "over (species, order) work items of each det D"}
        out["err_vs_oracle_roots_fp64"] = float(np.max(np.abs(wp - wo) / np.abs(wo)))
    return out


def relativistic_leg(args):
    """The relativistic configuration at Theta = 0.3: Juettner electrons on a
    128x256 (p_perp, p_par) grid remapped to 100 x 400 (Gamma, pparbar),
    closed-form bi-Maxwellian protons, v_A/c = 0.01; the whistler branch
    followed over k_par d_e 0.1 -> 2 in 64 log steps at 30 degrees (scan type
    2), each root polished to a relative step of 1e-12.  Preparation (the
    33 156-unknown spline system on the device) is timed apart."""
    import torch
    from alps_gb300 import api
    theta = 0.3
    w = workloads.config_relativistic(theta, nperp=128, npar=256, ngamma=100, npparbar=400)
    system, species = workloads.build_relativistic(w, api.generate_f0)
    t0 = time.perf_counter()
    G = api.Plasma(system, species)
    torch.cuda.synchronize()
    t_prep = time.perf_counter() - t0
    G.set_k(*w["k"])
    root = G.polish([w["extra"]["guess"][0]], om_rtol=POLISH_RTOL)[0]
    sc = w["extra"]["scan"]
    e0 = G.stats().n_eval_total
    t0 = time.perf_counter()
    rows, _ = G.om_scan(sc["type_s"], sc["swi"], sc["swf"], sc["log_scan"], sc["n_out"], sc["n_res"], root,
                        om_rtol=POLISH_RTOL)
    dt = time.perf_counter() - t0
    ev = G.stats().n_eval_total - e0
    nm = G.nmax()
    out = {"workload": "juettner_theta0.3_grid128x256_gamma100x400_whistler64", "prepare_s": t_prep,
           "spline_unknowns": (system.nperp + 1) * (system.npar + 1) + 3, "scan_wall_s": dt, "evals": int(ev),
           "evals_per_s": ev / dt, "roots_per_s": sc["n_out"] / dt, "nmax_end": nm,
           "root_start": [rows[0, 0, 2], rows[0, 0, 3]], "root_end": [rows[-1, 0, 2], rows[-1, 0, 3]]}
    G.close()
    return out


def make_plasmas(api, draws, precision, chunk=1024):
    """Prepared contexts (f0 tables, fits, k tables) of uneven_plasma draws:
    the per-run and per-k setup of each chunk of contexts in batched launches
    (alps_prepare_many, alps_set_k_many)."""
    out = []
    for c0 in range(0, len(draws), chunk):
        part = draws[c0:c0 + chunk]
        built = [workloads.build_uneven(w, api.generate_f0) for w in part]
        out += api.make_many(built, precision=precision, ks=[w["k"] for w in part])
    return out


def uneven_batch(api, args):
    """The uneven-batch configuration: args.uneven_solves root solves, each
    on its own uneven_plasma draw (1-3 species; N_perp in {64, 96, 128, 192,
    256}, N_par = 2 N_perp; k_perp rho_p in logU[0.01, 10], so nmax 2-80),
    polished to a relative step of 1e-12 from a guess in [0.2, 1.5] -
    i[0, 0.1] Omega_p, all in one device-resident graph launch
    (alps_solve_many), on the mixed and the plain FP64 path.  Preparation
    (f0, fits, k tables) is timed apart: the state stays on the device."""
    import torch
    rng = np.random.default_rng(3)
    n = args.uneven_solves
    draws = [workloads.uneven_plasma(rng) for _ in range(n)]
    guesses = rng.uniform(0.2, 1.5, n) - 1j * rng.uniform(0.0, 0.1, n)
    out = {"solves": n, "grids": sorted({"%dx%d" % (w["system"].nperp, w["system"].npar) for w in draws}),
           "species": [int(np.sum([w["system"].nspec == k for w in draws])) for k in (1, 2, 3)]}
    res = {}
    for precision in ("mixed", "fp64"):
        t0 = time.perf_counter()
        plasmas = make_plasmas(api, draws, precision)
        torch.cuda.synchronize()
        t_setup = time.perf_counter() - t0
        nmax = [max(G.nmax()) for G in plasmas]
        api.solve_many(plasmas[:8], guesses[:8])  # first graph build of the process
        t0 = time.perf_counter()
        roots, iters, _, conv = api.solve_many(plasmas, guesses)
        t_batch = time.perf_counter() - t0
        # lone solves of a sample: the latency of one solve on an idle GPU
        lat = []
        for k in range(0, n, max(1, n // 64)):
            t1 = time.perf_counter()
            api.solve_many([plasmas[k]], [guesses[k]])
            lat.append((time.perf_counter() - t1) * 1e3)
        evals = int(np.sum(2 + iters))  # the evaluations the root machines used (two initial, one per iteration)
        res[precision] = {"batch_s": t_batch, "converged": int(conv.sum()), "roots_per_s": int(conv.sum()) / t_batch,
                          "iterations": {"p50": float(np.percentile(iters, 50)), "max": int(iters.max())},
                          "root_evals_per_s": evals / t_batch,
                          "latency_ms_in_batch": t_batch * 1e3,
                          "latency_ms_alone": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                                               "samples": len(lat)},
                          "setup_s": t_setup, "nmax": {"min": int(min(nmax)), "max": int(max(nmax))}}
        res[precision]["_roots"] = roots
        res[precision]["_conv"] = conv
        if precision == "fp64":
            # the FP64 path's Newton step |D/D'| / |omega| at the roots of both
            # paths that ended on the same root but differ by more than 1e-8:
            # how far each is from the FP64 root, and whether the FP64 det D
            # itself fixes that root to 1e-8 (a near-double root does not)
            rm, cm = res["mixed"]["_roots"], res["mixed"]["_conv"]
            relm = np.abs(rm - roots) / np.abs(roots)
            far = np.nonzero(cm & conv & (relm > 1e-8) & (relm <= 1e-6))[0]

            def newton(G, w):
                h = 1e-7 * abs(w)
                D0, D1 = G.disp_batch(np.array([w, w + h]))
                return abs(D0 * h / (D1 - D0)) / abs(w) if D1 != D0 else float("inf")

            sm = np.array([newton(plasmas[i], rm[i]) for i in far[:64]])
            sf = np.array([newton(plasmas[i], roots[i]) for i in far[:64]])
            # a well-defined FP64 root: the FP64 Newton step there is below
            # 1e-10 of |omega| (a simple root of a smooth det D)
            wd = sf <= 1e-10
            res["_far"] = {"count": int(len(far)), "checked": int(len(sm)),
                           "fp64_root_well_defined": int(wd.sum()),
                           "fp64_newton_at_mixed_root_max_well_defined": float(sm[wd].max()) if wd.any() else None,
                           "max_rel_diff_well_defined": float(relm[far[:64]][wd].max()) if wd.any() else None,
                           "fp64_newton_at_fp64_root_min_other": float(sf[~wd].min()) if (~wd).any() else None}
        del plasmas
    both = res["mixed"]["_conv"] & res["fp64"]["_conv"]
    rel = np.abs(res["mixed"]["_roots"] - res["fp64"]["_roots"]) / np.abs(res["fp64"]["_roots"])
    far = res.pop("_far")
    for p in res.values():
        p.pop("_roots")
        p.pop("_conv")
    out.update(res)
    # random guesses: a root finder that wanders can settle on another root
    # on the other path; the agreement is stated over the solves that end
    # on the same root
    same = both & (rel <= 1e-6)
    out["mixed_vs_fp64"] = {"both_converged": int(both.sum()), "same_root": int(same.sum()),
                            "within_1e-8": int(np.sum(same & (rel <= 1e-8))),
                            "max_rel_diff_same_root": float(rel[same].max()) if same.any() else None,
                            "above_1e-8": far,
                            "note": ("roots of both paths within 1e-6 of each other count as the same root; for "
                                     "those apart by more than 1e-8 the FP64 path's Newton step at its own root "
                                     "says whether the FP64 det D has a simple root there (step below 1e-10 of "
                                     "|omega|), and at the mixed root how far that one is from it; a secant stop "
                                     "where the FP64 Newton step is large is not a simple root of a smooth det D "
                                     "(a jump of the piecewise integration or a near-double root)")}
    out["speedup_mixed_vs_fp64"] = res["fp64"]["batch_s"] / res["mixed"]["batch_s"]
    out["note"] = ("one graph launch per batch: fused det D of every root's two pending frequencies, then a device "
                   "step of every root machine, repeated by a conditional WHILE node; roots/s counts converged roots")
    return out


def seed_roots(api, plasmas, rng, tries=3):
    """One root per plasma where a batched solve from a few random guesses
    in [0.1, 1.5] - i[0, 0.1] finds one (alps_solve_many, polished to a
    relative step of 1e-12); None where none converged."""
    n = len(plasmas)
    rep = [G for G in plasmas for _ in range(tries)]
    g = rng.uniform(0.1, 1.5, n * tries) - 1j * rng.uniform(0.0, 0.1, n * tries)
    roots, _, _, conv = api.solve_many(rep, g)
    out = []
    for i in range(n):
        ok = [roots[i * tries + t] for t in range(tries) if conv[i * tries + t]]
        out.append(ok[0] if ok else None)
    return out


def served_stream(api, args, precision):
    """The served-stream configuration: Poisson arrivals at args.served_rate
    per second for args.served_seconds, 70 % single-k root polishes, 25 %
    32-step k scans with root following, 5 % 256 x 256 omega maps
    (args.served_mix), on plasmas drawn like the uneven batch (1-3 species,
    64x128 .. 256x512 grids), through one alps_server.

    The plasmas are device-resident pools, prepared before the stream and
    timed apart (setup_s): f0 tables, fits, Bessel tables and contractions.
    Polishes pick a random plasma of a pool of 512, scans one of 1024 (a
    scan owns its plasma while it moves k), maps one of 16; the server
    admits up to 1024 requests at once.  Each polish and scan
    plasma carries a root found at setup (seed_s); a polish starts from that
    root moved by up to 1 % in each of Re and Im, as refine_guess hands
    roots to the secant, and a scan starts from the root at the plasma's k,
    as om_scan does.  A scan is the k-scan of the plain k-scan
    configuration: k_par scanned in 32 log steps at fixed k_perp (scan type
    4: the k tables stay); a fraction args.served_kscans of them are |k|
    scans at fixed angle instead (type 2: nmax, Bessel tables and
    contractions rebuilt at each step).  A plasma's scans go up by 1.3 and
    back down in turn, each from the root its last scan ended on.  Latency
    runs from
    submission to result, with the requests overlapping on the GPU."""
    import torch
    rng = np.random.default_rng(5)
    rate, T = args.served_rate, args.served_seconds
    mix = np.asarray([float(x) for x in args.served_mix.split(",")])
    mix = mix / mix.sum()
    nreq = int(rate * T)
    kinds = rng.choice(3, nreq, p=mix)
    # a scan owns its plasma for its 32 steps: at 500 scans/s and a few
    # hundred ms per scan, a few hundred scan plasmas are busy at once
    n_pol, n_scan, n_map = 512, 1024, 16
    draws = [workloads.uneven_plasma(rng) for _ in range(n_pol + n_scan + n_map)]
    t0 = time.perf_counter()
    plasmas = make_plasmas(api, draws, precision)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    pol, scn, mpp = plasmas[:n_pol], plasmas[n_pol:n_pol + n_scan], plasmas[n_pol + n_scan:]
    t0 = time.perf_counter()
    roots = seed_roots(api, pol + scn, rng)
    t_seed = time.perf_counter() - t0
    pol_ok = [i for i in range(n_pol) if roots[i] is not None]
    scn_ok = [i for i in range(n_scan) if roots[n_pol + i] is not None]
    big = {i for i in pol_ok if draws[i]["system"].nperp == 256}
    mp = _abi.alps_map_params()
    mp.omi, mp.omf, mp.gami, mp.gamf, mp.nr, mp.ni = 0.05, 2.0, -0.3, 0.05, 256, 256
    srv = api.Server(max_active=1024)
    t_arr = np.cumsum(rng.exponential(1.0 / rate, nreq))
    # every request's random numbers are drawn here, apart from the
    # stream's timing, so both precision paths serve the same polishes
    u_pick, u_kind = rng.uniform(size=nreq), rng.uniform(size=nreq)
    u_d = rng.uniform(-0.01, 0.01, (nreq, 2))
    reqs = []
    # a scan owns its plasma until it is done and leaves it at its last k
    # with the root there: the next scan on that plasma starts from both,
    # and scans up (x1.3) and back down in turn
    scan_state = {i: (scn[i].kperp, scn[i].kpar, roots[n_pol + i], 1.3) for i in scn_ok}
    busy = {}
    n_scan_req = 0

    def release(i):
        r = busy.pop(i)
        rows, fin = r.wait()
        f = scan_state[i][3]
        if r._rq.status == 0 and np.isfinite(fin[0]) and fin[0] != 0:
            scan_state[i] = (float(rows[-1, 0, 0]), float(rows[-1, 0, 1]), complex(fin[0]), 1.0 / f)
        else:  # the scan lost its root: the plasma leaves the pool
            scan_state.pop(i)

    t0 = time.perf_counter()
    for k in range(nreq):
        wait = t_arr[k] - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        if kinds[k] == 1:
            for i in [i for i, r in busy.items() if r.done()]:
                release(i)
            free = [i for i in scan_state if i not in busy]
            if not free and busy:
                release(next(iter(busy)))
                free = [i for i in scan_state if i not in busy]
            if not free:
                kinds[k] = 0
        if kinds[k] == 0:
            i = pol_ok[min(int(u_pick[k] * len(pol_ok)), len(pol_ok) - 1)]
            g = complex(roots[i].real * (1 + u_d[k, 0]), roots[i].imag + u_d[k, 1] * abs(roots[i]))
            reqs.append(("polish", i in big, srv.polish(pol[i], [g], om_rtol=SERVED_RTOL), k))
        elif kinds[k] == 1:
            i = free[min(int(u_pick[k] * len(free)), len(free) - 1)]
            kp, kz, w0, f = scan_state[i]
            scn[i].kperp, scn[i].kpar = kp, kz
            n_scan_req += 1
            if u_kind[k] >= args.served_kscans:  # k_par scan: k_perp and the k tables stay
                sc = api.scan_def(4, 0.0, kz * f, True, 32, 1, kp, kz)
            else:  # |k| at fixed angle: nmax, Bessel tables and contractions each step
                sc = api.scan_def(2, 0.0, float(np.hypot(kp, kz)) * f, True, 32, 1, kp, kz)
            r = srv.scan(scn[i], sc, [w0], om_rtol=SERVED_RTOL)
            busy[i] = r
            reqs.append(("scan", False, r, k))
        else:
            reqs.append(("map", False, srv.map(mpp[min(int(u_pick[k] * n_map), n_map - 1)], mp), k))
    t_submit = time.perf_counter() - t0
    for _, _, r, _ in reqs:
        r.wait()
    wall = time.perf_counter() - t0
    st = srv.stats()
    prof = srv.profile()
    srv.close()
    out = {"precision": precision, "requests": nreq, "mix": [float(x) for x in mix], "arrival_rate_per_s": rate,
           "k_scan_fraction": args.served_kscans,
           "submit_s": t_submit, "wall_s": wall, "completed_per_s": nreq / wall, "setup_s": t_setup,
           "seed_s": t_seed, "pool": [n_pol, n_scan, n_map], "pool_with_root": [len(pol_ok), len(scn_ok)],
           "batches": st["batches"], "peak_in_flight": st["peak_active"],
           "peak_footprint_bytes": st["peak_bytes"], "latency_ms": {},
           # where the time goes (alps_server_get_profile)
           "breakdown": {"rounds": prof["rounds"], "jobs_per_round": prof["round_jobs"] / max(1, prof["rounds"]),
                         "round_device_ms_avg": prof["round_gpu_ms"] / max(1, prof["rounds"]),
                         "own_stream_batches": prof["group_batches"], "scan_steps": prof["scan_steps"],
                         "scan_step_batches": prof["scan_step_batches"],
                         "scan_step_batch_ms_avg": prof["step_ms"] / max(1, prof["scan_step_batches"]),
                         "server_loop_busy_s": prof["loop_busy_ms"] / 1e3, "admission_s": prof["admit_ms"] / 1e3,
                         "landing_rounds_s": prof["land_ms"] / 1e3, "group_pass_s": prof["groups_ms"] / 1e3,
                         "launching_rounds_s": prof["round_launch_ms"] / 1e3}}
    for kind in ("polish", "scan", "map"):
        lat = [r.latency_ms for kk, _, r, _ in reqs if kk == kind]
        if lat:
            out["latency_ms"][kind] = {"count": len(lat), "p50": float(np.percentile(lat, 50)),
                                       "p99": float(np.percentile(lat, 99))}
    lat = [r.latency_ms for kk, b, r, _ in reqs if kk == "polish" and b]
    if lat:
        out["latency_ms"]["polish_256x512"] = {"count": len(lat), "p50": float(np.percentile(lat, 50)),
                                               "p99": float(np.percentile(lat, 99)), "target_p99": 20.0}
    pol_conv = [bool(r.converged[0]) for kk, _, r, _ in reqs if kk == "polish"]
    out["polish_converged"] = int(np.sum(pol_conv))
    out["_polish_roots"] = {k: complex(r.om[0]) for kk, _, r, k in reqs if kk == "polish" and r.converged[0]}
    scan_ok = [r for kk, _, r, _ in reqs if kk == "scan" and r._rq.status == 0]
    out["scans_completed"] = len(scan_ok)
    nroots = int(np.sum(pol_conv)) + 33 * len(scan_ok)
    out["roots_per_s"] = nroots / wall
    out["note"] = ("latency from submission to result; polishes and scans start at roots found at setup (a polish "
                   "from the root moved by up to 1 %), polished until the secant update is at most 1e-10 |omega| "
                   "(or numiter = 50), two orders below the configuration's 1e-8 root tolerance; roots/s counts "
                   "converged polishes and scan rows; the k steps of the scans ready at one time go to the device "
                   "together; the stream is sustained when completed_per_s matches the arrival rate and wall_s "
                   "stays near the stream's duration")
    del plasmas, pol, scn, mpp
    return out


def served_both(api, args):
    """The served stream on the mixed and the plain FP64 path, with the
    relative difference of the polished roots that converged on both (the
    same requests on both paths)."""
    out = {p: served_stream(api, args, p) for p in ("mixed", "fp64")}
    # the same stream at a rate the server sustains: latency without queueing
    if args.served_light_rate > 0:
        light = argparse.Namespace(**vars(args))
        light.served_rate = args.served_light_rate
        out["mixed_light_load"] = served_stream(api, light, "mixed")
        out["mixed_light_load"].pop("_polish_roots", None)
    a, b = out["mixed"].pop("_polish_roots"), out["fp64"].pop("_polish_roots")
    both = sorted(set(a) & set(b))
    rel = np.array([abs(a[k] - b[k]) / abs(b[k]) for k in both]) if both else np.zeros(0)
    same = rel <= 1e-6  # both paths ended on the same root
    out["mixed_vs_fp64_polish"] = {"both_converged": len(both), "same_root": int(same.sum()),
                                   "max_rel_diff_same_root": float(rel[same].max()) if same.any() else None,
                                   "tolerance": 1e-8}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nr", type=int, default=512)
    ap.add_argument("--no-served", action="store_true", help="skip the served-stream measurement")
    ap.add_argument("--served-only", action="store_true",
                    help="run only the served stream and print its JSON object (for profiling the server)")
    ap.add_argument("--served-seconds", type=float, default=3.0, help="duration of the served stream's arrivals")
    ap.add_argument("--served-rate", type=float, default=2000.0, help="Poisson arrival rate of the served stream")
    ap.add_argument("--served-mix", default="0.70,0.25,0.05", help="polish, scan, map fractions of the served stream")
    ap.add_argument("--served-light-rate", type=float, default=100.0,
                    help="arrival rate of a second, lightly loaded served stream on the mixed path (0: none)")
    ap.add_argument("--served-kscans", type=float, default=0.0,
                    help="fraction of the served scans that scan |k| at fixed angle instead of k_par")
    ap.add_argument("--ni", type=int, default=512)
    ap.add_argument("--uneven-solves", type=int, default=4096, help="solves of the uneven-batch measurement")
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven-batch measurement")
    ap.add_argument("--no-kscan", action="store_true", help="skip the plain k-scan measurement")
    ap.add_argument("--no-relativistic", action="store_true", help="skip the relativistic k-scan measurement")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="time the default launch shapes")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.gpus else 1)))
    if "RANK" not in os.environ:
        world = 1
    w = workloads.config_map(args.nr, args.ni)
    mp = w["extra"]["map"]
    if args.impl == "reference":
        run_reference(args, w, mp, rank, world)
        return

    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from alps_gb300 import api
    if args.served_only:
        if rank == 0:
            print(json.dumps({"served": served_both(api, args)}))
        return
    # weak scaling: every replica evaluates a full lattice at its own k_par
    s = w["system"]
    kpar = s.kpar * (1.0 + 0.01 * rank)
    system, species = workloads.build(w, api.generate_f0)
    G = api.Plasma(system, species)
    G.set_k(s.kperp, kpar)
    nmax = G.nmax()
    oms = lattice(mp)
    n = len(oms)
    om_dev = torch.from_numpy(np.stack([oms.real, oms.imag], 1).copy()).cuda()
    D_dev = torch.empty_like(om_dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    # a dedicated stream: the library launches on exactly this stream, so the
    # CUDA events below bracket its kernels
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    assert sp != 0

    def step():
        G.disp_batch_device(n, om_dev.data_ptr(), D_dev.data_ptr(), sp)

    peak64 = peak32 = None

    def timed(precision):
        """warmup + K timed steps of one evaluation mode, then K more with
        CUDA events around each kernel for the kernel split; returns
        seconds, the split and the D values"""
        G.set_precision(precision)
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
            flush.fill_(1.0)
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t = e0.elapsed_time(e1) / 1e3
        if dist:
            tt = torch.tensor([t], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            t = float(tt.item())
        launches = G.stats().kernels_launched
        Dv = D_dev[:, 0].cpu().numpy() + 1j * D_dev[:, 1].cpu().numpy()
        G.set_profiling(True)
        for _ in range(args.steps):
            step()
            flush.fill_(1.0)
        torch.cuda.synchronize()
        prof = G.profile()
        G.set_profiling(False)
        timed.launches = launches
        return t, prof, Dv

    # the autotuner picks each path's launch shape for this batch on the
    # lattice itself, before any timing (alps_autotune)
    tune = {}
    if not args.no_autotune:
        for precision in ("fp64", "mixed"):
            G.set_precision(precision)
            t0 = time.perf_counter()
            tune[precision] = G.autotune(n, om_dev.data_ptr())
            tune[precision]["tuning_s"] = time.perf_counter() - t0
    # plain FP64 path (node sums everywhere): the baseline of the fast path
    t_plain, prof_plain, D_plain = timed("fp64")
    peak64 = fp64_peak_tflops(torch)
    peak32 = fp32_peak_tflops(torch)
    clocks = Clocks(local)
    t, (prof_ms, nb), D_fast = timed("mixed")
    clk = clocks.stop()
    value = world * n * args.steps / t
    value_plain = world * n * args.steps / t_plain
    ms_step = t / args.steps * 1e3
    st = G.stats()
    rel = np.abs(D_fast - D_plain) / np.maximum(np.abs(D_plain), 1e-300)

    # roofline of the dominant kernel of the timed (fast) path, from the live
    # CUDA-event split, with both main kernels' figures beside it
    names = ["classify", "pole_sums", "resonant", "finalize"]
    pm_plain, nb_plain = prof_plain
    per_fast = [x / max(nb, 1) for x in prof_ms]
    fast_pole_ms, res_ms = per_fast[1], per_fast[2]
    work = pole_sum_work_fast(system, species, kpar, oms, nmax)
    # pole sums: double-float node sums and series terms, FP32 series tails
    # and the per-order combinations, all on the FP32 pipes
    f32 = (work["nodes"] * DF_NODE_FLOPS + work["series_df"] * DF_TERM_FLOPS + work["series_fp32"] * FP32_TERM_FLOPS +
           work["node_orders"] * DF_ORDER_NODE_FLOPS + work["series_orders"] * DF_ORDER_SERIES_FLOPS)
    pole = {"kernel": "k_pole_sums_multi<false> (fast path)", "bound": "fp32", "kernel_ms": fast_pole_ms,
            "achieved": f32 / (fast_pole_ms / 1e3) / 1e12, "peak": peak32, "unit": "TFLOP/s",
            "frac": f32 / (fast_pole_ms / 1e3) / 1e12 / peak32, "fp32_flop_per_step": f32,
            "double_float_nodes_per_step": work["nodes"], "df_node_flops": DF_NODE_FLOPS,
            "series_terms_df": work["series_df"], "df_term_flops": DF_TERM_FLOPS,
            "series_terms_fp32": work["series_fp32"], "node_orders": work["node_orders"],
            "series_orders": work["series_orders"], "order_flops": [DF_ORDER_NODE_FLOPS, DF_ORDER_SERIES_FLOPS]}
    # resonant items: the algorithmic count per item, 24 M_P flops of
    # principal-value sums and 60 (N_perp + 1) of Landau rows, FP64
    f_res = work["items"] * (24.0 * system.n_resonance_interval + 60.0 * (system.nperp + 1))
    res = {"kernel": "k_resonant_multi (fast path)", "bound": "fp64-equivalent", "kernel_ms": res_ms,
           "achieved": f_res / (res_ms / 1e3) / 1e12, "peak": peak64, "unit": "TFLOP/s",
           "frac": f_res / (res_ms / 1e3) / 1e12 / peak64, "items_per_step": work["items"],
           "fp64_flop_per_step": f_res,
           "note": ("the reference algorithm's FP64 count per item over the DGEMM rate; the kernel runs the "
                    "principal-value sums in double-float on the FP32 pipes and factorises the Landau rows, "
                    "so the figure can read above 1")}
    dom = pole if fast_pole_ms >= res_ms else res
    # the plain path's pole sums: every order sums its nodes in FP64
    pole_ms = pm_plain[1] / max(nb_plain, 1)
    plain_achieved = pole_sum_flops(nmax, s.npar) * n / (pole_ms / 1e3) / 1e12
    plain_issued = pole_sum_flops_issued(nmax, s.npar) * n / (pole_ms / 1e3) / 1e12
    roofline = {"bound": dom["bound"], "achieved": dom["achieved"], "peak": dom["peak"], "unit": "TFLOP/s",
                "frac": dom["frac"], "traffic": None,
                "peak_source": ("cuBLAS DGEMM 4096^3 (fp64) and SGEMM 8192^3 with TF32 off (fp32), measured in "
                                "this run (burst); MEASURED_PEAKS.json has neither figure"),
                "kernel": dom["kernel"], "kernel_ms": dom["kernel_ms"],
                "kernel_share": dom["kernel_ms"] / max(sum(per_fast), 1e-30),
                "fp64_peak": peak64, "fp32_peak": peak32,
                "kernels": {"pole_sums": pole, "resonant": res},
                "plain_path": {"kernel": "k_pole_sums_multi<false> (plain FP64 path)", "kernel_ms": pole_ms,
                               "achieved": plain_achieved, "frac": plain_achieved / peak64,
                               "achieved_issued": plain_issued, "frac_issued": plain_issued / peak64},
                "per_kernel_ms_plain": dict(zip(names, [x / max(nb_plain, 1) for x in pm_plain])),
                "per_kernel_ms_fast": dict(zip(names, per_fast)),
                "kernel_split_note": ("kernel times from K further steps of the same lattice with CUDA events "
                                      "around each kernel on the launching stream, after the K timed steps")}

    # end to end through the C-ABI with host buffers (copies included)
    Dh = G.disp_batch(oms)
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps)):
        Dh = G.disp_batch(oms)
    e2e_t = (time.perf_counter() - t0) / max(1, args.steps)
    e2e = {"value": n / e2e_t, "unit": UNIT, "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": 16 * n}

    # polish the 8 deepest minima until the secant update is at most 1e-12
    # of |omega| (roots/s counts converged roots only; latency per solve)
    val = np.log10(np.abs(Dh))
    mins = api.find_minima(val, mp.nr, mp.ni, numroots=100)
    mins = sorted(mins, key=lambda ij: val[ij[0] * mp.ni + ij[1]])[:w["extra"]["n_polish"]]
    guesses = np.array([oms[i * mp.ni + j] for i, j in mins])
    lat = []
    for g in guesses:
        t0 = time.perf_counter()
        G.polish([g], om_rtol=POLISH_RTOL)
        lat.append((time.perf_counter() - t0) * 1e3)
    t0 = time.perf_counter()
    roots, iters, _, conv = G.polish(guesses, om_rtol=POLISH_RTOL)
    t_roots = time.perf_counter() - t0
    # the reference's own stopping rule (|D| < D_threshold, absolute) from the
    # same guesses: the parity mode, reported for its iteration counts
    _, iters_ref, _, conv_ref = G.polish(guesses, om_rtol=0.0)
    # the same solves on the plain FP64 path: root agreement of the fast path
    G.set_precision("fp64")
    roots_plain, _, _, conv_plain = G.polish(guesses, om_rtol=POLISH_RTOL)
    G.set_precision("mixed")
    both = conv & conv_plain
    root_rel = float(np.max(np.abs(roots[both] - roots_plain[both]) / np.abs(roots_plain[both]))) if both.any() \
        else None

    served = None if (args.no_served or rank != 0) else served_both(api, args)
    uneven = None if (args.no_uneven or rank != 0) else uneven_batch(api, args)
    kscan = None if (args.no_kscan or rank != 0) else kscan_leg(api, args)
    relat = None if (args.no_relativistic or rank != 0) else relativistic_leg(args)

    cpu = None
    err_vs_oracle = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        G_chk = api.Plasma(system, species)  # single-frequency checks with the side results
        G_chk.set_k(s.kperp, kpar)
        from oracle import pyoracle as po
        nthreads = os.cpu_count() or 1
        P = po.OraclePlasma(system, species)
        P.set_k(s.kperp, kpar)
        r, m, dt, idx, D_or = cpu_sample(P, oms, float(os.environ.get("ALPS_CPU_BASELINE_S", "10")), nthreads,
                                         values=True)
        # the same restatement on one core, a smaller sample
        r1, m1, dt1 = cpu_sample(P, oms, 3.0, 1)
        # error of both GPU paths against the FP64 oracle: det D on the timed
        # sample, chi entries and cofactor-normalised det D at 8 of its
        # points, and the polished roots
        rel_f = np.abs(D_fast[idx] - D_or) / np.abs(D_or)
        rel_p = np.abs(D_plain[idx] - D_or) / np.abs(D_or)
        pts = oms[idx[np.linspace(0, len(idx) - 1, 8).astype(int)]]
        chi_p, detn_p = chi_errors(P, G_chk, pts)
        G_chk.set_precision("mixed")
        chi_f, detn_f = chi_errors(P, G_chk, pts)
        G_chk.set_precision("fp64")
        err_vs_oracle = {
            "det_D_rel": {"mixed": float(rel_f.max()), "fp64": float(rel_p.max()), "points": int(m),
                          "note": "max |D - D_oracle| / |D_oracle| over the sample; det D of a 3x3 tensor with "
                                  "cancelling entries, see det_D_cofactor"},
            "det_D_cofactor": {"mixed": detn_f, "fp64": detn_p, "points": len(pts),
                               "note": "|dD| / sum_ij |cof_ij| max(|w_ij|, 1e-3 mag_ij): the bound the parity "
                                       "tests gate at 1e-10"},
            "chi_entry": {"mixed": chi_f, "fp64": chi_p, "points": len(pts),
                          "note": "max over species and entries of |dchi| / max(|chi|, 1e-3 mag)"},
            "roots": {"mixed": root_errors(P, roots[conv], nthreads),
                      "fp64": root_errors(P, roots_plain[conv_plain], nthreads),
                      "note": "oracle Newton step |D/D'| / |omega| at each converged root"},
            "fit": "each side's own Levenberg-Marquardt continuation fit"}
        cpu = {"value": r, "unit": UNIT, "cores": nthreads, "kind": "port", "cpu_model": cpu_model(),
               "sample": "%d lattice points of the same map (every %d-th), oracle threads over points, %.1f s"
                         % (m, max(1, n // m), dt),
               "single_core": {"value": r1, "unit": UNIT, "cores": 1,
                               "sample": "%d lattice points, %.1f s" % (m1, dt1)}}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "mixed: fp32 double-float + fp64", "data": "synthetic",
                "precision_path": G.precision, "err_vs_oracle": err_vs_oracle,
                "config": config_dict(w, mp.nr, mp.ni, world), "nmax": nmax, "autotune": tune or None,
                "plain_fp64": {"value": value_plain, "unit": UNIT, "dtype": "f64",
                               "ms_per_step": t_plain / args.steps * 1e3,
                               "speedup_of_fast_path": value / value_plain,
                               "max_rel_diff_det_D_fast_vs_plain": float(rel.max()),
                               "max_rel_diff_roots_fast_vs_plain": root_rel},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
                "gpu_launches": int(timed.launches) * args.steps,
                "roots": {"count": len(roots), "converged": int(conv.sum()),
                          "roots_per_s": int(conv.sum()) / t_roots, "iterations": iters,
                          "stop_rule": "secant update <= %g |omega|" % POLISH_RTOL,
                          "reference_rule": {"iterations": iters_ref, "converged": int(conv_ref.sum()),
                                             "note": "|D| < D_threshold = %g (absolute)" % system.D_threshold},
                          "latency_ms": {"p50": float(np.percentile(lat, 50)) if lat else None,
                                         "p99": float(np.percentile(lat, 99)) if lat else None},
                          "roots": [[r.real, r.imag] for r in roots]},
                "served": served, "uneven_batch": uneven, "kscan": kscan, "relativistic": relat}
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
