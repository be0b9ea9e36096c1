"""f0 table files from a generate_distribution input file.

Mirrors the reference's offline tool (distribution/generate_distribution.f90)
for every distribution kind (0 distribution_analyt, 1 bi-Maxwellian,
2 bi-kappa, 3 Juettner, 4 bi-Moyal): reads its &system / &spec_i namelists and writes
<outdir>/<writeName>.<is>.array in the layout ALPS reads (read_f0).
"""
import os
import re

from . import _abi
from .api import generate_f0, write_f0


def _namelists(text):
    groups = {}
    for m in re.finditer(r"&(\w+)(.*?)\n\s*/", text, flags=re.S):
        body = "\n".join(line.split("!")[0] for line in m.group(2).splitlines())
        kv = {}
        for k, v in re.findall(r"(\w+)\s*=\s*([^\s,]+)", body):
            kv[k.lower()] = v.strip()
        groups[m.group(1).lower()] = kv
    return groups


def _num(v):
    return float(v.replace("d", "e").replace("D", "e"))


def _log(v):
    v = v.strip(".").lower()
    return v.startswith("t")


def read_distribution_input(path):
    g = _namelists(open(path).read())
    s = g["system"]
    nspec = int(_num(s["nspec"]))
    out = {"nspec": nspec, "nperp": int(_num(s["nperp"])), "npar": int(_num(s["npar"])),
           "writeName": s["writename"].strip("'\""), "species": []}
    kappa1 = None
    for i in range(1, nspec + 1):
        sp = g["spec_%d" % i]
        d = _abi.alps_dist_params()
        d.kind = int(_num(sp["distributions"]))
        d.ms = _num(sp["ms_read"])
        d.tau = _num(sp["taus"])
        d.alph = _num(sp["alphs"])
        d.p_drift = _num(sp["ps"])
        d.kappa = _num(sp.get("kappas", "0"))
        d.beta = _num(s["beta"])
        d.vA = _num(s["va"])
        d.maxP = _num(s["maxp"])
        d.autoscale = 1 if _log(sp.get("autoscales", "T")) else 0
        d.maxPperp = _num(sp.get("maxpperps", "1"))
        d.maxPpar = _num(sp.get("maxppars", "1"))
        if kappa1 is None:
            kappa1 = d.kappa
        d.kappa1 = kappa1
        d.species = i
        out["species"].append(d)
    return out


def generate_distribution(input_path, outdir):
    """Writes the f0 tables of a generate_distribution input; returns the
    list of (path, ideal fit parameters)."""
    spec = read_distribution_input(input_path)
    os.makedirs(outdir, exist_ok=True)
    res = []
    for i, d in enumerate(spec["species"], start=1):
        pperp, ppar, f0, ideal = generate_f0(d, spec["nperp"], spec["npar"])
        p = os.path.join(outdir, "%s.%d.array" % (spec["writeName"], i))
        write_f0(p, pperp, ppar, f0)
        res.append((p, ideal))
    return res
