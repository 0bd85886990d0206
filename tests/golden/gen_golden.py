"""Write the golden fixtures of the reference's own C++ code.

Run in a container that has the reference sources (it builds
oracle/_ref/ref_<config> with oracle/Makefile, i.e. the reference's
pic::pic_run, particle, fields, Mglin, collision and boundary classes
compiled unchanged from their sources behind an in-process OpenCL stand-in).

    PIC_REFERENCE_DIR=<reference sources> python tests/golden/gen_golden.py [case ...]

For every case it writes tests/golden/<case>.npz holding
  params   JSON of the parameters.h-style inputs (picgb.make_params keywords)
  e_in, i_in         the loaded particle state (dataDump_e.txt / dataDump_i1.txt)
  nsteps             time steps run by pic_run
  e_out, i_out       particles after the run (6 doubles each, the reference's order)
  q_e, q_i, rho, phi, ex, ey   grids after the run, reference layouts
Field-only cases (mode "fields") hold rho and the reference's phi, ex, ey
for one fields::grid_potential + grid_electric_field call.  Cases with a
graph window also hold graph_window (start, end) and graph_<file> for every
text file the reference's graphs class wrote at the end of the window.

sigma_fits.npz holds the reference's six energy-dependent cross-section fits
(e_collisions.cpp:205-308, ion_collisions.cpp:170-199) on a fixed energy list.

The states are seeded synthetic plasmas sized so that every code path of the
case is exercised in a few steps (particles crossing walls, collisions,
secondary emission, steady-state re-insertion).  The numbers are test data
generated here, not data shipped with the reference.
"""
from __future__ import annotations

import json
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "vectorized-particle-in-cell-code-with-graphics_gb300"))
import picgb  # noqa: E402

AR_COLL = dict(HAVE_COLLISIONS=True, SIGMA="ENERGY_DEPENDENT", SIGMA_ELASTIC="ENERGY_DEPENDENT",
               SIGMA_IONIZATION="ENERGY_DEPENDENT")

# case -> (reference build, make_params keywords, state recipe, steps)
CASES = {
    "core33": ("core33", dict(X_NO_OF_CELLS=33), dict(n=1000, te=30.0, ti=5.0, seed=11), 10),
    "core65": ("core65", dict(X_NO_OF_CELLS=65), dict(n=2000, te=8.0, ti=2.0, seed=12), 6),
    "bfield33": ("bfield33", dict(X_NO_OF_CELLS=33, MAGNETIC_FIELD=0.05, PHI_RIGHT=2.0, PHI_TOP=-1.0, PHI_PERIOD=0.01),
                 dict(n=1000, te=20.0, ti=5.0, seed=13), 10),
    "steady33": ("steady33", dict(X_NO_OF_CELLS=33, STEADYSTATE="YES"),
                 dict(n=1000, te=20.0, ti=200.0, seed=14, outside=0.25), 8),
    "arcoll33": ("arcoll33", dict(X_NO_OF_CELLS=33, GAS_PRESSURE_TORR=1.0, TEMPERATURE=2.0, **AR_COLL),
                 dict(n=1000, te=10.0, ti=400.0, seed=15), 10),
    "arsee33": ("arsee33", dict(X_NO_OF_CELLS=33, NUMBER_TO_INJECT=10, E_IMPACT_SEE="YES", ION_IMPACT_SEE="YES",
                                REFLECTION="YES", BACKSCATTER="YES", **AR_COLL),
                dict(n=1000, te=150.0, ti=3000.0, seed=16), 8),
    "hsee33": ("hsee33", dict(X_NO_OF_CELLS=33, NUMBER_TO_INJECT=10, ION_MASS_AMU=1.0, THRESHOLD=13.6, SPECIES="HYDROGEN",
                              TEMPERATURE=3.0, E_IMPACT_SEE="YES", REFLECTION="YES", BACKSCATTER="YES", **AR_COLL),
               dict(n=1000, te=120.0, ti=20.0, seed=17), 8),
    "see33": ("see33", dict(X_NO_OF_CELLS=33, E_IMPACT_SEE="YES", ION_IMPACT_SEE="YES", REFLECTION="YES",
                            BACKSCATTER="YES"),
              dict(n=1000, te=200.0, ti=3000.0, seed=18, outside=0.2), 8),
    "reduce33": ("reduce33", dict(X_NO_OF_CELLS=33, NUMBER_TO_INJECT=20, SIZE_TO_CHECK=900, UPPER_GROUP_LIMIT=550,
                                  NEW_GROUP_SIZE=520, UPPER_GROUP_LIMIT2=200, NEW_GROUP_SIZE2=180),
                 dict(n=1000, te=3.0, ti=3.0, seed=19), 10),
    "graphs33": ("core33", dict(X_NO_OF_CELLS=33), dict(n=4000, te=10.0, ti=2.0, seed=23, graphs=(3, 8)), 10),
    "fields65": ("core65", dict(X_NO_OF_CELLS=65), dict(mode="fields", seed=21), 0),
    "fields129": ("core129", dict(X_NO_OF_CELLS=129), dict(mode="fields", seed=22), 0),
}


# files the reference's graphs class writes at the end of the graph window
# (graphs.cpp:1167-1370); e = electrons, i1 = the ion species
GRAPH_FILES = ["rho_phi_EgridX", "rho_phi_EgridY", "rho2d", "phi2d", "egrid2dX", "egrid2dY"] + [
    f"{stem}_{t}" for t in ("e", "i1")
    for stem in ("density2d", "av_velocity", "first_v_distX", "first_v_distY", "second_v_distX", "second_v_distY")]


def make_state(p: picgb.PgbParams, n: int, te: float, ti: float, seed: int, outside: float = 0.0):
    """Uniform positions in (0, L)^2 and Maxwellian velocities (per-component
    sigma sqrt(kT/m)); a fraction `outside` is placed just beyond a wall."""
    rng = np.random.default_rng(seed)
    L = p.xlength
    out = []
    for m, T in ((picgb.ELECTRON_MASS, te), (p.ion_mass, ti)):
        x = rng.uniform(0.0, L, n)
        y = rng.uniform(0.0, L, n)
        if outside > 0:
            k = int(outside * n)
            side = rng.integers(0, 4, k)
            d = rng.uniform(0.05, 0.9, k) * (L / (p.x_no_of_cells - 1))
            x[:k] = np.where(side == 0, -d, np.where(side == 1, L + L / (p.x_no_of_cells - 1) + d, x[:k]))
            y[:k] = np.where(side == 2, -d, np.where(side == 3, L + L / (p.x_no_of_cells - 1) + d, y[:k]))
        vt = math.sqrt(T * picgb.CHARGE / m)
        v = rng.normal(0.0, vt, (n, 3))
        out.append(np.column_stack([x, y, v, np.ones(n)]))
    return out


def make_rho(p: picgb.PgbParams, seed: int):
    """A smooth charge density plus noise, of PIC-like magnitude (C/m^2)."""
    rng = np.random.default_rng(seed)
    n = p.x_no_of_cells
    s = np.linspace(0.0, 1.0, n)
    X, Y = np.meshgrid(s, s)
    base = np.exp(-((X - 0.4) ** 2 + (Y - 0.6) ** 2) / 0.05) - 0.5 * np.exp(-((X - 0.7) ** 2 + (Y - 0.3) ** 2) / 0.02)
    return (1.0e-6 * base + 2.0e-8 * rng.standard_normal((n, n))).ravel()


def write_dump(path, a):
    with open(path, "w") as f:
        for r in a:
            f.write(" ".join("%.17g" % v for v in r) + "\n")


def run_case(name, cfg, kw, recipe, nsteps, refdir):
    p = picgb.make_params(RAND_SEED=1, STEADYSTATE=kw.get("STEADYSTATE", "NO"),
                          **{k: v for k, v in kw.items() if k != "STEADYSTATE"})
    exe = os.path.join(refdir, f"ref_{cfg}")
    rec = dict(params=json.dumps(dict(kw, STEADYSTATE=kw.get("STEADYSTATE", "NO"), RAND_SEED=1)))
    with tempfile.TemporaryDirectory() as d:
        if recipe.get("mode") == "fields":
            rho = make_rho(p, recipe["seed"])
            rho.tofile(os.path.join(d, "rho.bin"))
            subprocess.run([exe, "fields", d], check=True)
            rec.update(mode="fields", rho=rho)
        else:
            e, i = make_state(p, recipe["n"], recipe["te"], recipe["ti"], recipe["seed"], recipe.get("outside", 0.0))
            write_dump(os.path.join(d, "dataDump_e.txt"), e)
            write_dump(os.path.join(d, "dataDump_i1.txt"), i)
            window = recipe.get("graphs")
            args = [exe, "run", d, str(nsteps)] + ([str(window[0]), str(window[1])] if window else [])
            subprocess.run(args, check=True)
            if window:
                rec["graph_window"] = np.array(window)
                for stem in GRAPH_FILES:
                    rec["graph_" + stem] = np.loadtxt(os.path.join(d, stem + ".txt"), ndmin=2)
            rec.update(mode="run", e_in=e, i_in=i, nsteps=nsteps,
                       e_out=np.fromfile(os.path.join(d, "e.bin")).reshape(-1, 6),
                       i_out=np.fromfile(os.path.join(d, "i1.bin")).reshape(-1, 6),
                       q_e=np.fromfile(os.path.join(d, "q_e.bin")),
                       q_i=np.fromfile(os.path.join(d, "q_i1.bin")),
                       rho=np.fromfile(os.path.join(d, "rho.bin")))
            with open(os.path.join(d, "dump_e.txt")) as f:
                rec["dump_e_head"] = "".join(f.readlines()[:20])
        for g in ("phi", "ex", "ey"):
            rec[g] = np.fromfile(os.path.join(d, f"{g}.bin"))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    return rec


SIGMA_COLUMNS = ("ar_elastic", "ar_ionize", "h_elastic", "h_ionize", "ar_cx", "h_cx")
# branch edges of the fits (eV); at the first four the reference leaves sigma
# uninitialised (e_collisions.cpp:208-253), so only the points around them
# are tabulated
SIGMA_EDGES_UNDEFINED = (0.35, 15.0, 15.755, 100.0)
SIGMA_EDGES = (0.01, 20.0, 13.6, 4.0, 1.0e-4 * 1000.0 * 1.66054e-27, 2.0e10 * 1000.0 * 1.66054e-27)


def sigma_energies():
    """10^4 log-spaced energies from 1e-5 to 1e5 eV, and points on both sides
    of every branch edge (one FP64 step and a relative 1e-6 away), the edge
    itself where the reference defines it."""
    e = list(np.geomspace(1e-5, 1e5, 10000))
    for b in SIGMA_EDGES + SIGMA_EDGES_UNDEFINED:
        e += [np.nextafter(b, 0.0), np.nextafter(b, np.inf), b * (1 - 1e-6), b * (1 + 1e-6)]
    e += list(SIGMA_EDGES)
    return np.array(sorted(set(e)), dtype=np.float64)


def sigma_table(refdir):
    """The reference's six cross-section fits on sigma_energies()."""
    e = sigma_energies()
    with tempfile.TemporaryDirectory() as d:
        e.tofile(os.path.join(d, "energies.bin"))
        subprocess.run([os.path.join(refdir, "ref_core33"), "sigma", d], check=True)
        sig = np.fromfile(os.path.join(d, "sigma.bin")).reshape(-1, 6)
    np.savez_compressed(os.path.join(HERE, "sigma_fits.npz"), energies=e, sigma=sig,
                        columns=np.array(SIGMA_COLUMNS))
    return e.size


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref"], check=True)
    refdir = os.path.join(REPO, "oracle", "_ref")
    only = sys.argv[1:]
    if not only or "sigma_fits" in only:
        print(f"sigma_fits: {sigma_table(refdir)} energies")
    for name, (cfg, kw, recipe, nsteps) in CASES.items():
        if only and name not in only:
            continue
        rec = run_case(name, cfg, kw, recipe, nsteps, refdir)
        extra = "" if rec["mode"] == "fields" else f" e {rec['e_in'].shape[0]}->{rec['e_out'].shape[0]}" \
                                                      f" i {rec['i_in'].shape[0]}->{rec['i_out'].shape[0]}"
        print(f"{name}: {rec['mode']}{extra}")


if __name__ == "__main__":
    main()
