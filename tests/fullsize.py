"""Oracle comparison at the benchmark's sizes: the CUDA library and the FP64
oracle (oracle/picport.c in its library mode: Philox draws, stable order,
OpenMP over the host cores) step the same seeded state, and the states are
compared quantity by quantity.

Test infrastructure: used by tests/test_full_size_parity.py and by the
accuracy block of bench.py (outside its timed region).  The product never
imports it.

Workloads, as the benchmark configurations name them:
  hydrogen_513   513^2 nodes, 16Mi particles per species, H plasma with the
                 collisional boundary (e-H elastic and ionization, H+-H charge
                 exchange, secondary emission, reflection, backscatter,
                 injection), Gaussian density sigma = L/4, Te = 3 eV; the
                 benchmark's state (bench.workload_params, gaussian_state)
  argon_257      257^2 nodes, 4Mi particles per species, Ar plasma, absorbing
                 walls, e-Ar and Ar+-Ar collisions at 0.01 Torr, uniform
                 positions, Te = 2 eV, Ti = 0.026 eV, FP32 multigrid with FP64
                 defect correction

Reported errors (max norm relative to the oracle's max |value|):
  q_e, q_i, rho, phi, ex, ey     after the last step
  positions                      max |d| in cells, over particles matched by id
  velocities                     max |d| / thermal speed, over particles whose
                                 random decisions agree (see ties)
  ties                           particles (matched by id) present on one side
                                 only, NaN on one side only, or whose velocity
                                 differs by more than 1e-2 of the thermal speed,
                                 or that deposits on one side only: a collision,
                                 wall or deposit-region decision that fell within
                                 FP32 rounding of its threshold went the other
                                 way (a particle created after such a decision
                                 takes the next id, so ids, not slots, pair the
                                 particles)
  grids_tie_corrected            the same grids against the oracle's deposit and
                                 solve of its final particles with the ties
                                 replaced by the device's: the FP32 error alone
  grids_away_from_ties           the tie-corrected comparison at nodes farther
                                 than TIE_RADIUS cells from every tie particle
                                 (nodes_near_ties: how many are nearer): a tie
                                 particle's charge changed the field around it
                                 in the steps after the decision and so moved
                                 its neighbours, which the swap cannot undo
  solver                         phi, ex, ey against the oracle's solve of the
                                 device's own rho: the Poisson mode's error alone
  mean energy                    relative difference of the mean kinetic energy
                                 per species
  counts                         device counters minus the oracle's
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "vectorized-particle-in-cell-code-with-graphics_gb300"))
sys.path.insert(0, HERE)
import orc  # noqa: E402
import picgb  # noqa: E402

GRIDS = ("q_e", "q_i", "rho", "phi", "ex", "ey")
COUNTS = ("n_e", "n_i", "absorbed_e", "absorbed_i", "reflected", "backscattered", "see_events", "see_emitted",
          "ion_see_emitted", "elastic", "ionization", "charge_exchange", "injected_e", "injected_i")
TIE_VT = 1e-2
TIE_RADIUS = 6   # cells around a tie particle whose field moved its neighbours


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    scale = np.max(np.abs(b))
    d = float(np.max(np.abs(a - b))) if a.size else 0.0
    return d / scale if scale > 0 else d


def argon_257_params(n_per_species, poisson="FP32_DC", dc_passes=5, sort_interval=12, seed=1002):
    """257^2 nodes, Ar at 0.01 Torr, Te = 2 eV, absorbing walls, energy-dependent
    e-Ar and Ar+-Ar fits; the macro-particle size gives the design density
    1e15 m^-3 for n_per_species particles.  A uniform quasi-neutral plasma
    has a charge density of nearly white noise, the slowest right-hand side
    for the multigrid: five FP32_DC passes keep phi within 2e-6 of the FP64
    solution (four leave 9e-6)."""
    kw = dict(X_NO_OF_CELLS=257, TEMPERATURE=2.0, GAS_PRESSURE_TORR=0.01, HAVE_COLLISIONS=True,
              SIGMA="ENERGY_DEPENDENT", SIGMA_ELASTIC="ENERGY_DEPENDENT", SIGMA_IONIZATION="ENERGY_DEPENDENT",
              STEADYSTATE="NO", SIZE_TO_CHECK=2**31 - 1, RAND_SEED=seed, POISSON=poisson, DC_MAX_ITERS=dc_passes,
              SORT_INTERVAL=sort_interval)
    L = picgb.make_params(**kw).xlength
    size = 1.0e15 * L * L / n_per_species
    return picgb.make_params(E_MACROPARTICLE_SIZE=size, ION_MACROPARTICLE_SIZE=size, **kw)


def uniform_state(p, n, te, ti, seed):
    """Positions uniform in (0, L)^2; Maxwellian velocities (sigma = sqrt(kT/m))."""
    rng = np.random.default_rng(seed)
    L = p.xlength
    out = []
    for m, T in ((picgb.ELECTRON_MASS, te), (p.ion_mass, ti)):
        a = np.empty((n, 6))
        a[:, 0] = rng.uniform(0.0, L, n)
        a[:, 1] = rng.uniform(0.0, L, n)
        a[:, 2:5] = rng.normal(0.0, math.sqrt(T * picgb.CHARGE / m), (n, 3))
        a[:, 5] = 1.0
        out.append(a)
    return out


def _mean_energy(a, m):
    fin = np.isfinite(a).all(axis=1)
    v2 = np.sum(a[fin, 2:5] ** 2, axis=1)
    return 0.5 * m * float(np.mean(v2)) / picgb.CHARGE if v2.size else 0.0


def _deposits(a, p):
    """collect_charge's test per particle (pic.cl:31-37): jp < nx-1 && x > 0
    && kp < ny-1 && y > 0, with jp, kp truncated toward zero (the frozen
    strip (-DX, 0] and the ghost strip deposit nothing)."""
    dx = p.xlength / (p.x_no_of_cells - 1)
    dy = p.ylength / (p.y_no_of_cells - 1)
    with np.errstate(invalid="ignore"):
        jp, kp = np.trunc(a[:, 0] / dx), np.trunc(a[:, 1] / dy)
        return (a[:, 0] > 0) & (a[:, 1] > 0) & (jp < p.x_no_of_cells - 1) & (kp < p.y_no_of_cells - 1)


def _match(a, ia, b, ib, p, vt):
    """Device particles (a, ids ia) against the oracle's (b, ids ib), matched
    by id.  Ties: ids on one side only, NaN on one side only, a velocity
    difference above TIE_VT thermal speeds, or positions on the two sides of
    a wall of the deposit region (a position within FP32 rounding of x = 0
    deposits on one side only)."""
    dx = p.xlength / (p.x_no_of_cells - 1)
    top = int(max(ia.max(initial=0), ib.max(initial=0))) + 1
    where_b = np.full(top, -1, dtype=np.int64)
    where_b[ib] = np.arange(ib.size)
    kb = where_b[ia]
    inb = kb >= 0
    ka = np.nonzero(inb)[0]
    kb = kb[inb]
    a2, b2 = a[ka], b[kb]
    fa, fb = np.isfinite(a2).all(axis=1), np.isfinite(b2).all(axis=1)
    both = fa & fb
    dvel = np.zeros(ka.size)
    dvel[both] = np.max(np.abs(a2[both, 2:5] - b2[both, 2:5]), axis=1) / vt
    tie = (fa != fb) | (dvel > TIE_VT) | (_deposits(a2, p) != _deposits(b2, p))
    ok = both & ~tie
    dpos = np.max(np.abs(a2[ok, :2] - b2[ok, :2]), axis=1) / dx if ok.any() else np.zeros(1)
    in_a = np.zeros(top, dtype=bool)
    in_a[ia] = True
    only_a = ia[~inb]
    only_b = ib[~in_a[ib]]
    tie_ids = np.concatenate([only_a, only_b, ia[ka[tie]]])
    return {"n": int(a.shape[0]), "n_oracle": int(b.shape[0]), "ties": int(tie_ids.size),
            "pos_cells": float(dpos.max()), "vel_vt": float(dvel[ok].max()) if ok.any() else 0.0,
            "weights_equal": bool(np.array_equal(a2[ok, 5].astype(np.float32), b2[ok, 5].astype(np.float32)))}, tie_ids


def _isin(ids, sel):
    """ids in sel, by direct address (ids are below 2^32 and dense)"""
    if sel.size == 0:
        return np.zeros(ids.size, dtype=bool)
    top = int(max(ids.max(initial=0), sel.max())) + 1
    m = np.zeros(top, dtype=bool)
    m[sel] = True
    return m[ids]


def _tie_corrected_fields(p, t, parts):
    """The oracle's deposit, rho, Poisson and E of the final particles, with
    each species' tie particles taken from the device: what the oracle's
    fields would be had its threshold decisions gone the device's way."""
    o = orc.Oracle(p, rng=orc.ORC_RNG_PHILOX, order=orc.ORC_ORDER_STABLE, threads=os.cpu_count() or 1)
    try:
        for s, (a, ia, b, ib, ties) in enumerate(parts):
            keep = ~_isin(ib, ties)
            take = _isin(ia, ties)
            o.load_particles(s, np.concatenate([b[keep], a[take]]))
        for s in (1, 0):
            o.deposit(s)
        o.grid_rho()
        o.poisson(t)
        o.efield()
        return {g: o.get_grid(g) for g in GRIDS}
    finally:
        o.close()


def _far_from_ties(p, parts):
    """Nodes farther than TIE_RADIUS cells from every tie particle (its final
    position on either side).  A tie particle's different charge changed
    the field around it in the steps after the decision, which moved its
    neighbours together; the tie-corrected grids still hold that.  The rest
    of the grid carries the FP32 error alone."""
    nx, ny = p.x_no_of_cells, p.y_no_of_cells
    dx, dy = p.xlength / (nx - 1), p.ylength / (ny - 1)
    near = np.zeros((ny, nx), dtype=bool)
    r = TIE_RADIUS
    for a, ia, b, ib, ties in parts:
        for P, I in ((a, ia), (b, ib)):
            sel = P[_isin(I, ties)]
            for x, y in sel[:, :2]:
                if not (np.isfinite(x) and np.isfinite(y)):
                    continue
                cx, cy = int(round(x / dx)), int(round(y / dy))
                near[max(cy - r, 0):max(cy + r + 1, 0), max(cx - r, 0):max(cx + r + 1, 0)] = True
    return ~near.ravel()


def _far_e(far, p):
    """the node mask on the stride-nx E layout ((nx+1)(ny+1) entries)"""
    nx, ny = p.x_no_of_cells, p.y_no_of_cells
    m = np.ones((nx + 1) * (ny + 1), dtype=bool)
    m[: nx * ny] = far
    return m


def _solver_only(p, t, gg):
    """The device's phi and E against the oracle's solve of the device's own
    rho (the FP64 solve the mode approximates): the solver's error alone."""
    o = orc.Oracle(p, rng=orc.ORC_RNG_PHILOX, order=orc.ORC_ORDER_STABLE)
    try:
        o.set_rho(gg["rho"].reshape(p.y_no_of_cells, p.x_no_of_cells))
        o.poisson(t)
        o.efield()
        return {g: rel_err(gg[g], o.get_grid(g)) for g in ("phi", "ex", "ey")}
    finally:
        o.close()


def _reference_solver(p, t, gg):
    """The reference's own solver (its one-pass FP64 full multigrid) on the
    device's rho against the converged FP64 solve: the algebraic error the
    reference carries, for scale."""
    out = {}
    for mode in (picgb.PGB_POISSON_FMG_REF, picgb.PGB_POISSON_FP32_DC):
        q = type(p).from_buffer_copy(p)
        q.poisson_mode = mode
        o = orc.Oracle(q, rng=orc.ORC_RNG_PHILOX, order=orc.ORC_ORDER_STABLE)
        try:
            o.set_rho(gg["rho"].reshape(p.y_no_of_cells, p.x_no_of_cells))
            o.poisson(t)
            o.efield()
            out[mode] = {g: o.get_grid(g) for g in ("phi", "ex", "ey")}
        finally:
            o.close()
    a, b = out[picgb.PGB_POISSON_FMG_REF], out[picgb.PGB_POISSON_FP32_DC]
    return {g: rel_err(a[g], b[g]) for g in a}


def compare(p, e, i, steps, threads=None, run=None, reference_solver=False):
    """Step the same state on the device and in the oracle; return the errors.
    `run`: a fresh picgb.Run to use (one that has stepped keeps its counters
    and the field of its last step, which the comparison would inherit).
    `reference_solver`: also report the reference's one-pass FP64 multigrid
    against the converged solve on the device's rho."""
    threads = threads or (os.cpu_count() or 1)
    o = orc.Oracle(p, rng=orc.ORC_RNG_PHILOX, order=orc.ORC_ORDER_STABLE, threads=threads)
    r = run or picgb.Run(p)
    try:
        for x in (o, r):
            x.load_particles(0, e)
            x.load_particles(1, i)
            x.set_time_step(0)
            x.initial_boundary()
        r.step(steps)
        o.step(steps)
        cr, co = r.counters(), o.counters()
        gg = {g: r.get_grid(g) for g in GRIDS}
        out = {"steps": steps, "grids": {g: rel_err(gg[g], o.get_grid(g)) for g in GRIDS},
               "counts": {k: cr[k] - co[k] for k in COUNTS}, "oracle_counts": {k: co[k] for k in COUNTS}}
        species, parts = {}, []
        for s, m, vt in ((0, picgb.ELECTRON_MASS, p.vte), (1, p.ion_mass, p.vti)):
            a, ia = r.get_particles(s), r.get_ids(s)
            b, ib = o.get_particles(s, with_ids=True)
            d, ties = _match(a, ia, b, ib, p, vt)
            ea, eb = _mean_energy(a, m), _mean_energy(b, m)
            d["mean_energy_ev"] = eb
            d["mean_energy_rel"] = abs(ea - eb) / eb if eb > 0 else abs(ea - eb)
            species["electrons" if s == 0 else "ions"] = d
            parts.append((a, ia, b, ib, ties))
        out["particles"] = species
        out["ties"] = sum(d["ties"] for d in species.values())
        fixed = _tie_corrected_fields(p, steps - 1, parts) if out["ties"] else None
        out["grids_tie_corrected"] = ({g: rel_err(gg[g], fixed[g]) for g in GRIDS} if fixed is not None
                                      else dict(out["grids"]))
        ref = fixed if fixed is not None else {g: o.get_grid(g) for g in GRIDS}
        far = _far_from_ties(p, parts)
        out["nodes_near_ties"] = int((~far).sum())
        out["grids_away_from_ties"] = {}
        for g in GRIDS:
            a_, b_ = gg[g].ravel(), ref[g].ravel()
            m = far if a_.size == far.size else _far_e(far, p)
            scale = np.max(np.abs(b_))
            out["grids_away_from_ties"][g] = float(np.max(np.abs(a_[m] - b_[m])) / scale) if scale > 0 else 0.0
        out["solver"] = _solver_only(p, steps - 1, gg)
        if reference_solver:
            out["reference_solver"] = _reference_solver(p, steps - 1, gg)
        return out
    finally:
        o.close()
        if run is None:
            r.close()
