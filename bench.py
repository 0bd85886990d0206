"""Benchmark: particle-steps/s of the PIC time step on one GB300.

Workload (the configuration the headline metric is quoted on): H plasma
(electrons and H+) with the collisional boundary of the reference's
"H with coll-boundary" preset -- energy-dependent e-H elastic and ionization
and H+-H charge exchange, electron-impact secondary emission, reflection and
backscatter, 10 injected particles per species per step -- on a 512x512-cell
grid (513x513 nodes), 16Mi particles per species, Gaussian density centred in
the box (sigma = L/4, truncated to the box), Maxwellian Te = 3 eV and
Ti = 0.026 eV.  Synthetic seeded data; inputs resident in HBM when the timed
region starts (the particle state, 0.9 GB, is larger than L2).

One JSON line is printed:
  value      device-timed particle-steps/s (sum over species of live particles
             x steps / CUDA-event time of the steps on the run's stream)
  e2e        the same metric through the C ABI with host buffers: every step
             uploads both species from pinned host memory, steps, and
             downloads them again
  roofline   the electron kernel (collisions + gather + push + deposit) at
             44 algorithmic bytes per particle slot (vz is rewritten only for
             the few electrons an event changed), against the measured HBM copy
             bandwidth
  cpu_baseline  the CPU oracle (restatement of the reference's C++ path) on a
             bounded sample, all host threads
`--impl reference` times that CPU path alone on the same metric.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

# many runs on their own streams (the batched and served forms): 32 hardware
# work queues instead of the default 8, so that unrelated streams do not
# queue behind one another (read when the CUDA context is created)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "vectorized-particle-in-cell-code-with-graphics_gb300")
sys.path.insert(0, PKG)

N_PER_SPECIES = 16 * 1024 * 1024
GRID_NODES = 513
# The electron kernels that can dominate a step, with their algorithmic bytes
# per electron slot and the profile field that times them (CUDA events the
# library records around each kernel in a profiled pass).  B = 0 in this
# workload, so the push neither reads nor writes vz.
ELECTRON_KERNELS = {
    "k_mcc": {"desc": "k_mcc (electron collision test, ionization list, scattering list)", "prof": "ms_collide_e",
              "alg_bytes": 24, "bytes_note": "read x, y, vx, vy, vz, id (24 B); the ~5% of events write back"},
    "k_push_e": {"desc": "k_push<DEP> (electrons: gather, push, deposit, wall list)", "prof": "ms_push_e_kernel",
                 "alg_bytes": 36, "bytes_note": "read x, y, vx, vy, w (20 B); write x, y, vx, vy (16 B)"},
}
METRIC = "particle-steps/s"
POISSON_DESC = {"FMG32": "full multigrid, the reference's schedule, FP32",
                "FMG_REF": "full multigrid, the reference's schedule, FP64 (bit-identical to the reference)",
                "FP32_DC": "FP32 full multigrid + FP64 defect correction (FP32 V-cycles)",
                "DST_DC": "FP32 sine-transform solve of the discrete system + FP64 defect correction"}
# defect-correction passes per mode.  FP32_DC: the FP32 full-multigrid pass
# and three FP64 corrections, each an FP32 V-cycle (phi within 3e-7 and E
# within 2e-6 of the converged FP64 solution on this workload's charge).
# DST_DC: the FP32 sine-transform solve (exact up to FP32 rounding) and one
# FP64 correction.
DC_PASSES = {"FP32_DC": 4, "DST_DC": 2}
# the Ar configurations' charge is rougher: five FP32_DC passes keep phi within
# 2e-6 of the converged solution at 257^2
ARGON_DC_PASSES = {"FP32_DC": 5, "DST_DC": 2}


def workload_params(picgb, seed=1003, n_per_species=N_PER_SPECIES, poisson="DST_DC", sort_interval=0,
                    dc_passes=None):
    """H preset ("H with coll-boundary") at 513^2 nodes and Te = 3 eV.  The
    macro-particle size is set so that the mean density equals the design
    density ELECTRON_PARTICLE_DENSITY = 1e15 m^-3 (parameters.h:71) for
    n_per_species particles, as INIT_PARTICLE_NO x 1e6 does in the preset."""
    kw = dict(X_NO_OF_CELLS=GRID_NODES, TEMPERATURE=3.0, ION_MASS_AMU=1.0, THRESHOLD=13.6, SPECIES="HYDROGEN",
              HAVE_COLLISIONS=True, SIGMA="ENERGY_DEPENDENT", SIGMA_ELASTIC="ENERGY_DEPENDENT",
              SIGMA_IONIZATION="ENERGY_DEPENDENT", E_IMPACT_SEE="YES", ION_IMPACT_SEE="NO", REFLECTION="YES",
              BACKSCATTER="YES", STEADYSTATE="NO", NUMBER_TO_INJECT=10, SIZE_TO_CHECK=2**31 - 1, RAND_SEED=seed,
              POISSON=poisson, DC_MAX_ITERS=dc_passes or DC_PASSES.get(poisson, 1), SORT_INTERVAL=sort_interval)
    L = picgb.make_params(**kw).xlength
    size = 1.0e15 * L * L / n_per_species
    return picgb.make_params(E_MACROPARTICLE_SIZE=size, ION_MACROPARTICLE_SIZE=size, **kw)


def argon_params(picgb, nodes, n_per_species, poisson="DST_DC", dc_passes=None, sort_interval=12, seed=1002,
                 torr=0.01, te=2.0):
    """Ar plasma in a square box with absorbing walls (the small and mid
    configurations): energy-dependent e-Ar and Ar+-Ar fits at `torr`,
    Te = `te`, no secondary emission; the macro-particle size gives the design
    density 1e15 m^-3 for n_per_species particles."""
    kw = dict(X_NO_OF_CELLS=nodes, TEMPERATURE=te, GAS_PRESSURE_TORR=torr, HAVE_COLLISIONS=True,
              SIGMA="ENERGY_DEPENDENT", SIGMA_ELASTIC="ENERGY_DEPENDENT", SIGMA_IONIZATION="ENERGY_DEPENDENT",
              STEADYSTATE="NO", SIZE_TO_CHECK=2**31 - 1, RAND_SEED=seed, POISSON=poisson,
              DC_MAX_ITERS=dc_passes or ARGON_DC_PASSES.get(poisson, 1), SORT_INTERVAL=sort_interval)
    L = picgb.make_params(**kw).xlength
    size = 1.0e15 * L * L / n_per_species
    return picgb.make_params(E_MACROPARTICLE_SIZE=size, ION_MACROPARTICLE_SIZE=size, **kw)


def uniform_state(p, n, te, ti, seed):
    """Positions uniform in (0, L)^2; Maxwellian velocities (sigma = sqrt(kT/m))."""
    rng = np.random.default_rng(seed)
    L = p.xlength
    out = []
    for m, T in ((9.10939e-31, te), (p.ion_mass, ti)):
        a = np.empty((n, 6))
        a[:, 0] = rng.uniform(0.0, L, n)
        a[:, 1] = rng.uniform(0.0, L, n)
        a[:, 2:5] = rng.normal(0.0, math.sqrt(T * 1.602177e-19 / m), (n, 3))
        a[:, 5] = 1.0
        out.append(a)
    return out


def gaussian_state(p, n, te, ti, seed, ion_mass):
    """Positions ~ N(L/2, (L/4)^2) truncated to (0, L)^2; Maxwellian velocities."""
    rng = np.random.default_rng(seed)
    L = p.xlength
    out = []
    for m, T in ((9.10939e-31, te), (ion_mass, ti)):
        a = np.empty((n, 6))
        for col in (0, 1):
            v = rng.normal(0.5 * L, 0.25 * L, n)
            bad = (v <= 0) | (v >= L)
            while bad.any():
                v[bad] = rng.normal(0.5 * L, 0.25 * L, int(bad.sum()))
                bad = (v <= 0) | (v >= L)
            a[:, col] = v
        a[:, 2:5] = rng.normal(0.0, math.sqrt(T * 1.602177e-19 / m), (n, 3))
        a[:, 5] = 1.0
        out.append(a)
    return out


class Clocks:
    """nvidia-smi clock and throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(r[1]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" in r[5 + k] and "Not" not in r[5 + k]})
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows)}


def measured_peak_hbm():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per launch of the step's particle kernels from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d
    except (OSError, ValueError):
        return None


# ------------------------------------------------------------------ CPU path
def cpu_sample(n_per_species, steps, threads, warmup=1, params=None, state=None):
    """The CPU path (the oracle: the reference's algorithm restated in FP64,
    OpenMP over the gather/push and deposit loops, its serial collisions,
    walls and one-pass FP64 multigrid) on the workload: warm-up steps, then
    particle-steps/s over `steps` steps."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import orc
    import picgb
    orc.build_port()
    p = params or workload_params(picgb, n_per_species=n_per_species, poisson="FMG_REF", sort_interval=0)
    e, i = state or gaussian_state(p, n_per_species, 3.0, 0.026, 1003, p.ion_mass)
    o = orc.Oracle(p, threads=threads)
    o.load_particles(0, e)
    o.load_particles(1, i)
    o.initial_boundary()
    o.step(max(warmup, 0))
    c0 = o.counters()
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    c1 = o.counters()
    o.close()
    ps = 0.5 * (c0["n_e"] + c0["n_i"] + c1["n_e"] + c1["n_i"]) * steps
    return ps / dt, dt


# ------------------------------------------------------------------ batched
def batched_configs(picgb, nruns, seed=1004):
    """Independent Ar runs (the batched workload): grids of 64, 128 or 256
    cells a side, particles per species log-uniform in [50k, 2M], neutral
    pressure uniform in [0.005, 0.05] Torr, Te uniform in [1, 4] eV,
    Ti = 0.026 eV, uniform positions, absorbing walls, the reference's
    energy-dependent e-Ar and Ar+-Ar fits."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nruns):
        nodes = int(rng.choice([65, 129, 257]))
        n = int(round(math.exp(rng.uniform(math.log(5e4), math.log(2e6)))))
        torr = float(rng.uniform(0.005, 0.05))
        te = float(rng.uniform(1.0, 4.0))
        kw = dict(X_NO_OF_CELLS=nodes, TEMPERATURE=te, GAS_PRESSURE_TORR=torr, HAVE_COLLISIONS=True,
                  SIGMA="ENERGY_DEPENDENT", SIGMA_ELASTIC="ENERGY_DEPENDENT", SIGMA_IONIZATION="ENERGY_DEPENDENT",
                  STEADYSTATE="NO", SIZE_TO_CHECK=2**31 - 1, RAND_SEED=seed + k, POISSON="DST_DC", DC_MAX_ITERS=2, SORT_INTERVAL=8)
        L = picgb.make_params(**kw).xlength
        size = 1.0e15 * L * L / n
        p = picgb.make_params(E_MACROPARTICLE_SIZE=size, ION_MACROPARTICLE_SIZE=size, **kw)
        r2 = np.random.default_rng(seed + 1000 + k)
        st = []
        for m, T in ((9.10939e-31, te), (p.ion_mass, 0.026)):
            a = np.empty((n, 6))
            a[:, 0] = r2.uniform(0.0, L, n)
            a[:, 1] = r2.uniform(0.0, L, n)
            a[:, 2:5] = r2.normal(0.0, math.sqrt(T * 1.602177e-19 / m), (n, 3))
            a[:, 5] = 1.0
            st.append(a)
        out.append((p, st, nodes, n))
    return out


def run_batched(args):
    """Plain form (one run after the other, pgb_step) against the batched form
    (pgb_step_batch over all runs) from the same states."""
    import picgb
    cfgs = batched_configs(picgb, args.batch_runs)
    runs = [picgb.Run(p) for p, _, _, _ in cfgs]

    def load():
        for r, (_, st, _, _) in zip(runs, cfgs):
            r.load_particles(0, st[0])
            r.load_particles(1, st[1])
            r.set_time_step(0)

    def total():
        return sum(r.particle_size(0) + r.particle_size(1) for r in runs)

    res = {}
    for form in ("plain", "batched"):
        load()
        # warm-up: graphs of every run are captured outside the timed region
        for r in runs:
            r.step(2)
        load()
        n0 = total()
        t0 = time.perf_counter()
        if form == "plain":
            for r in runs:
                r.step(args.batch_steps)
        else:
            picgb.step_batch(runs, args.batch_steps)
        dt = time.perf_counter() - t0
        n1 = total()
        ps = 0.5 * (n0 + n1) * args.batch_steps
        res[form] = {"seconds": dt, "particle_steps_per_s": ps / dt, "runs_per_s": len(runs) / dt,
                     "ms_per_step_of_every_run": 1000.0 * dt / args.batch_steps}
    for r in runs:
        r.close()
    res["speedup"] = res["batched"]["particle_steps_per_s"] / res["plain"]["particle_steps_per_s"]
    res["config"] = {"runs": len(cfgs), "steps_per_run": args.batch_steps,
                     "grid_nodes": sorted(set(c[2] for c in cfgs)),
                     "particles_per_species": [min(c[3] for c in cfgs), max(c[3] for c in cfgs)],
                     "workload": "independent Ar runs, absorbing walls, e-Ar and Ar+-Ar collisions; grids "
                                 "64/128/256 cells, 50k-2M particles/species log-uniform, 0.005-0.05 Torr, "
                                 "Te 1-4 eV (seeded)"}
    return res


# ------------------------------------------------------------------ served
def served_requests(picgb, nreq, max_steps, seed=1005):
    """Run requests arriving as a Poisson process (mean 20 per second): Ar or
    H, grids of 64 to 512 cells a side, particles per species log-uniform in
    [50k, 8M], steps log-uniform in [max_steps/10, max_steps], uniform
    positions, absorbing walls with the species' energy-dependent collision
    fits."""
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    for k in range(nreq):
        t += float(rng.exponential(1.0 / 20.0))
        nodes = int(rng.choice([65, 129, 257, 513]))
        n = int(round(math.exp(rng.uniform(math.log(5e4), math.log(8e6)))))
        steps = int(round(math.exp(rng.uniform(math.log(max_steps / 10), math.log(max_steps)))))
        hydrogen = bool(rng.integers(0, 2))
        te = float(rng.uniform(1.0, 4.0))
        kw = dict(X_NO_OF_CELLS=nodes, TEMPERATURE=te, GAS_PRESSURE_TORR=float(rng.uniform(0.005, 0.05)),
                  HAVE_COLLISIONS=True, SIGMA="ENERGY_DEPENDENT", SIGMA_ELASTIC="ENERGY_DEPENDENT",
                  SIGMA_IONIZATION="ENERGY_DEPENDENT", STEADYSTATE="NO", SIZE_TO_CHECK=2**31 - 1,
                  RAND_SEED=seed + k, POISSON="DST_DC", DC_MAX_ITERS=2, SORT_INTERVAL=8)
        if hydrogen:
            kw.update(ION_MASS_AMU=1.0, THRESHOLD=13.6, SPECIES="HYDROGEN")
        L = picgb.make_params(**kw).xlength
        size = 1.0e15 * L * L / n
        p = picgb.make_params(E_MACROPARTICLE_SIZE=size, ION_MACROPARTICLE_SIZE=size, **kw)
        r2 = np.random.default_rng(seed + 1000 + k)
        st = []
        for m, T in ((9.10939e-31, te), (p.ion_mass, 0.026)):
            a = np.empty((n, 6))
            a[:, 0] = r2.uniform(0.0, L, n)
            a[:, 1] = r2.uniform(0.0, L, n)
            a[:, 2:5] = r2.normal(0.0, math.sqrt(T * 1.602177e-19 / m), (n, 3))
            a[:, 5] = 1.0
            st.append(a)
        out.append((t, p, st, steps, nodes))
    return out


def _quantile(pairs, q):
    """q-quantile of (value, weight) pairs"""
    if not pairs:
        return None
    pairs = sorted(pairs)
    tot = sum(w for _, w in pairs)
    acc = 0
    for v, w in pairs:
        acc += w
        if acc >= q * tot:
            return v
    return pairs[-1][0]


def run_served(args):
    """The served form (pgb_server: requests admitted by HBM footprint as they
    arrive, resident runs stepped together in rounds) against the plain
    form (each request run alone, in arrival order), on the same arrivals."""
    import torch
    import picgb
    reqs = served_requests(picgb, args.serve_requests, args.serve_max_steps)
    free, _ = torch.cuda.mem_get_info()
    budget = int(0.5 * free)
    res = {}
    # served
    srv = picgb.Server(budget, round_steps=args.serve_round, max_active=64)
    arrival, finish, particle_steps = {}, {}, 0.0
    t0 = time.perf_counter()
    nxt = 0
    while len(finish) < len(reqs):
        now = time.perf_counter() - t0
        while nxt < len(reqs) and reqs[nxt][0] <= now:
            t, p, st, steps, _ = reqs[nxt]
            rid = srv.submit(p, st[0], st[1], steps)
            arrival[rid] = t
            nxt += 1
        s = srv.stats()
        if s["active"] == 0 and s["queued"] == 0:
            time.sleep(max(0.0, reqs[nxt][0] - now))
            continue
        srv.round()
        for rid in srv.results():
            finish[rid] = time.perf_counter() - t0
    wall = time.perf_counter() - t0
    s = srv.stats()
    srv.close()
    res["served"] = {"seconds": wall, "particle_steps_per_s": s["particle_steps"] / wall,
                     "step_ms_p50": s["step_ms_p50"], "step_ms_p99": s["step_ms_p99"],
                     "host_seconds": {k: s[k] for k in ("busy_seconds", "admit_seconds", "retire_seconds",
                                                        "issue_seconds")},
                     "ttc_s_p50": _quantile([(finish[k] - arrival[k], 1) for k in finish], 0.5),
                     "ttc_s_p99": _quantile([(finish[k] - arrival[k], 1) for k in finish], 0.99)}
    # plain: one request at a time in arrival order
    steps_ms, ttc, ps = [], [], 0.0
    solo = []
    t0 = time.perf_counter()
    for t, p, st, steps, _ in reqs:
        now = time.perf_counter() - t0
        if now < t:
            time.sleep(t - now)
        ta = time.perf_counter()
        with picgb.Run(p) as r:
            r.load_particles(0, st[0])
            r.load_particles(1, st[1])
            r.initial_boundary()
            n0 = r.particle_size(0) + r.particle_size(1)
            a = time.perf_counter()
            r.step(steps)
            b = time.perf_counter()
            n1 = r.particle_size(0) + r.particle_size(1)
            r.get_particles(0)
            r.get_particles(1)
        steps_ms.append((1000.0 * (b - a) / steps, steps))
        ps += 0.5 * (n0 + n1) * steps
        solo.append(time.perf_counter() - ta)
        ttc.append((time.perf_counter() - t0 - t, 1))
    wall = time.perf_counter() - t0
    res["plain"] = {"seconds": wall, "particle_steps_per_s": ps / wall, "step_ms_p50": _quantile(steps_ms, 0.5),
                    "step_ms_p99": _quantile(steps_ms, 0.99), "ttc_s_p50": _quantile(ttc, 0.5),
                    "ttc_s_p99": _quantile(ttc, 0.99)}
    res["speedup"] = res["served"]["particle_steps_per_s"] / res["plain"]["particle_steps_per_s"]
    # no schedule can finish before every request's arrival plus its time alone
    res["critical_path_s"] = max(r[0] + d for r, d in zip(reqs, solo))
    res["config"] = {"requests": len(reqs), "arrivals": "Poisson, mean 20 per second (seeded)",
                     "grid_nodes": sorted(set(r[4] for r in reqs)),
                     "particles_per_species": [min(r[2][0].shape[0] for r in reqs), max(r[2][0].shape[0] for r in reqs)],
                     "steps": [min(r[3] for r in reqs), max(r[3] for r in reqs)], "round_steps": args.serve_round,
                     "hbm_budget_bytes": budget,
                     "workload": "Ar or H runs, absorbing walls, energy-dependent collision fits, uniform positions, "
                                 "grids 64-512 cells, 50k-8M particles/species, 500-5000 steps; a bounded number "
                                 "of requests of the served workload"}
    return res


# ------------------------------------------------------------------ GPU path
def run_render(run, args, picgb, size=1024):
    """Wall time of one pgb_render call (the viewer's plots at size x size,
    the 3 MB image copied to host memory) on the bench state after its
    steps.  The reference draws these with OpenGL, which is unavailable on
    this box, so no reference time exists."""
    frames = {}
    cases = [("particle_xy", 0), ("particle_xy", picgb.NUM_PARTICLES_TO_PLOT), ("electron_vx_vy", 0), ("phi", 0),
             ("e_density", 0)]
    for plot, max_points in cases:
        run.render(plot, size, size, max_points)   # allocation and warm-up
        t0 = time.perf_counter()
        for k in range(args.render_frames):
            run.render(plot, size, size, max_points, seed=k)
        ms = 1000.0 * (time.perf_counter() - t0) / args.render_frames
        frames[f"{plot}{'' if max_points == 0 else f'_{max_points}_per_species'}"] = ms
    return {"ms_per_frame": frames, "width": size, "height": size,
            "particles_per_species": [run.particle_size(0), run.particle_size(1)],
            "note": "wall time of pgb_render through the C ABI, image copied to pageable host memory; "
                    "OpenGL reference unavailable on this box"}


def run_gpu(args, rank, world):
    import torch
    import picgb
    import build_lib
    build_lib.build()
    torch.cuda.set_device(rank % max(torch.cuda.device_count(), 1))
    n = int(N_PER_SPECIES * args.scale)
    p = workload_params(picgb, seed=1003 + rank, n_per_species=n, poisson=args.poisson, sort_interval=args.sort)
    e, i = gaussian_state(p, n, 3.0, 0.026, 1003 + rank, p.ion_mass)
    # launch shapes (they change no result): pgb_autotune on a separate run
    # of the same state, then the measured run uses the fastest candidate
    tune = None
    if args.autotune_steps > 0:
        with picgb.Run(p) as tr:
            tr.load_particles(0, e)
            tr.load_particles(1, i)
            tr.initial_boundary()
            tune = tr.autotune(args.autotune_steps)
    run = picgb.Run(p)
    run.load_particles(0, e)
    run.load_particles(1, i)
    run.initial_boundary()
    if tune:
        run.set_launch_config(tune["push_blocks_per_sm"], tune["field_sms"])
    run.step(args.warmup)
    stream = torch.cuda.ExternalStream(run.stream())
    c0 = run.counters()
    l0 = run.profile()["launches"]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(torch.cuda.current_device()) as clk:
        ev0.record(stream)
        run.step(args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = ev0.elapsed_time(ev1)
    c1 = run.counters()
    launches = run.profile()["launches"] - l0
    ps = 0.5 * (c0["n_e"] + c0["n_i"] + c1["n_e"] + c1["n_i"]) * args.steps
    # per-phase device time of the same step sequence (separate pass)
    run.set_profiling(True)
    run.step(min(args.steps, 50))
    prof = run.profile()
    run.set_profiling(False)
    # end to end through the C ABI with host buffers
    e2e = None
    if args.e2e_steps > 0:
        ne, ni = run.particle_size(0), run.particle_size(1)
        he = torch.empty((max(ne, 1) + 4096, 6), dtype=torch.float64, pin_memory=True)
        hi = torch.empty((max(ni, 1) + 4096, 6), dtype=torch.float64, pin_memory=True)
        ne = run.dump_particles_ptr(0, he.data_ptr(), he.shape[0])
        ni = run.dump_particles_ptr(1, hi.data_ptr(), hi.shape[0])
        h2d = d2h = 0
        tot = 0.0
        parts = {"load": 0.0, "step": 0.0, "dump": 0.0}
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            ta = time.perf_counter()
            run.load_particles_ptr(0, he.data_ptr(), ne)
            run.load_particles_ptr(1, hi.data_ptr(), ni)
            h2d += 48 * (ne + ni)
            tb = time.perf_counter()
            run.step(1)
            tc = time.perf_counter()
            ne2 = run.dump_particles_ptr(0, he.data_ptr(), he.shape[0])
            ni2 = run.dump_particles_ptr(1, hi.data_ptr(), hi.shape[0])
            td = time.perf_counter()
            parts["load"] += tb - ta
            parts["step"] += tc - tb
            parts["dump"] += td - tc
            d2h += 48 * (min(ne2, he.shape[0]) + min(ni2, hi.shape[0]))
            tot += 0.5 * (ne + ni + ne2 + ni2)
            ne, ni = min(ne2, he.shape[0]), min(ni2, hi.shape[0])
        wall = time.perf_counter() - t0
        e2e = {"value": tot / wall, "unit": METRIC, "h2d_bytes_per_step": h2d // args.e2e_steps,
               "d2h_bytes_per_step": d2h // args.e2e_steps, "steps": args.e2e_steps,
               "ms_per_step": {k: 1000.0 * v / args.e2e_steps for k, v in parts.items()},
               "note": "wall time per call: pgb_load_species (both species, pinned AoS doubles to device SoA), "
                       "pgb_step(1), pgb_dump_species (both)"}
    render = run_render(run, args, picgb) if args.render_frames > 0 else None
    run.close()
    # accuracy against the FP64 oracle, from the bench state, on a fresh run
    accuracy = None
    if args.accuracy_steps > 0 and world == 1:
        accuracy = run_accuracy(args, picgb, p, e, i)
        accuracy["poisson"] = POISSON_DESC[args.poisson] + (f", {p.dc_max_iters} passes"
                                                            if args.poisson in DC_PASSES else "")
    modes = run_modes(args, picgb, e, i, n) if (args.mode_steps > 0 and world == 1) else None
    del e, i
    configs = run_configs(args, picgb, os.cpu_count() or 1) if (args.configs and world == 1) else None
    batched = run_batched(args) if (args.batch_runs > 0 and world == 1) else None
    served = run_served(args) if (args.serve_requests > 0 and world == 1) else None
    return dict(ms=ms, ps=ps, counts=(c0, c1), prof=prof, launches=launches, clocks=clk.summary(), e2e=e2e, n=n,
                tune=tune,
                batched=batched, served=served, render=render, accuracy=accuracy, modes=modes, configs=configs)


def time_steps(run, steps):
    """CUDA-event time of `steps` steps on the run's stream (ms) and the
    particle-steps they did."""
    import torch
    st = torch.cuda.ExternalStream(run.stream())
    c0 = run.counters()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    run.step(steps)
    b.record(st)
    torch.cuda.synchronize()
    c1 = run.counters()
    return a.elapsed_time(b), 0.5 * (c0["n_e"] + c0["n_i"] + c1["n_e"] + c1["n_i"]) * steps


def run_modes(args, picgb, e, i, n):
    """The step with the other Poisson modes, same state and schedule:
    FMG_REF (the reference's one-pass FP64 full multigrid, bit-identical to
    it), FMG32 (that schedule in FP32, 1e-5-2e-5 of phi from it), and the
    two converged modes FP32_DC and DST_DC, whichever is not the headline."""
    out = {}
    for mode in [m for m in ("FMG_REF", "FMG32", "FP32_DC", "DST_DC") if m != args.poisson]:
        p = workload_params(picgb, n_per_species=n, poisson=mode, sort_interval=args.sort)
        with picgb.Run(p) as r:
            r.load_particles(0, e)
            r.load_particles(1, i)
            r.initial_boundary()
            r.step(args.warmup)
            ms, ps = time_steps(r, args.mode_steps)
        out[mode] = {"ms_per_step": ms / args.mode_steps, "value": ps / (ms / 1000.0), "steps": args.mode_steps}
    return out


def run_accuracy(args, picgb, p, e, i):
    """Errors against the FP64 oracle (the checker: tests/fullsize.py) after
    args.accuracy_steps steps of the bench state on a fresh run (a used run
    keeps its counters and the field of its last step), outside every timed
    region."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import fullsize
    d = fullsize.compare(p, e, i, args.accuracy_steps, reference_solver=True)
    pt = d["particles"]
    return {"vs": "FP64 oracle: the reference's algorithm restated in FP64 with the same Philox draws and particle "
                  "order, its Poisson solve converged; tie particles (FP32-vs-FP64 threshold decisions that went "
                  "the other way) matched by id and counted",
            "steps": d["steps"], "norm": "max |d| / max |oracle|",
            "fields": d["grids_away_from_ties"], "fields_tie_corrected": d["grids_tie_corrected"],
            "fields_raw": d["grids"], "nodes_near_ties": d["nodes_near_ties"],
            "poisson_solver": d["solver"], "reference_one_pass_fmg": d["reference_solver"],
            "mean_energy_rel": {k: v["mean_energy_rel"] for k, v in pt.items()},
            "mean_energy_ev": {k: v["mean_energy_ev"] for k, v in pt.items()},
            "positions_cells": {k: v["pos_cells"] for k, v in pt.items()},
            "velocities_vt": {k: v["vel_vt"] for k, v in pt.items()},
            "ties": d["ties"], "count_diffs": {k: v for k, v in d["counts"].items() if v}}


def run_configs(args, picgb, threads):
    """The other single-run configurations.  C1: 65^2 nodes, 200k particles per
    species, Ar at 0.01 Torr, absorbing walls, Te = 2 eV, the reference's FP64
    Poisson solve, 1000 steps, on the GPU and on the CPU path (all host
    threads).  C2: 257^2 nodes, 4Mi per species, the same Ar setup, the FP32
    sine-transform solve with one FP64 defect correction, on the GPU."""
    out = {}
    for name, nodes, n, mode, steps, seed in (("C1_65_200k", 65, 200000, "FMG_REF", args.c1_steps, 1001),
                                              ("C2_257_4Mi", 257, 4 * 1024 * 1024, "DST_DC", args.c2_steps, 1002)):
        p = argon_params(picgb, nodes, n, poisson=mode, sort_interval=args.sort, seed=seed)
        e, i = uniform_state(p, n, 2.0, 0.026, seed)
        with picgb.Run(p) as r:
            r.load_particles(0, e)
            r.load_particles(1, i)
            r.initial_boundary()
            r.step(args.warmup)
            ms, ps = time_steps(r, steps)
        out[name] = {"gpu": {"value": ps / (ms / 1000.0), "ms_per_step": ms / steps, "steps": steps},
                     "poisson": POISSON_DESC[mode] + (f", {p.dc_max_iters} passes" if mode in DC_PASSES else "")}
        if name.startswith("C1") and not args.no_cpu and args.c1_cpu_steps > 0:
            p0 = argon_params(picgb, nodes, n, poisson="FMG_REF", sort_interval=0, seed=seed)
            v, dt = cpu_sample(n, args.c1_cpu_steps, threads, warmup=5, params=p0, state=(e, i))
            out[name]["cpu"] = {"value": v, "seconds": dt, "steps": args.c1_cpu_steps, "cores": threads,
                                "kind": "port"}
            out[name]["ratio_gpu_cpu"] = out[name]["gpu"]["value"] / v
    return out


def combine_ranks(ms: float, ps: float):
    """Every rank steps its own replica (weak scaling, no data-path
    collective): the job's time is the slowest rank's, its work the sum of
    the ranks' particle-steps.  Needs an initialised process group."""
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    tmax = torch.tensor([ms], dtype=torch.float64, device=dev)
    tsum = torch.tensor([ps], dtype=torch.float64, device=dev)
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
    return float(tmax[0]), float(tsum[0])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the 16Mi particles per species")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=4, help="timed steps of the CPU baseline (bench workload)")
    ap.add_argument("--ref-max-steps", type=int, default=50,
                    help="the reference arm times at most this many of --steps (stated in its line)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--poisson", default="DST_DC", choices=["FMG32", "FMG_REF", "FP32_DC", "DST_DC"])
    ap.add_argument("--sort", type=int, default=12,
                    help="spatial sort of the electrons every k steps, of the ions every 4k (0 = off)")
    ap.add_argument("--mode-steps", type=int, default=40, help="steps timed per other Poisson mode (0 = skip)")
    ap.add_argument("--accuracy-steps", type=int, default=2, help="steps of the oracle comparison (0 = skip)")
    ap.add_argument("--no-configs", dest="configs", action="store_false", help="skip the C1/C2 configurations")
    ap.add_argument("--c1-steps", type=int, default=1000)
    ap.add_argument("--c1-cpu-steps", type=int, default=1000)
    ap.add_argument("--c2-steps", type=int, default=200)
    ap.add_argument("--batch-runs", type=int, default=64, help="runs of the batched workload (0 = skip it)")
    ap.add_argument("--batch-steps", type=int, default=200, help="steps per run of the batched workload")
    ap.add_argument("--serve-requests", type=int, default=32, help="requests of the served workload (0 = skip it)")
    ap.add_argument("--serve-max-steps", type=int, default=5000, help="longest request of the served workload")
    ap.add_argument("--serve-round", type=int, default=10, help="steps per server round")
    ap.add_argument("--render-frames", type=int, default=10, help="frames per viewer plot timed (0 = skip)")
    ap.add_argument("--autotune-steps", type=int, default=16,
                    help="timed steps per launch-shape candidate before the run (0 = default shapes)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    n = int(N_PER_SPECIES * args.scale)
    config = {"workload": "H plasma, collisional boundary (SEE+reflection+backscatter, e-H elastic+ionization, "
                          "H+-H CX), 512x512 cells (513^2 nodes), Gaussian density sigma=L/4, Te=3 eV, Ti=0.026 eV",
              "grid_nodes": GRID_NODES, "particles_per_species": n,
              "l2": "inputs larger than L2 (particle state 0.9 GB at 16Mi per species)",
              "poisson": POISSON_DESC[args.poisson] + (f", {DC_PASSES[args.poisson]} passes"
                                                       if args.poisson in DC_PASSES else ""),
              "macro_particle_size": "mean density 1e15 m^-3", "sort_interval": args.sort,
              "parallelism": "replicas" if world > 1 else "single"}
    threads = os.cpu_count() or 1
    if args.impl == "reference":
        # the reference's algorithm (the FP64 restatement pinned bit for bit to
        # the reference's own code) on the host cores, on the bench workload
        if rank != 0:
            return
        steps = max(1, min(args.steps, args.ref_max_steps))
        v, dt = cpu_sample(n, steps, threads, warmup=args.warmup)
        rconfig = dict(config, poisson="the reference's one-pass full multigrid, FP64", sort_interval=0)
        line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus, "steps": steps,
                "warmup": args.warmup, "ms_per_step": 1000.0 * dt / steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "config": rconfig, "impl": "reference",
                "cpu_baseline": {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
                                 "sample": f"the bench workload at {n} particles per species on 513^2 nodes, "
                                           f"{args.warmup} warm-up and {steps} timed steps; the reference's "
                                           "algorithm restated in FP64 (bit-identical to the reference's own code "
                                           "on x86-64), OpenMP on the gather/push and deposit loops"},
                "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    res = run_gpu(args, rank, world)
    ms, ps = combine_ranks(res["ms"], res["ps"]) if world > 1 else (res["ms"], res["ps"])
    if rank != 0:
        return
    value = ps / (ms / 1000.0)
    prof = res["prof"]
    peak, peak_kind = measured_peak_hbm()
    steps_prof = max(prof["steps"], 1)
    slots = prof["slots_e"] / steps_prof
    tr = (ncu_traffic() or {}).get("kernels", {})
    lines = {}
    for key, k in ELECTRON_KERNELS.items():
        kms = prof[k["prof"]] / steps_prof
        ach = k["alg_bytes"] * slots / (kms / 1000.0) / 1e9 if kms > 0 else None
        lines[key] = {"kernel": k["desc"], "ms_per_launch": kms, "achieved": ach,
                      "frac": (ach / peak) if ach else None, "alg_bytes_per_particle": k["alg_bytes"],
                      "alg_bytes_note": k["bytes_note"],
                      "traffic": (tr.get(key) or {}).get("bytes_per_launch")}
    dom = max(lines, key=lambda key: lines[key]["ms_per_launch"])
    d = lines[dom]
    roofline = {"bound": "hbm", "achieved": d["achieved"], "peak": peak, "unit": "GB/s", "frac": d["frac"],
                "traffic": d["traffic"], "kernel": d["kernel"], "alg_bytes_per_particle": d["alg_bytes_per_particle"],
                "peak_kind": f"{peak_kind} hbm_gbs",
                "others": {key: v for key, v in lines.items() if key != dom},
                "phase_ms_per_step": {k: prof[k] / steps_prof for k in
                                      ("ms_push_e", "ms_collide_e", "ms_scatter_e", "ms_push_e_kernel", "ms_push_i",
                                       "ms_collide_ions", "ms_walls", "ms_fields")}}
    cpu = None
    if not args.no_cpu and world == 1:
        try:
            v, dt = cpu_sample(n, args.cpu_steps, threads, warmup=1)
            cpu = {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
                   "sample": f"the bench workload at {n} particles per species, 1 warm-up and {args.cpu_steps} "
                             f"timed steps ({dt:.1f} s CPU wall); the reference's algorithm restated in FP64 with "
                             "its one-pass FP64 multigrid"}
        except Exception as ex:  # the CPU baseline never blocks the GPU line
            cpu = {"value": None, "unit": METRIC, "cores": threads, "kind": "port", "sample": f"failed: {ex}"}
    c0, c1 = res["counts"]
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": ("f32 velocities and Poisson solve, int32 fixed-point positions, int64 fixed-point charge, "
                      "f64 defect correction and fields") if args.poisson in DC_PASSES else
                     "f32 velocities, int32 fixed-point positions; " + POISSON_DESC[args.poisson],
            "data": "synthetic (seeded)",
            "config": config, "e2e": res["e2e"], "roofline": roofline, "cpu_baseline": cpu,
            "gpu_launches": res["launches"], "clocks": res["clocks"],
            "autotune": res.get("tune") or {"off": "default launch shapes (push 8 blocks/SM, 32 SMs for the field solve)"},
            "accuracy": res.get("accuracy"), "poisson_modes": res.get("modes"), "configs": res.get("configs"),
            "particles": {"start": [c0["n_e"], c0["n_i"]], "end": [c1["n_e"], c1["n_i"]]},
            "batched": res.get("batched"), "served": res.get("served"), "render": res.get("render")}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
