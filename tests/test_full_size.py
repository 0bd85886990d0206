"""The benchmark's full size: 513^2 nodes and 16 Mi particles per species
of the hydrogen preset with the collisional boundary (SEE, reflection,
backscatter, e-H elastic and ionization, H+-H charge exchange), a Gaussian
density and the spatial sort every 8 steps; and the same for the argon
preset (Ar+-Ar charge exchange really fires, ion-impact SEE on).  The
oracle would take minutes at this size, so the checks are properties that
do not depend on size:

- the run is deterministic: the pipelined step run twice, and the same
  steps run in order (profiling), end bit for bit in the same state;
- the populations balance exactly with the device counters:
  n_e' = n_e + injected_e + see_emitted + ion_see_emitted + ionization
             - absorbed_e - see_events
  n_i' = n_i + injected_i + ionization - absorbed_i
  (a secondary-emission event replaces its parent electron by the emitted
  ones, boundary.cpp:494-529; ionization products that the reference's
  non-steady step drops count as added and absorbed at once);
- every particle left is finite and inside the domain or its ghost strip
  (pic.cl:112 gathers up to jp < nx), and the field is finite.
"""
import math

import numpy as np
import pytest

import picgb

pytestmark = pytest.mark.gpu

N = 16 * 1024 * 1024
STEPS = 12


SPECIES = {"hydrogen": dict(ION_MASS_AMU=1.0, THRESHOLD=13.6, SPECIES="HYDROGEN", ION_IMPACT_SEE="NO"),
           "argon": dict(SPECIES="ARGON", ION_IMPACT_SEE="YES")}


def _workload(species):
    kw = dict(X_NO_OF_CELLS=513, TEMPERATURE=3.0, HAVE_COLLISIONS=True, SIGMA="ENERGY_DEPENDENT",
              SIGMA_ELASTIC="ENERGY_DEPENDENT", SIGMA_IONIZATION="ENERGY_DEPENDENT", E_IMPACT_SEE="YES",
              REFLECTION="YES", BACKSCATTER="YES", STEADYSTATE="NO", NUMBER_TO_INJECT=10, SIZE_TO_CHECK=2**31 - 1,
              RAND_SEED=1003, POISSON="FMG32", SORT_INTERVAL=8, **SPECIES[species])
    L = picgb.make_params(**kw).xlength
    size = 1.0e15 * L * L / N
    p = picgb.make_params(E_MACROPARTICLE_SIZE=size, ION_MACROPARTICLE_SIZE=size, **kw)
    rng = np.random.default_rng(1003)
    out = []
    for m, t in ((picgb.ELECTRON_MASS, 3.0), (p.ion_mass, 0.026)):
        a = np.empty((N, 6))
        for col in (0, 1):
            v = rng.normal(0.5 * L, 0.25 * L, N)
            bad = (v <= 0) | (v >= L)
            while bad.any():
                v[bad] = rng.normal(0.5 * L, 0.25 * L, int(bad.sum()))
                bad = (v <= 0) | (v >= L)
            a[:, col] = v
        a[:, 2:5] = rng.normal(0.0, math.sqrt(t * picgb.CHARGE / m), (N, 3))
        a[:, 5] = 1.0
        out.append(a)
    return p, out[0], out[1]


@pytest.fixture(scope="module", params=sorted(SPECIES))
def full_runs(request):
    p, e, i = _workload(request.param)
    res = {}
    for mode in ("pipelined", "pipelined again", "in order"):
        with picgb.Run(p) as r:
            r.load_particles(0, e)
            r.load_particles(1, i)
            r.initial_boundary()
            c0 = r.counters()
            if mode == "in order":
                r.set_profiling(True)
            r.step(STEPS)
            res[mode] = (r.get_particles(0), r.get_particles(1), r.get_grid("phi"), r.get_grid("ex"), c0, r.counters())
    return request.param, p, res


def test_full_size_runs_are_deterministic_and_pipelining_changes_nothing(full_runs):
    _, _, res = full_runs
    ref = res["in order"]
    for mode in ("pipelined", "pipelined again"):
        got = res[mode]
        for k in range(4):
            assert np.array_equal(ref[k], got[k], equal_nan=True), (mode, k)
        assert ref[5] == got[5], mode


def test_full_size_populations_balance_with_the_counters(full_runs):
    species, _, res = full_runs
    _, _, _, _, c0, c1 = res["pipelined"]
    d = {k: c1[k] - c0[k] for k in c1}
    assert c1["step"] - c0["step"] == STEPS
    assert d["ionization"] > 0 and d["elastic"] > 0 and d["absorbed_e"] > 0
    assert d["see_events"] > 0
    if species == "argon":
        assert d["charge_exchange"] > 0
    assert c1["n_e"] == (c0["n_e"] + d["injected_e"] + d["see_emitted"] + d["ion_see_emitted"] + d["ionization"]
                         - d["absorbed_e"] - d["see_events"])
    assert c1["n_i"] == c0["n_i"] + d["injected_i"] + d["ionization"] - d["absorbed_i"]


def test_full_size_state_is_finite_and_in_the_domain(full_runs):
    _, p, res = full_runs
    e, i, phi, ex, _, c1 = res["pipelined"]
    assert e.shape[0] == c1["n_e"] and i.shape[0] == c1["n_i"]
    dx = p.xlength / (p.x_no_of_cells - 1)
    for a in (e, i):
        assert np.all(np.isfinite(a))
        assert np.all((a[:, 0] >= -dx) & (a[:, 0] < p.xlength + dx) & (a[:, 1] >= -dx) & (a[:, 1] < p.xlength + dx))
    assert np.all(np.isfinite(phi)) and np.all(np.isfinite(ex))
