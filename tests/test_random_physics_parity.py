"""Random physics against the FP64 oracle at 65^2 nodes, 50k particles per
species.

The presets of the collision and emission fixtures (tests/golden/
gen_golden.py: see33, arcoll33, arsee33, hsee33), widened to 65^2 nodes and 50k particles per species with
the macro-particle size set for the design density 1e15 m^-3:
  see     secondary emission, reflection, backscatter, ion-impact emission
  arcoll  e-Ar elastic and ionization, Ar+-Ar charge exchange at 1 Torr,
          absorbing walls (Te 10 eV: scattering and exchange dominate)
  arsee   emission with e-Ar elastic and ionization, Ar+-Ar charge exchange,
          10 injected particles per species per step
  hsee    e-H collisions, H+-H charge exchange, electron emission, injection
The device and the oracle (library mode: the same Philox draws, the same
stable order) step the same state for five steps; tests/fullsize.py
matches the particles by id and counts the ties (decisions within FP32
rounding of their threshold, and the particles they shift).

Bounds, each derived from what a tie can change:
  ties ............ at most 1e-5 of the particle-steps plus the particles
                    created in the run (a particle created after a tie takes
                    an id one apart, and a secondary's draws follow its id)
  event counts .... |device - oracle| <= 3 x ties: one tie moves a counter by
                    at most one event, or by the two absorbed electrons of an
                    ionization, or by the secondaries of one emission (at
                    most three at these yields)
  fields .......... q, rho, phi, E within 1e-5 of the tie-corrected oracle
                    away from ties (more than 6 cells from a tie particle);
                    phi and E within 1e-4 everywhere
  particles ....... positions 2e-4 cell, velocities 1e-3 thermal speed
                    (non-tie particles), mean energies 1e-4 (the secondaries
                    of a tie are drawn apart)
"""
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import fullsize  # noqa: E402
import gen_golden  # noqa: E402
import picgb  # noqa: E402

pytestmark = pytest.mark.gpu
N = 50_000
STEPS = 5


@pytest.fixture(scope="module", autouse=True)
def _lib(lib):
    return lib


def _case(name):
    _, kw, recipe, _ = gen_golden.CASES[name]
    kw = dict(kw, X_NO_OF_CELLS=65, RAND_SEED=7)
    kw.setdefault("STEADYSTATE", "NO")
    L = picgb.make_params(**kw).xlength
    size = 1.0e15 * L * L / N
    p = picgb.make_params(E_MACROPARTICLE_SIZE=size, ION_MACROPARTICLE_SIZE=size, **kw)
    e, i = gen_golden.make_state(p, N, recipe["te"], recipe["ti"], recipe["seed"] + 100, recipe.get("outside", 0.0))
    return p, e, i


@pytest.mark.parametrize("name", ["see33", "arcoll33", "arsee33", "hsee33"])
def test_random_physics_matches_oracle_at_50k(name):
    p, e, i = _case(name)
    d = fullsize.compare(p, e, i, STEPS)
    print(name, {k: d[k] for k in ("ties", "counts", "grids_away_from_ties", "grids_tie_corrected", "nodes_near_ties")})
    print(name, d["particles"], d["oracle_counts"])
    oc = d["oracle_counts"]
    created = oc["see_emitted"] + oc["ion_see_emitted"] + oc["injected_e"] + oc["injected_i"]
    steps = sum(x["n_oracle"] for x in d["particles"].values()) * STEPS
    assert d["ties"] <= created + 1e-5 * steps, f"{name}: {d['ties']} ties"
    events = sum(oc[k] for k in ("elastic", "ionization", "charge_exchange", "see_events", "reflected",
                                 "backscattered", "absorbed_e"))
    assert events > 100, f"{name}: the case should exercise its random physics ({events} events)"
    for k, dv in d["counts"].items():
        assert abs(dv) <= 3 * d["ties"], f"{name} {k}: device - oracle = {dv} with {d['ties']} ties"
    for g, v in d["grids_away_from_ties"].items():
        assert v <= 1e-5, f"{name} {g}: {v:.3g} away from ties"
    for g in ("phi", "ex", "ey"):
        assert d["grids_tie_corrected"][g] <= 1e-4, f"{name} {g}: {d['grids_tie_corrected'][g]:.3g}"
    for sp, x in d["particles"].items():
        assert x["pos_cells"] <= 2e-4, f"{name} {sp} positions {x['pos_cells']:.3g}"
        assert x["vel_vt"] <= 1e-3, f"{name} {sp} velocities {x['vel_vt']:.3g}"
        assert x["mean_energy_rel"] <= 1e-4, f"{name} {sp} mean energy {x['mean_energy_rel']:.3g}"
