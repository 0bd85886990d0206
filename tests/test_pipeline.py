"""The pipelined step against the same steps run in order.

pgb_step runs the electron collisions of step t+1 on the run's stream while
the field solve of step t is still in flight on a side stream (the
collisions read no field).  Profiling switches that off: every step then
runs collisions, particle phases and field solve one after the other, as
pic_run does (pic.cpp:1069-1161).  Both orders, and a run that steps one
call at a time (the pending field solve is issued at the end of every
call), must end bit for bit in the same state: particles, grids and
counters.  The cases cover argon and hydrogen collisions with wall
secondaries and injection, ion steps every other step (DTI_RATIO 2), the
spatial sort, and a diagnostics window (its sums follow each step's field
solve).
"""
import math

import numpy as np
import pytest

import picgb
from conftest import load_golden

pytestmark = pytest.mark.gpu


def _gaussian(p, n, te, ti, seed):
    """positions ~ N(L/2, (L/4)^2) inside the box, Maxwellian velocities"""
    rng = np.random.default_rng(seed)
    L = p.xlength
    out = []
    for m, t in ((picgb.ELECTRON_MASS, te), (p.ion_mass, ti)):
        x = np.clip(rng.normal(0.5 * L, 0.25 * L, (n, 2)), 0.01 * L, 0.99 * L)
        v = rng.normal(0.0, math.sqrt(t * picgb.CHARGE / m), (n, 3))
        out.append(np.column_stack([x, v, np.ones(n)]))
    return out


_H129 = dict(X_NO_OF_CELLS=129, TEMPERATURE=3.0, ION_MASS_AMU=1.0, THRESHOLD=13.6, SPECIES="HYDROGEN",
             HAVE_COLLISIONS=True, SIGMA="ENERGY_DEPENDENT", SIGMA_ELASTIC="ENERGY_DEPENDENT",
             SIGMA_IONIZATION="ENERGY_DEPENDENT", E_IMPACT_SEE="YES", REFLECTION="YES", BACKSCATTER="YES",
             STEADYSTATE="NO", NUMBER_TO_INJECT=10, SIZE_TO_CHECK=2**31 - 1, SORT_INTERVAL=4, POISSON="FMG32")


def _case(name):
    if name in ("h_sorted_129", "h_sorted_129_dst"):
        kw = dict(_H129)
        if name.endswith("_dst"):
            kw.update(POISSON="DST_DC", DC_MAX_ITERS=2)
        n = 60000
        L = picgb.make_params(**kw).xlength
        p = picgb.make_params(E_MACROPARTICLE_SIZE=1.0e15 * L * L / n, ION_MACROPARTICLE_SIZE=1.0e15 * L * L / n, **kw)
        e, i = _gaussian(p, n, 3.0, 0.026, 7)
        return p, e, i, 13
    if name == "arcoll33_dti2":
        g = load_golden("arcoll33")
        return picgb.make_params(**{**g["kw"], "DTI_RATIO": 2.0}), g["e_in"], g["i_in"], 11
    g = load_golden(name)
    return g["p"], g["e_in"], g["i_in"], int(g["nsteps"]) + 3


def _run(p, e, i, n, mode, window=None):
    with picgb.Run(p) as r:
        r.load_particles(0, e)
        r.load_particles(1, i)
        r.initial_boundary()
        if window:
            r.graphs_enable(picgb.graphs_params(p, *window))
        if mode == "in order":
            r.set_profiling(True)
        if mode == "one call per step":
            for _ in range(n):
                r.step(1)
        else:
            r.step(n)
        out = [r.get_particles(0), r.get_particles(1)] + [r.get_grid(k) for k in ("q_e", "q_i", "phi", "ex", "ey")]
        out.append(r.counters())
        if window:
            out += [r.graphs_get("phi"), r.graphs_get("density", 0), r.graphs_get("vx", 1)]
        return out


@pytest.mark.parametrize("name", ["arcoll33", "arsee33", "hsee33", "arcoll33_dti2", "h_sorted_129", "h_sorted_129_dst"])
def test_pipelined_steps_equal_steps_in_order(name):
    p, e, i, n = _case(name)
    window = (2, n - 2) if name in ("arsee33", "h_sorted_129", "h_sorted_129_dst") else None
    res = {m: _run(p, e, i, n, m, window) for m in ("in order", "pipelined", "one call per step")}
    ref = res["in order"]
    assert ref[7]["n_e"] > 0
    for m in ("pipelined", "one call per step"):
        got = res[m]
        for k, (a, b) in enumerate(zip(ref, got)):
            if isinstance(a, dict):
                assert a == b, (m, name)
            else:
                assert np.array_equal(a, b, equal_nan=True), (m, name, k)


def test_launch_shapes_change_no_result():
    """pgb_set_launch_config changes how the push grid and the collision
    kernels beside the field solve are laid out, not what they compute:
    the same state stepped under three shapes ends bit for bit the same
    (particles, grids, counters)."""
    p, e, i, n = _case("h_sorted_129")
    res = []
    for push, field in ((8, 32), (4, 8), (12, 48)):
        with picgb.Run(p) as r:
            r.load_particles(0, e)
            r.load_particles(1, i)
            r.initial_boundary()
            r.set_launch_config(push, field)
            assert r.launch_config() == {"push_blocks_per_sm": push, "field_sms": field}
            r.step(n)
            res.append([r.get_particles(0), r.get_particles(1)] + [r.get_grid(k) for k in ("q_e", "q_i", "phi")]
                       + [r.counters()])
    for got in res[1:]:
        for k, (a, b) in enumerate(zip(res[0], got)):
            if isinstance(a, dict):
                assert a == b
            else:
                assert np.array_equal(a, b, equal_nan=True), k


def test_autotune_keeps_the_fastest_candidate():
    """pgb_autotune times the 12 candidates and keeps the fastest; the run's
    launch configuration is then that candidate, and a bad shape is refused."""
    p, e, i, _ = _case("h_sorted_129")
    with picgb.Run(p) as r:
        r.load_particles(0, e)
        r.load_particles(1, i)
        r.initial_boundary()
        t = r.autotune(2)
        assert len(t["candidates"]) == 12 and all(c["ms_per_step"] > 0 for c in t["candidates"])
        fastest = min(t["candidates"], key=lambda c: c["ms_per_step"])
        assert (t["push_blocks_per_sm"], t["field_sms"]) == (fastest["push_blocks_per_sm"], fastest["field_sms"])
        assert r.launch_config() == {"push_blocks_per_sm": t["push_blocks_per_sm"], "field_sms": t["field_sms"]}
        with pytest.raises(picgb.PicError):
            r.set_launch_config(0, 8)
