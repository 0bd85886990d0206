"""Random collision physics against the reference's own random source.

The device draws from Philox streams; the reference draws from rand() in
loop order.  The oracle's LIBC mode is the reference's algorithm with
rand() (bit-pinned to the reference's binaries), so the two are compared
statistically on 500k particles per species over two steps:
  - elastic e-Ar scattering (e_collisions.cpp:480-597, collisions.cpp:107-171):
    the number of scattered electrons, and the distribution of the
    scattering angle between the velocities before and after;
  - Ar+-Ar charge exchange (ion_collisions.cpp:255-308): the number of
    exchanges, and the speed distribution of the exchanged ions, drawn from
    the neutral table (vz >= 0 there, collisions.cpp:66-89).
All particles have weight 0, so E = 0 and only collisions change a
velocity; ionization is switched off so that the rows of both runs stay
matched.  Counts must agree within 5 sigma; the distributions must pass a
two-sample chi-square test at p > 1e-4.
"""
import math

import numpy as np
import pytest

import orc
import picgb

pytestmark = pytest.mark.gpu
stats = pytest.importorskip("scipy.stats")

N = 500_000
STEPS = 2


def _params():
    return picgb.make_params(X_NO_OF_CELLS=65, STEADYSTATE="NO", GAS_PRESSURE_TORR=1.0, TEMPERATURE=2.0,
                             HAVE_COLLISIONS=True, SIGMA="ENERGY_DEPENDENT", SIGMA_ELASTIC="ENERGY_DEPENDENT",
                             SIGMA_IONIZATION="CONSTANT", IONIZATION_SIGMA_VALUE=0.0)


def _state(p, seed):
    rng = np.random.default_rng(seed)
    L = p.xlength
    out = []
    for m, t in ((picgb.ELECTRON_MASS, 5.0), (p.ion_mass, 0.5)):
        x = rng.uniform(0.2 * L, 0.8 * L, (N, 2))
        v = rng.normal(0.0, math.sqrt(t * picgb.CHARGE / m), (N, 3))
        out.append(np.column_stack([x, v, np.zeros(N)]))
    return out


def _chi2_two_sample(a, b, edges):
    ha, _ = np.histogram(a, edges)
    hb, _ = np.histogram(b, edges)
    keep = (ha + hb) > 0
    ha, hb = ha[keep].astype(float), hb[keep].astype(float)
    ka, kb = math.sqrt(hb.sum() / ha.sum()), math.sqrt(ha.sum() / hb.sum())
    chi2 = float(np.sum((ka * ha - kb * hb) ** 2 / (ha + hb)))
    return chi2, float(stats.chi2.sf(chi2, len(ha) - 1))


def _changed(before, after):
    """rows whose velocity changed (the device stores FP32 velocities)"""
    v0 = before[:, 2:5].astype(np.float32).astype(np.float64)
    return np.linalg.norm(after[:, 2:5] - v0, axis=1) > 1e-4 * np.linalg.norm(v0, axis=1)


def test_collisions_match_the_reference_random_source_statistically():
    p = _params()
    e, i = _state(p, 11)
    o = orc.Oracle(p, rng=orc.ORC_RNG_LIBC, order=orc.ORC_ORDER_STABLE)
    with picgb.Run(p) as r:
        for x in (o, r):
            x.load_particles(0, e)
            x.load_particles(1, i)
            x.step(STEPS)
        cg, co = r.counters(), o.counters()
        res = {"gpu": (r.get_particles(0), r.get_particles(1)), "ref": (o.get_particles(0), o.get_particles(1))}
    for k in ("elastic", "charge_exchange"):
        assert cg[k] > 1000 and co[k] > 1000, (k, cg[k], co[k])
        assert abs(cg[k] - co[k]) <= 5 * math.sqrt(cg[k] + co[k]), (k, cg[k], co[k])
    assert cg["ionization"] == co["ionization"] == 0
    cos = {}
    speed = {}
    for side, (pe, pi) in res.items():
        assert pe.shape == e.shape and pi.shape == i.shape, side
        hit = _changed(e, pe)
        v0, v1 = e[hit, 2:5], pe[hit, 2:5]
        cos[side] = np.sum(v0 * v1, axis=1) / (np.linalg.norm(v0, axis=1) * np.linalg.norm(v1, axis=1))
        cx = _changed(i, pi)
        speed[side] = np.linalg.norm(pi[cx, 2:5], axis=1)
        assert np.all(pi[cx, 4] >= 0.0), side   # neutral-table vz >= 0
    chi2, pv = _chi2_two_sample(cos["gpu"], cos["ref"], np.linspace(-1.0, 1.0, 21))
    assert pv > 1e-4, ("scattering angle", chi2, pv)
    edges = np.quantile(np.concatenate([speed["gpu"], speed["ref"]]), np.linspace(0, 1, 21))
    edges[-1] *= 1.0 + 1e-12
    chi2, pv = _chi2_two_sample(speed["gpu"], speed["ref"], edges)
    assert pv > 1e-4, ("exchanged-ion speed", chi2, pv)


def test_energy_distributions_after_ten_steps_match_the_reference_random_source():
    """Ten steps of elastic e-Ar scattering and Ar+-Ar charge exchange: the
    electron and ion energy distributions of the device (Philox) and of the
    reference's algorithm with its own rand() pass a two-sample chi-square
    test at p > 1e-4 over 20 equal-count bins, and the mean energies agree
    within 5 standard errors.  Charge exchange replaces an ion's energy by a
    neutral's, so after ten steps a large share of the ions carries the
    neutral temperature; for the electrons the test checks that scattering
    leaves the same (nearly elastic) distribution on both sides."""
    steps = 10
    p = _params()
    e, i = _state(p, 12)
    o = orc.Oracle(p, rng=orc.ORC_RNG_LIBC, order=orc.ORC_ORDER_STABLE)
    with picgb.Run(p) as r:
        for x in (o, r):
            x.load_particles(0, e)
            x.load_particles(1, i)
            x.step(steps)
        out = {"gpu": (r.get_particles(0), r.get_particles(1)), "ref": (o.get_particles(0), o.get_particles(1))}
        cg, co = r.counters(), o.counters()
    assert cg["charge_exchange"] > 5000 and co["charge_exchange"] > 5000
    for s, m in ((0, picgb.ELECTRON_MASS), (1, p.ion_mass)):
        en = {k: 0.5 * m * np.sum(v[s][:, 2:5] ** 2, axis=1) / picgb.CHARGE for k, v in out.items()}
        a, b = en["gpu"], en["ref"]
        edges = np.quantile(np.concatenate([a, b]), np.linspace(0, 1, 21))
        edges[-1] *= 1.0 + 1e-12
        chi2, pv = _chi2_two_sample(a, b, edges)
        assert pv > 1e-4, ("energy distribution", s, chi2, pv)
        se = math.sqrt(a.var() / a.size + b.var() / b.size)
        assert abs(a.mean() - b.mean()) <= 5 * se, ("mean energy", s, a.mean(), b.mean(), se)
