"""The library's FP32 cross-section fits against the reference's FP64 ones.

tests/golden/sigma_fits.npz holds the reference's own six energy-dependent
fits (e_collisions.cpp:205-308, ion_collisions.cpp:170-199), tabulated by
the reference's code compiled unchanged, on 10^4 log-spaced energies from
1e-5 to 1e5 eV and on points either side of every branch edge.  The device
evaluates the same formulas in FP32 (pgb_cross_sections), from the energy
converted to FP32 as the collision kernels hold it.

Tolerances, per fit with peak P = max |sigma| over the table:
  |device - reference| <= 1e-5 |reference| + 1e-6 P
    1e-5: FP32 rounding of the energy (6e-8) times the fits' logarithmic
          slopes, and the FP32 power and logarithm (a few 1e-6 at the
          largest exponents of the power-law tails);
    1e-6 P: FP32 cancellation where a fit passes through zero (the Ar
          low-energy polynomial, the H ionization fit at its threshold) and
          values below FP32's range (the H charge-exchange tail, 1e-100).
  Energies within 1e-6 of a branch edge are left out of that bound: FP32
  rounding of the energy or of the edge constant can select the other branch
  there, and at the edges where the reference leaves sigma uninitialised
  the device returns 0.  They are counted, and each must still take the
  value of one of the two branches or 0.
"""
import os

import numpy as np
import pytest

import picgb

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "sigma_fits.npz")
EDGES = {"ar_elastic": (0.35, 15.0), "ar_ionize": (15.755, 100.0), "h_elastic": (0.01, 20.0),
         "h_ionize": (13.6,), "ar_cx": (4.0,), "h_cx": (1.0e-4 * 1000.0 * 1.66054e-27,)}


@pytest.fixture(scope="module")
def table(lib):
    with np.load(GOLDEN) as z:
        return z["energies"], z["sigma"], [str(c) for c in z["columns"]]


@pytest.mark.parametrize("name", list(EDGES))
def test_fp32_fit_matches_reference(table, name):
    e, sig, cols = table
    ref = sig[:, cols.index(name)]
    dev = picgb.cross_sections(name, e)
    near = np.zeros(e.size, dtype=bool)
    for b in EDGES[name]:
        near |= np.abs(e / b - 1.0) < 1e-6
    peak = np.max(np.abs(ref))
    bound = 1e-5 * np.abs(ref) + 1e-6 * peak
    err = np.abs(dev - ref)
    bad = (~near) & ~(err <= bound)
    print(name, "points", e.size, "near edges", int(near.sum()), "max err/bound", float(np.max(err[~near] / bound[~near])))
    assert not bad.any(), f"{name}: {int(bad.sum())} energies beyond the bound, e.g. e={e[bad][:3]} " \
                          f"dev={dev[bad][:3]} ref={ref[bad][:3]}"
    # near an edge: the value of one branch (its neighbour's) or 0
    for k in np.nonzero(near)[0]:
        lo, hi = ref[max(k - 1, 0)], ref[min(k + 1, e.size - 1)]
        ok = dev[k] == 0.0 or any(abs(dev[k] - c) <= 1e-4 * abs(c) + 1e-6 * peak for c in (ref[k], lo, hi))
        assert ok, f"{name} at the edge e={e[k]}: device {dev[k]}, reference {ref[k]} (neighbours {lo}, {hi})"


def test_cross_sections_rejects_a_bad_selector(lib):
    with pytest.raises(picgb.PicError):
        picgb.cross_sections(9, np.ones(3))
