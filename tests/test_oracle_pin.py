"""Pin the CPU oracle (oracle/picport.c) to the reference's own outputs.

The golden fixtures were written by the reference's C++ code
(pic::pic_run, particle, fields, Mglin, collision and boundary classes,
built unchanged by oracle/Makefile; see tests/golden/gen_golden.py).  With
the reference's random source (rand()) and removal order (swap with last),
the oracle must reproduce every particle and grid value.  On x86-64 -- the
host the fixtures were written on -- the match is exact; elsewhere the C
library's transcendental functions may differ in the last bit, so a 1e-9
relative tolerance applies there.
"""
import os
import platform

import numpy as np
import pytest

from conftest import golden_cases, load_golden
import orc

EXACT = platform.machine() in ("x86_64", "AMD64")


def _close(a, b, what):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    if EXACT:
        same = (a == b) | (np.isnan(a) & np.isnan(b))
        assert same.all(), f"{what}: {np.count_nonzero(~same)} values differ, max |d| {np.nanmax(np.abs(a - b))}"
    else:
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-30, equal_nan=True, err_msg=what)


@pytest.mark.parametrize("case", golden_cases("run"))
def test_port_matches_reference_run(case):
    g = load_golden(case)
    o = orc.Oracle(g["p"], rng=orc.ORC_RNG_LIBC, order=orc.ORC_ORDER_REF)
    o.load_particles(0, g["e_in"])
    o.load_particles(1, g["i_in"])
    o.initial_boundary()
    o.step(int(g["nsteps"]))
    _close(o.get_particles(0), g["e_out"], f"{case} electrons")
    _close(o.get_particles(1), g["i_out"], f"{case} ions")
    for grid in ("q_e", "q_i", "rho", "phi", "ex", "ey"):
        _close(o.get_grid(grid).ravel(), g[grid], f"{case} {grid}")


@pytest.mark.parametrize("case", golden_cases("fields"))
def test_port_matches_reference_fields(case):
    g = load_golden(case)
    o = orc.Oracle(g["p"], rng=orc.ORC_RNG_LIBC, order=orc.ORC_ORDER_REF)
    o.set_rho(g["rho"])
    o.poisson(0)
    o.efield()
    for grid in ("phi", "ex", "ey"):
        _close(o.get_grid(grid).ravel(), g[grid], f"{case} {grid}")


def test_golden_cases_exercise_the_paths():
    """The fixtures must cover walls, collisions, emission and re-insertion."""
    seen = {}
    for case in golden_cases("run"):
        g = load_golden(case)
        o = orc.Oracle(g["p"], rng=orc.ORC_RNG_LIBC, order=orc.ORC_ORDER_REF)
        o.load_particles(0, g["e_in"])
        o.load_particles(1, g["i_in"])
        o.initial_boundary()
        o.step(int(g["nsteps"]))
        for k, v in o.counters().items():
            seen[k] = seen.get(k, 0) + v
    for k in ("absorbed_e", "absorbed_i", "plopped", "reflected", "backscattered", "see_events",
              "ion_see_emitted", "elastic", "ionization", "charge_exchange", "injected_e", "reductions_e",
              "reductions_i"):
        assert seen[k] > 0, f"no golden case exercises {k}"


def test_philox_known_answers():
    """Philox4x32-10 vectors published with the Random123 library."""
    import ctypes as C
    lib = orc.load()
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
        ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
        ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
         [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
    ]
    for ctr, key, want in kat:
        c = (C.c_uint32 * 4)(*ctr)
        k = (C.c_uint32 * 2)(*key)
        o = (C.c_uint32 * 4)()
        lib.orc_philox4x32(c, k, o)
        assert list(o) == want


def graph_files_from(get, p, gp):
    """The reference's graph files (graphs.cpp:1167-1370) assembled from
    averaged graphs; get(which, species) returns one graph."""
    nx, ny = p.x_no_of_cells, p.y_no_of_cells
    yp, xp = ny // 2, nx // 2
    rho, phi, ex, ey = (get(w, 0) for w in ("rho", "phi", "ex", "ey"))
    i = np.arange(nx, dtype=np.float64)
    files = {
        "rho_phi_EgridX": np.column_stack([i, rho[yp, :], phi[yp, :], ex[yp, :]]),
        "rho_phi_EgridY": np.column_stack([i, rho[:nx, xp], phi[:nx, xp], ey[:nx, xp]]),
        "rho2d": rho, "phi2d": phi, "egrid2dX": ex, "egrid2dY": ey,
    }
    half = (gp.no_bins - 1) // 2
    vbin = (np.arange(gp.no_bins) - half) / float(gp.divide_bins_by)
    for s, t in ((0, "e"), (1, "i1")):
        files[f"density2d_{t}"] = get("density", s)
        files[f"av_velocity_{t}"] = np.column_stack([i, get("vx", s)[:nx], get("vy", s)[:nx]])
        for stem, w in (("first_v_distX", "dist_x1"), ("first_v_distY", "dist_y1"),
                        ("second_v_distX", "dist_x2"), ("second_v_distY", "dist_y2")):
            files[f"{stem}_{t}"] = np.column_stack([vbin, get(w, s)])
    return files


def test_port_graphs_match_reference_files():
    """The oracle's graph sums over a window of steps reproduce the files the
    reference's graphs class wrote (printed with %e, so to 6 digits),
    including the histograms taken from the location's own cell only."""
    import picgb
    g = load_golden("graphs33")
    p = g["p"]
    start, end = (int(v) for v in g["graph_window"])
    gp = picgb.graphs_params(p, start, end)
    o = orc.Oracle(p, rng=orc.ORC_RNG_LIBC, order=orc.ORC_ORDER_REF)
    o.graphs_enable(gp)
    o.load_particles(0, g["e_in"])
    o.load_particles(1, g["i_in"])
    o.initial_boundary()
    o.step(int(g["nsteps"]))
    mine = graph_files_from(o.graphs_get, p, gp)
    counted = 0
    for stem, a in mine.items():
        ref = g["graph_" + stem]
        assert a.shape == ref.shape, (stem, a.shape, ref.shape)
        np.testing.assert_allclose(a, ref, rtol=1e-6, atol=1e-300, err_msg=stem)
        if "dist" in stem:
            counted += a[:, 1].sum()
    assert counted > 0, "the window's histograms are empty"
    m = o.graphs_get("maxima")
    assert m[0] == np.max(mine["phi2d"]) and m[3] == np.max(mine["density2d_e"])



def test_port_cross_sections_match_reference():
    """The oracle's six cross-section fits equal the reference's own
    functions (e_collisions.cpp:205-308, ion_collisions.cpp:170-199) on the
    fixture's 10^4 energies and around every branch edge."""
    import picgb
    with np.load(os.path.join(os.path.dirname(__file__), "golden", "sigma_fits.npz")) as z:
        e, sig, cols = z["energies"], z["sigma"], [str(c) for c in z["columns"]]
    for k, name in enumerate(cols):
        _close(orc.sigma(picgb.XS[name], e), sig[:, k], f"sigma {name}")


@pytest.mark.parametrize("n", [65, 129])
def test_converged_poisson_is_the_exact_discrete_solution(n):
    """The oracle's converged solve (FP64 defect correction around its full
    multigrid, 30 passes), the reference that DST_DC and FP32_DC are tested
    against, equals the exact solution of the 5-point system computed a
    different way: FP64 type-I sine transforms (scipy), whose eigenvalues
    are -(s_k + s_l)/h^2, s_k = 4 sin^2(pi k / 2N).  Walls at 0 V, a smooth
    charge plus white noise; max difference within 1e-12 of max |phi|."""
    sf = pytest.importorskip("scipy.fft")
    import picgb
    p = picgb.make_params(X_NO_OF_CELLS=n, POISSON="DST_DC", PHI_LEFT=0.0, PHI_RIGHT=0.0, PHI_TOP=0.0,
                          PHI_BOTTOM=0.0, PHI_PERIOD=0.0)
    rng = np.random.default_rng(n + 5)
    s = np.linspace(0, 1, n)
    X, Y = np.meshgrid(s, s)
    rho = 1e-6 * np.sin(3 * X) * np.cos(2 * Y) + 1e-7 * rng.standard_normal((n, n))
    o = orc.Oracle(p)
    o.set_rho(rho)
    o.poisson_converged(0, 30)
    phi = o.get_grid("phi")
    N = n - 1
    h = p.xlength / N
    f = -rho[1:-1, 1:-1] / picgb.EPSILON
    sk = 4 * np.sin(np.pi * np.arange(1, N) / (2 * N)) ** 2
    lam = -(sk[:, None] + sk[None, :]) / h**2
    u = sf.idst(sf.idst(sf.dst(sf.dst(f, type=1, axis=0), type=1, axis=1) / lam, type=1, axis=0), type=1, axis=1)
    err = np.max(np.abs(phi[1:-1, 1:-1] - u)) / np.max(np.abs(u))
    assert np.max(np.abs(phi[0])) == 0.0 and np.max(np.abs(phi[:, 0])) == 0.0
    assert err <= 1e-12, err
