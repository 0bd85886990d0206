"""CPU checks of the viewer-plot rules, on the oracle's restatement of
pgb_render (the GPU tests compare the two)."""
import numpy as np

from conftest import load_golden
import orc
import picgb

LIME, PINK = (142, 255, 29), (255, 29, 142)


def _colours(img):
    return set(map(tuple, img.reshape(-1, 3).tolist()))


def _oracle_with_particles(case="core65"):
    g = load_golden(case)
    o = orc.Oracle(g["p"], rng=orc.ORC_RNG_PHILOX, order=orc.ORC_ORDER_STABLE)
    o.load_particles(0, g["e_in"])
    o.load_particles(1, g["i_in"])
    return o, g


def test_particle_plots_use_the_viewer_colours():
    o, _ = _oracle_with_particles()
    assert _colours(o.render("particle_xy", 128, 128, 0)) == {(0, 0, 0), LIME, PINK}
    assert _colours(o.render("electron_vx_vy", 128, 128, 0)) == {(0, 0, 0), LIME}
    assert _colours(o.render("ion_vx_vy", 128, 128, 0)) == {(0, 0, 0), PINK}


def test_sample_is_deterministic_and_sized():
    """A hashed sample of max_points per species: the same seed gives the same
    image, another seed another sample of about the same size."""
    o, g = _oracle_with_particles()
    a = o.render("electron_vx_vy", 512, 512, 300, seed=1)
    assert np.array_equal(a, o.render("electron_vx_vy", 512, 512, 300, seed=1))
    b = o.render("electron_vx_vy", 512, 512, 300, seed=2)
    assert not np.array_equal(a, b)
    full = np.count_nonzero(np.any(o.render("electron_vx_vy", 512, 512, 0) != 0, axis=2))
    part = np.count_nonzero(np.any(a != 0, axis=2))
    frac = 300 / len(g["e_in"])
    assert 0.5 * frac * full < part < 1.6 * frac * full


def test_field_quads_are_inset_and_density_skips_the_outer_ring():
    """One quad per cell with a gap of a fifth of a cell between quads; the
    density plots start one cell in (gridStart 1)."""
    o, _ = _oracle_with_particles()
    o.deposit(0)
    o.deposit(1)
    o.grid_rho()
    o.poisson(0)
    o.efield()
    n = o.params.x_no_of_cells
    w = 40 * (n - 1)   # 40 pixels per cell
    phi = o.render("phi", w, w)
    covered = np.any(phi != 0, axis=2)
    assert abs(covered.mean() - 0.8 * 0.8) < 0.01
    dens = o.render("e_density", w, w)
    assert not np.any(dens[:, :40]) and not np.any(dens[-40:, :])
    assert np.any(dens[40:-40, 40:-40])
