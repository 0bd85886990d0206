"""The workloads bench.py measures, checked on the CPU (no GPU needed).

The headline is quoted on the 513^2-node, 16Mi-per-species hydrogen
workload in the DST_DC Poisson mode with two passes; the argon
configurations use five FP32_DC passes or two DST_DC passes; the
macro-particle size gives the design density 1e15 m^-3 (parameters.h:71)
for the particle count asked for."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import bench  # noqa: E402
import picgb  # noqa: E402


def _density(p, n):
    """particles per m^2 times the macro-particle size, over the box area"""
    size = -p.qce / picgb.CHARGE
    return n * size / (p.xlength * p.ylength)


def test_headline_workload_is_the_sine_transform_mode_with_two_passes():
    p = bench.workload_params(picgb)
    assert p.x_no_of_cells == p.y_no_of_cells == bench.GRID_NODES == 513
    assert p.poisson_mode == picgb.PGB_POISSON_DST_DC and p.dc_max_iters == 2
    assert np.isclose(_density(p, bench.N_PER_SPECIES), 1.0e15, rtol=1e-12)
    assert p.have_collisions and p.species == picgb.PGB_HYDROGEN


def test_pass_counts_follow_the_mode():
    for mode, passes in (("FP32_DC", 4), ("DST_DC", 2), ("FMG_REF", 1), ("FMG32", 1)):
        p = bench.workload_params(picgb, n_per_species=1 << 20, poisson=mode)
        assert p.poisson_mode == picgb.POISSON_MODES[mode]
        assert p.dc_max_iters == passes, mode
    for mode, passes in (("FP32_DC", 5), ("DST_DC", 2)):
        p = bench.argon_params(picgb, 257, 4 * 1024 * 1024, poisson=mode)
        assert p.dc_max_iters == passes, mode
        assert p.species == picgb.PGB_ARGON
        assert np.isclose(_density(p, 4 * 1024 * 1024), 1.0e15, rtol=1e-12)


def test_every_mode_has_a_description():
    for mode in picgb.POISSON_MODES:
        assert mode in bench.POISSON_DESC
