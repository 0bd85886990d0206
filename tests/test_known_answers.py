"""Known answers that need no oracle: cases whose result follows from the
reference's formulas in closed form.

- CIC deposit of single particles, with the edge and corner doubling of
  particle::collect_charge (pic.cl:22-52, particle.cpp:829-845).
- E = 0 (weight-0 particles, walls at 0 V): free streaming and the exact
  rotation about B of move_particles (pic.cl:95-149).
- The gather: weight-0 test electrons in the field of weighted ions change
  velocity by dt*q/m times the CIC average of the library's own E grid
  (pic.cl:56-92, stride-nx layout).
- Poisson (fields::grid_potential, Mglin) on a manufactured discrete
  solution, and with every wall at the same potential and no charge.
"""
import math

import numpy as np
import pytest

import picgb

pytestmark = pytest.mark.gpu

EPS0 = 8.854e-12   # constants.h EPSILON


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_single_particle_deposit_cic_weights():
    """One electron in the interior spreads qc/(DX*DY) over its four nodes
    with weights (1-wj)(1-wk), wj(1-wk), wk(1-wj), wj*wk; one next to the
    origin has its edge nodes doubled and the corner node x8."""
    p = picgb.make_params(X_NO_OF_CELLS=33, STEADYSTATE="NO")
    n, dx = p.x_no_of_cells, p.xlength / (p.x_no_of_cells - 1)
    scale = p.qce / (dx * dx)
    cases = [((10, 0.25), (7, 0.625), {}), ((0, 0.375), (0, 0.75), {(0, 0): 8.0, (0, 1): 2.0, (1, 0): 2.0})]
    for (jp, wj), (kp, wk), factor in cases:
        e = np.array([[(jp + wj) * dx, (kp + wk) * dx, 0.0, 0.0, 0.0, 1.0]])
        i = np.array([[0.5 * p.xlength, 0.5 * p.xlength, 0.0, 0.0, 0.0, 1.0]])
        with picgb.Run(p) as r:
            r.load_particles(0, e)
            r.load_particles(1, i)
            r.deposit(0)
            q = r.get_grid("q_e").reshape(n, n)
        want = np.zeros((n, n))
        for (dk, dj), a in (((0, 0), (1 - wj) * (1 - wk)), ((0, 1), wj * (1 - wk)), ((1, 0), wk * (1 - wj)),
                            ((1, 1), wj * wk)):
            want[kp + dk, jp + dj] = scale * a * factor.get((kp + dk, jp + dj), 1.0)
        assert np.allclose(q, want, rtol=1e-12, atol=0.0), (jp, kp, np.argwhere(~np.isclose(q, want)))


def _orbit(v, x, y, p, steps, b):
    """the push of pic.cl:95-149 with E = 0, in FP64"""
    dt, qm = p.dt, p.q_over_me
    ca, sa = math.cos(p.angle), math.sin(p.angle)
    w = dt * qm * b
    co, so = math.cos(w), math.sin(w)
    vx, vy, vz = v[:, 0].copy(), v[:, 1].copy(), v[:, 2].copy()
    for _ in range(steps):
        if b > 0.0:
            vpar = ca * vx + sa * vy
            vperp = -sa * vx + ca * vy
            va = vperp * co + so * vz
            vz = -vperp * so + co * vz
            vx, vy = ca * vpar - sa * va, sa * vpar + ca * va
        x = x + dt * vx
        y = y + dt * vy
    return x, y, np.column_stack([vx, vy, vz])


@pytest.mark.parametrize("b", [0.0, 0.05])
def test_free_streaming_and_gyration_with_zero_field(b):
    """Weight-0 particles and walls at 0 V give E = 0 exactly.  Electrons
    then stream freely (B = 0) or gyrate about B at ANGLE: the parallel
    speed is kept and (vperp, vz) turns by dt*q/m*B per step."""
    p = picgb.make_params(X_NO_OF_CELLS=33, STEADYSTATE="NO", MAGNETIC_FIELD=b, ANGLE_DEG=30.0)
    rng = np.random.default_rng(3)
    n, L = 256, p.xlength
    e = np.column_stack([rng.uniform(0.3 * L, 0.7 * L, (n, 2)), rng.normal(0, p.vte, (n, 3)), np.zeros(n)])
    i = np.column_stack([rng.uniform(0.3 * L, 0.7 * L, (n, 2)), rng.normal(0, p.vti, (n, 3)), np.zeros(n)])
    steps = 12
    with picgb.Run(p) as r:
        r.load_particles(0, e)
        r.load_particles(1, i)
        r.step(steps)
        assert not np.any(r.get_grid("ex")) and not np.any(r.get_grid("ey"))
        got = r.get_particles(0)
    x, y, v = _orbit(e[:, 2:5], e[:, 0], e[:, 1], p, steps, b)
    dx = L / (p.x_no_of_cells - 1)
    assert got.shape[0] == n
    # fixed-point positions round to 2^-23 of a cell per step (33 nodes), the FP32
    # displacement to 6e-8 of itself; velocities to 1e-7 per rotation
    assert np.max(np.abs(got[:, 0] - x)) / dx < 2e-6 and np.max(np.abs(got[:, 1] - y)) / dx < 2e-6
    assert np.max(np.abs(got[:, 2:5] - v)) < 1e-5 * np.max(np.abs(v))
    if b > 0:   # the rotation really happened
        assert np.max(np.abs(v - e[:, 2:5])) > 0.1 * p.vte


def _gather(ex, ey, xs, ys, nx):
    """CIC average of the stride-nx E grids at cell-unit positions (pic.cl:66-88)"""
    jp, kp = xs.astype(int), ys.astype(int)
    wj, wk = xs - jp, ys - kp
    a4, a3, a2, a1 = (1 - wj) * (1 - wk), wj * (1 - wk), wk * (1 - wj), wj * wk
    out = []
    for f in (ex, ey):
        out.append(a4 * f[kp * nx + jp] + a3 * f[kp * nx + jp + 1] + a2 * f[(kp + 1) * nx + jp] +
                   a1 * f[(kp + 1) * nx + jp + 1])
    return out


def test_gather_push_uses_the_cic_average_of_the_field():
    """Weight-0 electrons in the field of a weighted ion cloud: one step
    changes each velocity by dt*q/m*E_p, E_p the CIC average of the E grid
    of the step before, and moves it by dt times the new velocity."""
    p = picgb.make_params(X_NO_OF_CELLS=65, STEADYSTATE="NO", MAGNETIC_FIELD=0.0)
    rng = np.random.default_rng(5)
    L, nx = p.xlength, p.x_no_of_cells
    dx = L / (nx - 1)
    ni, ne = 20000, 2000
    ions = np.column_stack([np.clip(rng.normal(0.5 * L, 0.12 * L, (ni, 2)), 0.05 * L, 0.95 * L),
                            np.zeros((ni, 3)), np.ones(ni)])
    e = np.column_stack([rng.uniform(0.2 * L, 0.8 * L, (ne, 2)), rng.normal(0, p.vte, (ne, 3)), np.zeros(ne)])
    with picgb.Run(p) as r:
        r.load_particles(0, e)
        r.load_particles(1, ions)
        r.step(1)
        ex, ey = r.get_grid("ex"), r.get_grid("ey")
        before = r.get_particles(0)
        r.step(1)
        after = r.get_particles(0)
    assert before.shape == after.shape == (ne, 6)
    # the dumped position is the library's fixed-point position times DX
    xs, ys = before[:, 0] / dx, before[:, 1] / dx
    exp_, eyp = _gather(ex, ey, xs, ys, nx)
    dv = p.dt * p.q_over_me
    want_vx, want_vy = before[:, 2] + dv * exp_, before[:, 3] + dv * eyp
    kick = np.max(np.abs(dv * np.hypot(exp_, eyp)))
    assert kick > 1e-3 * p.vte, "the field is too weak to test the gather"
    tol = 2e-6 * np.max(np.abs(before[:, 2:4])) + 1e-5 * kick
    assert np.max(np.abs(after[:, 2] - want_vx)) < tol and np.max(np.abs(after[:, 3] - want_vy)) < tol
    assert np.max(np.abs(after[:, 0] - (before[:, 0] + p.dt * after[:, 2]))) < 1e-5 * dx


def _laplacian_rho(phi, h):
    """rho with -eps0 * (5-point Laplacian of phi) = rho at interior nodes"""
    lap = np.zeros_like(phi)
    lap[1:-1, 1:-1] = (phi[2:, 1:-1] + phi[:-2, 1:-1] + phi[1:-1, 2:] + phi[1:-1, :-2] - 4 * phi[1:-1, 1:-1]) / h**2
    return -EPS0 * lap


def test_poisson_recovers_a_manufactured_discrete_solution():
    """phi = 10 x(1-x) y(1-y) exp(x+2y) on the unit-scaled domain, walls at
    0 V, and rho its discrete Laplacian.  The defect-corrected solves
    (multigrid and sine transform) return phi to 1e-9.  The reference's single FMG pass (FP64 and FP32)
    leaves its truncation error, 5e-5 at 65^2, and it shrinks by more than
    2.5x from 65^2 to 129^2.  (sin x sin is no test of the multigrid: it is
    an eigenfunction of the discrete Laplacian, which one pass solves
    exactly.)"""
    fmg = {}
    for n in (65, 129):
        s = np.linspace(0.0, 1.0, n)
        X, Y = np.meshgrid(s, s)
        phi = 10.0 * X * (1 - X) * Y * (1 - Y) * np.exp(X + 2 * Y)
        for mode, tol in (("FP32_DC", 1e-9), ("DST_DC", 1e-9), ("FMG_REF", 1e-4), ("FMG32", 1e-4)):
            p = picgb.make_params(X_NO_OF_CELLS=n, POISSON=mode, DC_MAX_ITERS=12)
            h = p.xlength / (n - 1)
            with picgb.Run(p) as r:
                r.set_rho(_laplacian_rho(phi, h))
                r.poisson(0)
                err = _rel(r.get_grid("phi"), phi)
            assert err <= tol, (n, mode, err)
            fmg[(n, mode)] = err
    assert fmg[(129, "FMG_REF")] < fmg[(65, "FMG_REF")] / 2.5, fmg


def test_poisson_with_equal_walls_and_no_charge_is_constant():
    """Every wall at 2 V and no charge: phi = 2 V at every node."""
    p = picgb.make_params(X_NO_OF_CELLS=65, POISSON="FP32_DC", DC_MAX_ITERS=12, PHI_LEFT=2.0, PHI_RIGHT=2.0,
                          PHI_TOP=2.0, PHI_BOTTOM=2.0, PHI_PERIOD=0.0)
    with picgb.Run(p) as r:
        r.set_rho(np.zeros((65, 65)))
        r.poisson(0)
        got = r.get_grid("phi")
    assert np.max(np.abs(got - 2.0)) < 1e-8
