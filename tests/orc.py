"""ctypes wrapper of the oracle (oracle/picport.c, built as liborcport.so).

Test infrastructure: imported by tests, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py only.  The product never loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "vectorized-particle-in-cell-code-with-graphics_gb300"))
import picgb  # noqa: E402

ORC_RNG_LIBC, ORC_RNG_PHILOX = 0, 1
ORC_ORDER_REF, ORC_ORDER_STABLE = 0, 1
LIB_PATH = os.path.join(REPO, "oracle", "_build", "liborcport.so")
REF_DIR = os.path.join(REPO, "oracle", "_ref")

_LIB = None


def build_port():
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "port"], check=True)


def load():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        build_port()
    lib = C.CDLL(LIB_PATH)
    R, i64, dp = C.c_void_p, C.c_int64, C.POINTER(C.c_double)
    sig = {
        "orc_create": (R, [C.POINTER(picgb.PgbParams), C.c_int, C.c_int]),
        "orc_destroy": (None, [R]),
        "orc_load_species": (C.c_int, [R, C.c_int, dp, i64]),
        "orc_count": (i64, [R, C.c_int]),
        "orc_dump_species": (i64, [R, C.c_int, dp, C.POINTER(C.c_uint32), i64]),
        "orc_set_time_step": (None, [R, i64]),
        "orc_set_threads": (None, [R, C.c_int]),
        "orc_initial_boundary": (None, [R]),
        "orc_step": (None, [R, C.c_int]),
        "orc_collide_electrons": (None, [R]),
        "orc_inject": (None, [R]),
        "orc_gather_push": (None, [R, C.c_int]),
        "orc_collide_ions": (None, [R]),
        "orc_boundary": (None, [R, C.c_int]),
        "orc_contain_growth": (None, [R, C.c_int]),
        "orc_deposit": (None, [R, C.c_int]),
        "orc_grid_rho": (None, [R]),
        "orc_poisson": (None, [R, i64]),
        "orc_efield": (None, [R]),
        "orc_get_grid": (C.c_int, [R, C.c_int, dp, i64]),
        "orc_set_rho": (C.c_int, [R, dp, i64]),
        "orc_get_counters": (None, [R, C.POINTER(picgb.PgbCounters)]),
        "orc_get_neutral_table": (C.c_int, [R, C.c_int, dp, i64]),
        "orc_poisson_residual": (None, [R, dp, dp]),
        "orc_poisson_converged": (None, [R, i64, C.c_int]),
        "orc_graphs_enable": (C.c_int, [R, C.POINTER(picgb.PgbGraphsParams)]),
        "orc_graphs_get": (C.c_int, [R, C.c_int, C.c_int, dp, i64]),
        "orc_render": (C.c_int, [R, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint32, C.POINTER(C.c_uint8), i64]),
        "orc_sigma": (C.c_double, [C.c_int, C.c_double]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def sigma(which, energies):
    """The oracle's FP64 form of one cross-section fit (picgb.PGB_XS_*)."""
    lib = load()
    return np.array([lib.orc_sigma(which, float(e)) for e in energies])


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """The FP64 CPU restatement, with the same method names as picgb.Run."""

    def __init__(self, params, rng=ORC_RNG_PHILOX, order=ORC_ORDER_STABLE, threads=1):
        self.lib = load()
        self.params = params
        self.h = self.lib.orc_create(C.byref(params), rng, order)
        if not self.h:
            raise ValueError("orc_create rejected the parameters")
        if threads != 1:
            self.lib.orc_set_threads(self.h, threads)

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_particles(self, species, aos6):
        a = np.ascontiguousarray(aos6, dtype=np.float64).reshape(-1, 6)
        assert self.lib.orc_load_species(self.h, species, _dp(a), a.shape[0]) == 0

    def particle_size(self, species):
        return int(self.lib.orc_count(self.h, species))

    def get_particles(self, species, with_ids=False):
        n = self.particle_size(species)
        out = np.empty((max(n, 1), 6))
        ids = np.empty(max(n, 1), dtype=np.uint32)
        self.lib.orc_dump_species(self.h, species, _dp(out), ids.ctypes.data_as(C.POINTER(C.c_uint32)), n)
        if with_ids:
            return out[:n].copy(), ids[:n].copy()
        return out[:n].copy()

    def set_time_step(self, t):
        self.lib.orc_set_time_step(self.h, t)

    def initial_boundary(self):
        self.lib.orc_initial_boundary(self.h)

    def step(self, n=1):
        self.lib.orc_step(self.h, n)

    def collide_electrons(self):
        self.lib.orc_collide_electrons(self.h)

    def inject(self):
        self.lib.orc_inject(self.h)

    def gather_push(self, species):
        self.lib.orc_gather_push(self.h, species)

    def collide_ions(self):
        self.lib.orc_collide_ions(self.h)

    def boundary(self, which):
        self.lib.orc_boundary(self.h, which)

    def contain_growth(self, species):
        self.lib.orc_contain_growth(self.h, species)

    def deposit(self, species):
        self.lib.orc_deposit(self.h, species)

    def grid_rho(self):
        self.lib.orc_grid_rho(self.h)

    def poisson(self, t):
        self.lib.orc_poisson(self.h, t)

    def poisson_converged(self, t, iters=30):
        self.lib.orc_poisson_converged(self.h, t, iters)

    def poisson_residual(self):
        a, b = C.c_double(), C.c_double()
        self.lib.orc_poisson_residual(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def efield(self):
        self.lib.orc_efield(self.h)

    def get_grid(self, which):
        shape = picgb.grid_shape(self.params, which)
        out = np.empty(shape)
        assert self.lib.orc_get_grid(self.h, picgb.GRID[which], _dp(out), out.size) == 0
        return out

    def set_rho(self, rho):
        a = np.ascontiguousarray(rho, dtype=np.float64)
        assert self.lib.orc_set_rho(self.h, _dp(a), a.size) == 0

    def counters(self):
        c = picgb.PgbCounters()
        self.lib.orc_get_counters(self.h, C.byref(c))
        return c.as_dict()

    def graphs_enable(self, gp):
        self._gp = gp
        assert self.lib.orc_graphs_enable(self.h, C.byref(gp)) == 0

    def graphs_get(self, which, species=0):
        p = self.params
        out = np.empty(picgb.graph_size(which, p, self._gp))
        assert self.lib.orc_graphs_get(self.h, picgb.GRAPH[which], species, _dp(out), out.size) == 0
        return out.reshape(p.y_no_of_cells, p.x_no_of_cells) if picgb.GRAPH[which] <= 4 else out

    def render(self, plot, width=512, height=512, max_points=picgb.NUM_PARTICLES_TO_PLOT, seed=0):
        img = np.empty((height, width, 3), dtype=np.uint8)
        assert self.lib.orc_render(self.h, picgb.PLOT[plot], width, height, max_points, seed,
                                   img.ctypes.data_as(C.POINTER(C.c_uint8)), img.size) == 0
        return img

    def neutral_table(self, which):
        n = self.params.init_no_neutrals
        out = np.empty(3 * n)
        assert self.lib.orc_get_neutral_table(self.h, which, _dp(out), out.size) == 0
        return out.reshape(3, n)
