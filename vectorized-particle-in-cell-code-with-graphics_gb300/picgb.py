"""Python host mirror of the reference PIC driver over the libpicgb C ABI.

The reference configures a run with compile-time macros in parameters.h
(parameters.h:41-366) and drives it with pic::pic_run (pic.cpp:1040-1279).
This module offers the same inputs as keyword arguments named after those
macros (`make_params`), derives the dependent quantities with the
reference's formulas, and wraps libpicgb.so (include/picgb.h) with ctypes so
that tests and benchmarks can call the exact C entry points a C++ or FFI
caller would use.  No computation happens here: every physics call goes to
the CUDA library, and a missing library raises instead of falling back.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)

# constants.h:17-26
PI = 3.141592654
CHARGE = 1.602177e-19
ELECTRON_CHARGE2 = 2.566971e-38
ELECTRON_MASS = 9.10939e-31
AMU = 1.66054e-27
EPSILON = 8.854e-12

PGB_ELECTRONS, PGB_IONS = 0, 1
PGB_ARGON, PGB_HYDROGEN = 0, 1
PGB_SIGMA_CONSTANT, PGB_SIGMA_ENERGY_DEPENDENT = 0, 1
GRID = {"q_e": 0, "q_i": 1, "rho": 2, "phi": 3, "ex": 4, "ey": 5}
PGB_POISSON_FMG_REF, PGB_POISSON_FP32_DC, PGB_POISSON_FMG32, PGB_POISSON_DST_DC = 0, 1, 2, 3
POISSON_MODES = {"FMG_REF": 0, "FP32_DC": 1, "FMG32": 2, "DST_DC": 3}
PGB_BOUNDARY_IONS, PGB_BOUNDARY_ELECTRONS = 0, 1


class PgbParams(C.Structure):
    """ctypes image of `pgb_params` (include/picgb.h)."""

    _fields_ = [
        ("x_no_of_cells", C.c_int32), ("y_no_of_cells", C.c_int32),
        ("xlength", C.c_double), ("ylength", C.c_double),
        ("dt", C.c_double), ("dti", C.c_double),
        ("electron_mass", C.c_double), ("ion_mass", C.c_double),
        ("q_over_me", C.c_double), ("q_over_mi", C.c_double),
        ("qce", C.c_double), ("qci", C.c_double),
        ("vte", C.c_double), ("vti", C.c_double), ("vtn", C.c_double),
        ("magnetic_field", C.c_double), ("angle", C.c_double),
        ("phi_left", C.c_double), ("phi_right", C.c_double),
        ("phi_bottom", C.c_double), ("phi_top", C.c_double), ("phi_period", C.c_double),
        ("neutral_density", C.c_double), ("threshold", C.c_double), ("work_function", C.c_double),
        ("have_collisions", C.c_int32), ("species", C.c_int32),
        ("sigma_cx_mode", C.c_int32), ("sigma_elastic_mode", C.c_int32),
        ("sigma_ionization_mode", C.c_int32),
        ("sigma_value", C.c_double), ("elastic_sigma_value", C.c_double),
        ("ionization_sigma_value", C.c_double),
        ("e_impact_see", C.c_int32), ("ion_impact_see", C.c_int32), ("reflection", C.c_int32),
        ("backscatter", C.c_int32), ("steadystate", C.c_int32),
        ("number_to_inject", C.c_int32), ("init_no_neutrals", C.c_int32),
        ("see_e0", C.c_double), ("see_max_yield", C.c_double), ("see_emax0", C.c_double),
        ("no_groups", C.c_int32),
        ("v_limit_e", C.c_double * 3), ("v_limit_i", C.c_double * 3),
        ("group_limit_e", C.c_int32 * 3), ("group_limit_i", C.c_int32 * 3),
        ("new_group_size_e", C.c_int32 * 3), ("new_group_size_i", C.c_int32 * 3),
        ("size_to_check_e", C.c_int64), ("size_to_check_i", C.c_int64),
        ("seed", C.c_uint64), ("poisson_mode", C.c_int32), ("dc_max_iters", C.c_int32),
        ("dc_tolerance", C.c_double), ("sort_interval", C.c_int32),
        ("capacity_e", C.c_int64), ("capacity_i", C.c_int64),
    ]


class PgbCounters(C.Structure):
    """ctypes image of `pgb_counters` (include/picgb.h)."""

    _fields_ = [(name, C.c_int64) for name in (
        "n_e", "n_i", "step", "absorbed_e", "absorbed_i", "plopped", "reflected",
        "backscattered", "see_events", "see_emitted", "ion_see_emitted", "elastic",
        "ionization", "charge_exchange", "injected_e", "injected_i",
        "reductions_e", "reductions_i")]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


class PgbServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64), ("active", C.c_int64),
                ("queued", C.c_int64), ("run_steps", C.c_int64), ("particle_steps", C.c_double),
                ("busy_seconds", C.c_double), ("step_ms_p50", C.c_double), ("step_ms_p99", C.c_double),
                ("ttc_s_p50", C.c_double), ("ttc_s_p99", C.c_double), ("hbm_in_use", C.c_int64),
                ("hbm_budget", C.c_int64), ("admit_seconds", C.c_double), ("retire_seconds", C.c_double),
                ("issue_seconds", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PgbGraphsParams(C.Structure):
    """pgb_graphs_params: window and settings of the averaged diagnostics
    (the graphs class, graphs.cpp; parameters.h:227-302)."""
    _fields_ = [("start_step", C.c_int64), ("end_step", C.c_int64), ("no_graph_steps", C.c_int32),
                ("no_bins", C.c_int32), ("divide_bins_by", C.c_int32), ("spread", C.c_int32),
                ("dist_location_x", C.c_int32), ("dist_location_y", C.c_int32),
                ("dist_location2_x", C.c_int32), ("dist_location2_y", C.c_int32)]


# PGB_GRAPH_*: which averaged graph to read
GRAPH = {"rho": 0, "phi": 1, "ex": 2, "ey": 3, "density": 4, "vx": 5, "vy": 6, "dist_x1": 7, "dist_y1": 8,
         "dist_x2": 9, "dist_y2": 10, "maxima": 11}


def graphs_params(p, start: int, end: int, no_graph_steps: int = None, **kw) -> PgbGraphsParams:
    """parameters.h's graph settings for this grid (NO_BINS, DIVIDE_BINS_BY,
    SPREAD, DIST_LOCATION*; parameters.h:288-302), summing steps
    [start, end) and averaging over no_graph_steps (default end - start).
    Keyword arguments override single fields."""
    g = PgbGraphsParams()
    nx, ny = p.x_no_of_cells, p.y_no_of_cells
    f32 = lambda v: float(np.float32(v))   # the (float) casts of parameters.h
    g.start_step, g.end_step = start, end
    g.no_graph_steps = no_graph_steps if no_graph_steps is not None else max(end - start, 1)
    g.no_bins = 30001
    g.divide_bins_by = (g.no_bins - 1) // 100
    g.spread = int(0.05 * f32(nx))
    g.dist_location_x, g.dist_location_y = int(0.9 * f32(nx)), int(0.5 * f32(ny))
    g.dist_location2_x, g.dist_location2_y = int(0.1 * f32(nx)), int(0.5 * f32(ny))
    for k, v in kw.items():
        setattr(g, k, v)
    return g


# PGB_PLOT_*: the viewer's plot selector (graphics.cpp:68-77)
PLOT = {"particle_xy": 0, "electron_vx_vy": 1, "ion_vx_vy": 2, "phi": 3, "efield_x": 4, "efield_y": 5,
        "e_density": 6, "ion_density": 7}
NUM_PARTICLES_TO_PLOT = 5000   # graphics.h:77


def write_ppm(path: str, img: np.ndarray):
    """an (H, W, 3) uint8 image as binary PPM"""
    h, w, _ = img.shape
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(img, dtype=np.uint8).tobytes())


def graph_size(which: str, p, gp: PgbGraphsParams) -> int:
    """number of values pgb_graphs_get returns for `which`"""
    w = GRAPH[which]
    if w <= 4:
        return p.x_no_of_cells * p.y_no_of_cells
    return {5: p.x_no_of_cells, 6: p.y_no_of_cells, 11: 5}.get(w, gp.no_bins)


class PgbLaunchConfig(C.Structure):
    _fields_ = [("push_blocks_per_sm", C.c_int32), ("field_sms", C.c_int32)]


class PgbProfile(C.Structure):
    """ctypes image of `pgb_profile` (include/picgb.h)."""

    _fields_ = [("ms_push_e", C.c_double), ("ms_push_i", C.c_double), ("ms_collide_ions", C.c_double),
                ("ms_walls", C.c_double), ("ms_fields", C.c_double), ("steps", C.c_int64),
                ("slots_e", C.c_int64), ("slots_i", C.c_int64), ("launches", C.c_int64),
                ("ms_push_e_kernel", C.c_double), ("ms_collide_e", C.c_double),
                ("ms_scatter_e", C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


def _yes(v) -> int:
    if isinstance(v, str):
        return 1 if v.upper() == "YES" else 0
    return 1 if v else 0


def make_params(**kw) -> PgbParams:
    """Build run parameters from parameters.h-style inputs.

    Keyword names are the parameters.h macros (upper case); the derived
    quantities use the reference's formulas (parameters.h:71-262):
    NEUTRAL_DENSITY from GAS_PRESSURE_TORR, VTE/VTI/VTN from TEMPERATURE,
    XLENGTH = NO_OF_DEBYE_LENGTHS * DEBYE_LENGTH, DX = XLENGTH/(X_NO_OF_CELLS-1),
    DT = 0.1/PLASMA_FREQUENCY (scale DT_SCALE), DTI = DTI_RATIO*DT.
    Defaults are those of the reference's parameters.h.
    """
    g = dict(
        X_NO_OF_CELLS=257, TEMPERATURE=1.5, GAS_PRESSURE_TORR=0.2, ION_MASS_AMU=39.948,
        THRESHOLD=15.75, WORK_FUNCTION=4.6, HAVE_COLLISIONS=False, SPECIES="ARGON",
        SIGMA="CONSTANT", SIGMA_VALUE=0.0, SIGMA_ELASTIC="CONSTANT", ELASTIC_SIGMA_VALUE=0.0,
        SIGMA_IONIZATION="CONSTANT", IONIZATION_SIGMA_VALUE=0.0, E_IMPACT_SEE="NO",
        ION_IMPACT_SEE="NO", REFLECTION="NO", BACKSCATTER="NO", STEADYSTATE="YES",
        NUMBER_TO_INJECT=0, INIT_NO_NEUTRALS=10000, NO_OF_DEBYE_LENGTHS=64,
        ELECTRON_PARTICLE_DENSITY=1.0e15, DT_SCALE=0.1, DTI_RATIO=1.0, MAGNETIC_FIELD=0.0,
        ANGLE_DEG=30.0, PHI_LEFT=0.0, PHI_RIGHT=0.0, PHI_PERIOD=0.0, PHI_TOP=0.0,
        PHI_BOTTOM=0.0, E_MACROPARTICLE_SIZE=1.0e6, ION_MACROPARTICLE_SIZE=1.0e6,
        SIZE_TO_CHECK=1000001, SIZE_TO_CHECK_E=None, UPPER_GROUP_LIMIT=400000, UPPER_GROUP_LIMIT2=100000,
        NEW_GROUP_SIZE=200000, NEW_GROUP_SIZE2=50000, RAND_SEED=1, POISSON="FMG_REF",
        DC_MAX_ITERS=8, DC_TOLERANCE=1e-10, SORT_INTERVAL=0, CAPACITY_E=0, CAPACITY_I=0,
    )
    for k, v in kw.items():
        if k not in g:
            raise KeyError(f"unknown parameter {k}")
        g[k] = v
    T = float(g["TEMPERATURE"])
    ion_mass = float(g["ION_MASS_AMU"]) * AMU
    gas_pressure = float(g["GAS_PRESSURE_TORR"]) * 133.32
    n_e = float(g["ELECTRON_PARTICLE_DENSITY"])
    debye = math.sqrt((EPSILON * T) / (n_e * CHARGE))
    xlength = float(int(g["NO_OF_DEBYE_LENGTHS"])) * debye
    plasma_frequency = math.sqrt((n_e * ELECTRON_CHARGE2) / (EPSILON * ELECTRON_MASS))
    dt = float(g["DT_SCALE"]) / plasma_frequency
    vte = math.sqrt(T * CHARGE / ELECTRON_MASS)
    vti = math.sqrt(T * CHARGE / ion_mass)
    p = PgbParams()
    n = int(g["X_NO_OF_CELLS"])
    p.x_no_of_cells = p.y_no_of_cells = n
    p.xlength = p.ylength = xlength
    p.dt = dt
    p.dti = float(g["DTI_RATIO"]) * dt
    p.electron_mass = ELECTRON_MASS
    p.ion_mass = ion_mass
    p.q_over_me = -CHARGE / ELECTRON_MASS
    p.q_over_mi = CHARGE / ion_mass
    p.qce = float(g["E_MACROPARTICLE_SIZE"]) * -CHARGE
    p.qci = float(g["ION_MACROPARTICLE_SIZE"]) * CHARGE
    p.vte, p.vti = vte, vti
    p.vtn = math.sqrt(0.025 * CHARGE / ion_mass)
    p.magnetic_field = float(g["MAGNETIC_FIELD"])
    p.angle = float(g["ANGLE_DEG"]) * PI / 180.0
    p.phi_left, p.phi_right = float(g["PHI_LEFT"]), float(g["PHI_RIGHT"])
    p.phi_bottom, p.phi_top = float(g["PHI_BOTTOM"]), float(g["PHI_TOP"])
    p.phi_period = float(g["PHI_PERIOD"])
    p.neutral_density = gas_pressure / (0.025 * CHARGE)
    p.threshold = float(g["THRESHOLD"])
    p.work_function = float(g["WORK_FUNCTION"])
    p.have_collisions = 1 if g["HAVE_COLLISIONS"] else 0
    p.species = PGB_ARGON if str(g["SPECIES"]).upper() == "ARGON" else PGB_HYDROGEN
    mode = lambda s: PGB_SIGMA_CONSTANT if str(s).upper() == "CONSTANT" else PGB_SIGMA_ENERGY_DEPENDENT
    p.sigma_cx_mode = mode(g["SIGMA"])
    p.sigma_elastic_mode = mode(g["SIGMA_ELASTIC"])
    p.sigma_ionization_mode = mode(g["SIGMA_IONIZATION"])
    p.sigma_value = float(g["SIGMA_VALUE"])
    p.elastic_sigma_value = float(g["ELASTIC_SIGMA_VALUE"])
    p.ionization_sigma_value = float(g["IONIZATION_SIGMA_VALUE"])
    p.e_impact_see = _yes(g["E_IMPACT_SEE"])
    p.ion_impact_see = _yes(g["ION_IMPACT_SEE"])
    p.reflection = _yes(g["REFLECTION"])
    p.backscatter = _yes(g["BACKSCATTER"])
    p.steadystate = _yes(g["STEADYSTATE"])
    p.number_to_inject = int(g["NUMBER_TO_INJECT"])
    p.init_no_neutrals = int(g["INIT_NO_NEUTRALS"])
    p.see_e0, p.see_max_yield, p.see_emax0 = 4.32, 1.4, 650.0
    # Kunhardt groups (parameters.h:339-366, pic.cpp:257-327)
    p.no_groups = 3
    for k, v in enumerate((2.0 * vte, 3.0 * vte, 1000.0 * vte)):
        p.v_limit_e[k] = v
    for k, v in enumerate((2.0 * vti, 3.0 * vti, 1000.0 * vti)):
        p.v_limit_i[k] = v
    gl, gl2 = int(g["UPPER_GROUP_LIMIT"]), int(g["UPPER_GROUP_LIMIT2"])
    ng, ng2 = int(g["NEW_GROUP_SIZE"]), int(g["NEW_GROUP_SIZE2"])
    for k in range(3):
        p.group_limit_e[k] = gl
        p.new_group_size_e[k] = ng
    p.group_limit_i[0], p.group_limit_i[1], p.group_limit_i[2] = gl, gl2, gl2
    p.new_group_size_i[0], p.new_group_size_i[1], p.new_group_size_i[2] = ng, ng2, ng2
    stc = int(g["SIZE_TO_CHECK"])
    p.size_to_check_i = stc
    p.size_to_check_e = int(g["SIZE_TO_CHECK_E"]) if g["SIZE_TO_CHECK_E"] is not None else stc
    p.seed = int(g["RAND_SEED"])
    p.poisson_mode = POISSON_MODES[str(g["POISSON"]).upper()]
    p.dc_max_iters = int(g["DC_MAX_ITERS"])
    p.dc_tolerance = float(g["DC_TOLERANCE"])
    p.sort_interval = int(g["SORT_INTERVAL"])
    p.capacity_e = int(g["CAPACITY_E"])
    p.capacity_i = int(g["CAPACITY_I"])
    return p


def grid_shape(p: PgbParams, which: str) -> tuple:
    nx, ny = p.x_no_of_cells, p.y_no_of_cells
    if which in ("ex", "ey"):
        return ((nx + 1) * (ny + 1),)
    return (ny, nx)


# ---------------------------------------------------------------- library
def library_path() -> str:
    return os.path.join(PKG_DIR, "libpicgb.so")


_LIB = None


def load_library():
    """Load libpicgb.so; raise if it was not built (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"libpicgb.so not built at {path}: run __graft_entry__.build()")
    lib = C.CDLL(path)
    R = C.c_void_p
    i32, i64, dp = C.c_int32, C.c_int64, C.POINTER(C.c_double)
    sig = {
        "pgb_params_default": (C.c_int, [C.POINTER(PgbParams)]),
        "pgb_create": (C.c_int, [C.POINTER(PgbParams), C.POINTER(R)]),
        "pgb_destroy": (C.c_int, [R]),
        "pgb_last_error": (C.c_char_p, [R]),
        "pgb_load_species": (C.c_int, [R, C.c_int, dp, i64]),
        "pgb_dump_species": (C.c_int, [R, C.c_int, dp, i64, C.POINTER(i64)]),
        "pgb_species_count": (C.c_int, [R, C.c_int, C.POINTER(i64)]),
        "pgb_dump_ids": (C.c_int, [R, C.c_int, C.POINTER(C.c_uint32), i64, C.POINTER(i64)]),
        "pgb_cross_sections": (C.c_int, [C.c_int32, dp, i64, dp]),
        "pgb_set_time_step": (C.c_int, [R, i64]),
        "pgb_initial_boundary": (C.c_int, [R]),
        "pgb_step": (C.c_int, [R, i32]),
        "pgb_step_batch": (C.c_int, [C.POINTER(R), i32, i32]),
        "pgb_step_async": (C.c_int, [R, i32]),
        "pgb_graphs_params_default": (C.c_int, [C.POINTER(PgbParams), C.POINTER(PgbGraphsParams)]),
        "pgb_graphs_enable": (C.c_int, [R, C.POINTER(PgbGraphsParams)]),
        "pgb_graphs_get": (C.c_int, [R, C.c_int, C.c_int, dp, i64]),
        "pgb_graphs_write": (C.c_int, [R, C.c_char_p]),
        "pgb_render": (C.c_int, [R, C.c_int, i32, i32, i32, C.c_uint32, C.POINTER(C.c_uint8), i64]),
        "pgb_query": (C.c_int, [R, C.POINTER(i32)]),
        "pgb_footprint": (C.c_int, [C.POINTER(PgbParams), i64, i64, C.POINTER(i64)]),
        "pgb_server_create": (C.c_int, [i64, i32, i32, C.POINTER(R)]),
        "pgb_server_destroy": (C.c_int, [R]),
        "pgb_server_submit": (C.c_int, [R, C.POINTER(PgbParams), dp, i64, dp, i64, i32, C.POINTER(i64)]),
        "pgb_server_round": (C.c_int, [R, C.POINTER(i32)]),
        "pgb_server_done": (C.c_int, [R, C.POINTER(i64), i32, C.POINTER(i32)]),
        "pgb_server_result_size": (C.c_int, [R, i64, C.POINTER(i64), C.POINTER(i64)]),
        "pgb_server_result": (C.c_int, [R, i64, dp, i64, dp, i64, C.POINTER(PgbCounters)]),
        "pgb_server_get_stats": (C.c_int, [R, C.POINTER(PgbServerStats)]),
        "pgb_collide_electrons": (C.c_int, [R]),
        "pgb_inject": (C.c_int, [R]),
        "pgb_gather_push": (C.c_int, [R, C.c_int]),
        "pgb_collide_ions": (C.c_int, [R]),
        "pgb_boundary": (C.c_int, [R, C.c_int]),
        "pgb_contain_growth": (C.c_int, [R, C.c_int]),
        "pgb_deposit": (C.c_int, [R, C.c_int]),
        "pgb_grid_rho": (C.c_int, [R]),
        "pgb_poisson": (C.c_int, [R, i64]),
        "pgb_efield": (C.c_int, [R]),
        "pgb_get_grid": (C.c_int, [R, C.c_int, dp, i64]),
        "pgb_set_rho": (C.c_int, [R, dp, i64]),
        "pgb_get_counters": (C.c_int, [R, C.POINTER(PgbCounters)]),
        "pgb_sync": (C.c_int, [R]),
        "pgb_get_stream": (C.c_int, [R, C.POINTER(C.c_void_p)]),
        "pgb_set_profiling": (C.c_int, [R, C.c_int]),
        "pgb_get_profile": (C.c_int, [R, C.POINTER(PgbProfile)]),
        "pgb_get_launch_config": (C.c_int, [R, C.POINTER(PgbLaunchConfig)]),
        "pgb_set_launch_config": (C.c_int, [R, C.POINTER(PgbLaunchConfig)]),
        "pgb_autotune": (C.c_int, [R, i32, C.POINTER(PgbLaunchConfig), dp, dp]),
        "pgb_deposit_static": (C.c_int, [C.c_void_p, i64, i32, i32, C.c_double, C.c_double, C.c_double,
                                         C.c_void_p, C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


PGB_ERR_ARG, PGB_ERR_CUDA, PGB_ERR_NOMEM, PGB_ERR_CAPACITY, PGB_ERR_STATE, PGB_ERR_IO = -1, -2, -3, -4, -5, -6
# cross-section fits (pgb_cross_sections)
XS = {"ar_elastic": 0, "ar_ionize": 1, "h_elastic": 2, "h_ionize": 3, "ar_cx": 4, "h_cx": 5}
PGB_XS_AR_ELASTIC, PGB_XS_AR_IONIZE, PGB_XS_H_ELASTIC, PGB_XS_H_IONIZE, PGB_XS_AR_CX, PGB_XS_H_CX = range(6)


def cross_sections(which, energies) -> np.ndarray:
    """The library's FP32 cross-section fit `which` (a key of XS or a
    PGB_XS_* index) evaluated on the GPU at the energies (eV)."""
    lib = load_library()
    w = XS[which] if isinstance(which, str) else int(which)
    e = np.ascontiguousarray(energies, dtype=np.float64)
    out = np.empty_like(e)
    rc = lib.pgb_cross_sections(w, _dptr(e), e.size, _dptr(out))
    if rc != 0:
        raise PicError(f"pgb_cross_sections failed ({rc}): {lib.pgb_last_error(None).decode()}", rc)
    return out


class PicError(RuntimeError):
    """A failed call; `code` is the library's PGB_ERR_* status (0 when the
    error was found on the Python side)."""

    def __init__(self, msg: str, code: int = 0):
        super().__init__(msg)
        self.code = code


class Run:
    """One simulation on the GPU (a `pgb_run` handle).

    Method names follow the reference's pic / particle / fields calls so that
    a test reads like the reference's step sequence (pic.cpp:1069-1250).
    """

    def __init__(self, params: PgbParams):
        self.lib = load_library()
        self.params = params
        h = C.c_void_p()
        rc = self.lib.pgb_create(C.byref(params), C.byref(h))
        if rc != 0:
            raise PicError(f"pgb_create failed ({rc}): {self.lib.pgb_last_error(None).decode()}")
        self.h = h

    def _check(self, rc: int, what: str):
        if rc != 0:
            raise PicError(f"{what} failed ({rc}): {self.lib.pgb_last_error(self.h).decode()}", rc)

    def close(self):
        if self.h:
            self.lib.pgb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # particles
    def load_particles(self, species: int, aos6: np.ndarray):
        a = np.ascontiguousarray(aos6, dtype=np.float64).reshape(-1, 6)
        self._check(self.lib.pgb_load_species(self.h, species, _dptr(a), a.shape[0]), "pgb_load_species")

    def particle_size(self, species: int) -> int:
        n = C.c_int64()
        self._check(self.lib.pgb_species_count(self.h, species, C.byref(n)), "pgb_species_count")
        return int(n.value)

    def get_particles(self, species: int) -> np.ndarray:
        n = self.particle_size(species)
        out = np.empty((max(n, 1), 6), dtype=np.float64)
        got = C.c_int64()
        self._check(self.lib.pgb_dump_species(self.h, species, _dptr(out), n, C.byref(got)), "pgb_dump_species")
        return out[: got.value].copy()

    def get_ids(self, species: int) -> np.ndarray:
        """Particle ids in get_particles' order (the key of each particle's
        random streams)."""
        n = self.particle_size(species)
        out = np.empty(max(n, 1), dtype=np.uint32)
        got = C.c_int64()
        self._check(self.lib.pgb_dump_ids(self.h, species, out.ctypes.data_as(C.POINTER(C.c_uint32)), n,
                                          C.byref(got)), "pgb_dump_ids")
        return out[: got.value].copy()

    # driver
    def set_time_step(self, t: int):
        self._check(self.lib.pgb_set_time_step(self.h, t), "pgb_set_time_step")

    def initial_boundary(self):
        self._check(self.lib.pgb_initial_boundary(self.h), "pgb_initial_boundary")

    def step(self, n: int = 1):
        self._check(self.lib.pgb_step(self.h, n), "pgb_step")

    # phases
    def collide_electrons(self):
        self._check(self.lib.pgb_collide_electrons(self.h), "pgb_collide_electrons")

    def inject(self):
        self._check(self.lib.pgb_inject(self.h), "pgb_inject")

    def gather_push(self, species: int):
        self._check(self.lib.pgb_gather_push(self.h, species), "pgb_gather_push")

    def collide_ions(self):
        self._check(self.lib.pgb_collide_ions(self.h), "pgb_collide_ions")

    def boundary(self, which: int):
        self._check(self.lib.pgb_boundary(self.h, which), "pgb_boundary")

    def contain_growth(self, species: int):
        self._check(self.lib.pgb_contain_growth(self.h, species), "pgb_contain_growth")

    def deposit(self, species: int):
        self._check(self.lib.pgb_deposit(self.h, species), "pgb_deposit")

    def grid_rho(self):
        self._check(self.lib.pgb_grid_rho(self.h), "pgb_grid_rho")

    def poisson(self, t: int):
        self._check(self.lib.pgb_poisson(self.h, t), "pgb_poisson")

    def efield(self):
        self._check(self.lib.pgb_efield(self.h), "pgb_efield")

    # grids / counters
    def get_grid(self, which: str) -> np.ndarray:
        shape = grid_shape(self.params, which)
        out = np.empty(shape, dtype=np.float64)
        self._check(self.lib.pgb_get_grid(self.h, GRID[which], _dptr(out), out.size), "pgb_get_grid")
        return out

    def set_rho(self, rho: np.ndarray):
        a = np.ascontiguousarray(rho, dtype=np.float64)
        self._check(self.lib.pgb_set_rho(self.h, _dptr(a), a.size), "pgb_set_rho")

    def counters(self) -> dict:
        c = PgbCounters()
        self._check(self.lib.pgb_get_counters(self.h, C.byref(c)), "pgb_get_counters")
        return c.as_dict()

    def sync(self):
        self._check(self.lib.pgb_sync(self.h), "pgb_sync")

    def stream(self) -> int:
        v = C.c_void_p()
        self._check(self.lib.pgb_get_stream(self.h, C.byref(v)), "pgb_get_stream")
        return int(v.value or 0)

    def launch_config(self) -> dict:
        c = PgbLaunchConfig()
        self._check(self.lib.pgb_get_launch_config(self.h, C.byref(c)), "pgb_get_launch_config")
        return {"push_blocks_per_sm": c.push_blocks_per_sm, "field_sms": c.field_sms}

    def set_launch_config(self, push_blocks_per_sm: int, field_sms: int):
        c = PgbLaunchConfig(push_blocks_per_sm, field_sms)
        self._check(self.lib.pgb_set_launch_config(self.h, C.byref(c)), "pgb_set_launch_config")

    def autotune(self, steps: int = 8) -> dict:
        """pgb_autotune: time the 12 launch-shape candidates on this run (it
        advances 12 * (steps + 2) steps) and keep the fastest."""
        c = PgbLaunchConfig()
        best = C.c_double()
        allms = (C.c_double * 12)()
        self._check(self.lib.pgb_autotune(self.h, steps, C.byref(c), C.byref(best), allms), "pgb_autotune")
        cands = [{"push_blocks_per_sm": p, "field_sms": f, "ms_per_step": allms[k]}
                 for k, (p, f) in enumerate((p, f) for p in (4, 8, 12) for f in (8, 16, 32, 48))]
        return {"push_blocks_per_sm": c.push_blocks_per_sm, "field_sms": c.field_sms, "ms_per_step": best.value,
                "candidates": cands}

    def set_profiling(self, on: bool):
        self._check(self.lib.pgb_set_profiling(self.h, 1 if on else 0), "pgb_set_profiling")

    def profile(self) -> dict:
        pr = PgbProfile()
        self._check(self.lib.pgb_get_profile(self.h, C.byref(pr)), "pgb_get_profile")
        return pr.as_dict()

    # averaged diagnostics (the graphs class)
    def graphs_enable(self, gp: PgbGraphsParams):
        """sum the graphs over steps [gp.start_step, gp.end_step) of what is
        stepped from now on"""
        self._gp = gp
        self._check(self.lib.pgb_graphs_enable(self.h, C.byref(gp)), "pgb_graphs_enable")

    def graphs_get(self, which: str, species: int = 0) -> np.ndarray:
        """one averaged graph: [ny, nx] for the grids, 1-D otherwise"""
        p = self.params
        out = np.empty(graph_size(which, p, self._gp))
        self._check(self.lib.pgb_graphs_get(self.h, GRAPH[which], species, _dptr(out), out.size), "pgb_graphs_get")
        return out.reshape(p.y_no_of_cells, p.x_no_of_cells) if GRAPH[which] <= 4 else out

    def graphs_write(self, directory: str):
        """the reference's graph text files, written into directory"""
        self._check(self.lib.pgb_graphs_write(self.h, os.fsencode(directory)), "pgb_graphs_write")

    def render(self, plot: str, width: int = 512, height: int = 512, max_points: int = NUM_PARTICLES_TO_PLOT,
               seed: int = 0) -> np.ndarray:
        """one of the viewer's plots as an (height, width, 3) uint8 image,
        row 0 at the top (pgb_render)"""
        img = np.empty((height, width, 3), dtype=np.uint8)
        self._check(self.lib.pgb_render(self.h, PLOT[plot], width, height, max_points, seed,
                                        img.ctypes.data_as(C.POINTER(C.c_uint8)), img.size), "pgb_render")
        return img

    def load_particles_ptr(self, species: int, ptr: int, n: int):
        """Load n records from a host address (e.g. pinned memory)."""
        self._check(self.lib.pgb_load_species(self.h, species, C.cast(ptr, C.POINTER(C.c_double)), n),
                    "pgb_load_species")

    def dump_particles_ptr(self, species: int, ptr: int, cap: int) -> int:
        got = C.c_int64()
        self._check(self.lib.pgb_dump_species(self.h, species, C.cast(ptr, C.POINTER(C.c_double)), cap,
                                              C.byref(got)), "pgb_dump_species")
        return int(got.value)


# ------------------------------------------------------------- dataDump I/O
def footprint(params: PgbParams, ne: int, ni: int) -> int:
    """Device bytes of a run of these parameters with ne + ni particles."""
    lib = load_library()
    out = C.c_int64()
    if lib.pgb_footprint(C.byref(params), ne, ni, C.byref(out)) != 0:
        raise PicError(lib.pgb_last_error(None).decode())
    return out.value


class Server:
    """pgb_server_*: a request loop keeping many runs resident on the GPU.

    submit() queues a run (parameters, initial particles, steps); round()
    admits queued runs that fit the HBM budget, steps every resident run
    together and retires finished ones; results() returns the finished
    runs' particles and counters."""

    def __init__(self, hbm_budget: int, round_steps: int = 10, max_active: int = 64):
        self.lib = load_library()
        h = C.c_void_p()
        self._check(self.lib.pgb_server_create(hbm_budget, round_steps, max_active, C.byref(h)), "pgb_server_create")
        self.h = h

    def _check(self, rc, what):
        if rc != 0:
            raise PicError(f"{what} failed ({rc}): {self.lib.pgb_last_error(None).decode()}", rc)

    def submit(self, params: PgbParams, e: np.ndarray, i: np.ndarray, nsteps: int) -> int:
        e = np.ascontiguousarray(e, dtype=np.float64)
        i = np.ascontiguousarray(i, dtype=np.float64)
        rid = C.c_int64()
        self._check(self.lib.pgb_server_submit(self.h, C.byref(params), _dptr(e), e.shape[0], _dptr(i), i.shape[0],
                                               nsteps, C.byref(rid)), "pgb_server_submit")
        return rid.value

    def round(self) -> int:
        n = C.c_int32()
        self._check(self.lib.pgb_server_round(self.h, C.byref(n)), "pgb_server_round")
        return n.value

    def results(self) -> dict:
        """{id: (electrons, ions, counters)} for every finished request not taken yet."""
        out = {}
        while True:
            ids = (C.c_int64 * 64)()
            n = C.c_int32()
            self._check(self.lib.pgb_server_done(self.h, ids, 64, C.byref(n)), "pgb_server_done")
            if n.value == 0:
                return out
            for k in range(n.value):
                ne, ni = C.c_int64(), C.c_int64()
                self._check(self.lib.pgb_server_result_size(self.h, ids[k], C.byref(ne), C.byref(ni)),
                            "pgb_server_result_size")
                e = np.empty((max(ne.value, 1), 6))
                i = np.empty((max(ni.value, 1), 6))
                c = PgbCounters()
                self._check(self.lib.pgb_server_result(self.h, ids[k], _dptr(e), ne.value, _dptr(i), ni.value,
                                                       C.byref(c)), "pgb_server_result")
                out[ids[k]] = (e[:ne.value], i[:ni.value], c.as_dict())

    def stats(self) -> dict:
        st = PgbServerStats()
        self._check(self.lib.pgb_server_get_stats(self.h, C.byref(st)), "pgb_server_get_stats")
        return st.as_dict()

    def close(self):
        if self.h:
            self.lib.pgb_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def step_batch(runs, n: int = 1):
    """pgb_step_batch: step independent runs together (each on its own
    stream); every run ends as after Run.step(n) alone."""
    lib = load_library()
    arr = (C.c_void_p * len(runs))(*[r.h.value for r in runs])
    rc = lib.pgb_step_batch(arr, len(runs), n)
    if rc != 0:
        msgs = [r.lib.pgb_last_error(r.h).decode() for r in runs]
        msgs.append(lib.pgb_last_error(None).decode())
        raise PicError(f"pgb_step_batch failed ({rc}): " + "; ".join(m for m in msgs if m and m != "no error"))


def read_datadump(path: str) -> np.ndarray:
    """particle::load_particles (particle.cpp:359-401): whitespace-separated
    records `x y vx vy vz weight`, read while `in >> x >> ... >> weight`
    succeeds: up to the first incomplete record or the first token that is
    not a number."""
    with open(path, "rb") as f:
        toks = f.read().split()
    try:
        vals = np.array(toks, dtype=np.float64)
    except ValueError:
        good = []
        for t in toks:
            try:
                good.append(float(t))
            except ValueError:
                break
        vals = np.array(good, dtype=np.float64)
    n = vals.size // 6
    return vals[: n * 6].reshape(n, 6)


def write_datadump(path: str, aos6: np.ndarray):
    """particle::dump_data (particle.cpp:1361-1382): `ofstream <<` of each
    double at the default precision (6 significant digits, %g style)."""
    a = np.asarray(aos6, dtype=np.float64).reshape(-1, 6)
    with open(path, "w") as f:
        for row in a:
            f.write(" ".join(_ostream_double(v) for v in row) + "\n")


DUMP_MAGIC = b"PGBDUMP1"


def read_datadump_bin(path: str) -> np.ndarray:
    """The lossless binary dump (no reference counterpart): "PGBDUMP1", an
    int64 record count, then little-endian doubles {x, y, vx, vy, vz, w}."""
    with open(path, "rb") as f:
        head = f.read(16)
        if len(head) != 16 or head[:8] != DUMP_MAGIC:
            raise PicError(f"{path}: not a binary particle dump")
        n = int(np.frombuffer(head[8:], dtype="<i8")[0])
        a = np.fromfile(f, dtype="<f8", count=6 * n)
    if a.size != 6 * n:
        raise PicError(f"{path}: truncated binary particle dump")
    return a.reshape(n, 6).astype(np.float64)


def write_datadump_bin(path: str, aos6: np.ndarray):
    a = np.ascontiguousarray(aos6, dtype="<f8").reshape(-1, 6)
    with open(path, "wb") as f:
        f.write(DUMP_MAGIC)
        f.write(np.array([a.shape[0]], dtype="<i8").tobytes())
        f.write(a.tobytes())


def _ostream_double(v: float) -> str:
    if v != v:
        return "nan" if math.copysign(1.0, v) > 0 else "-nan"
    if v in (math.inf, -math.inf):
        return "inf" if v > 0 else "-inf"
    return "%g" % v
