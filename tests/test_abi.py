"""The C ABI boundary: exported symbols, parameter defaults, loud failure.

These run without a GPU: loading libpicgb.so and calling the functions that
do not touch the device is enough to check the boundary.
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "picgb.h")


def header_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^PGB_API\s+[\w\s\*]+?\b(pgb_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_entry_points():
    names = header_functions()
    for required in ("pgb_create", "pgb_destroy", "pgb_step", "pgb_load_species", "pgb_dump_species",
                     "pgb_gather_push", "pgb_deposit", "pgb_poisson", "pgb_efield", "pgb_boundary",
                     "pgb_collide_electrons", "pgb_collide_ions"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    import picgb
    for name in header_functions():
        assert hasattr(lib, name), f"libpicgb.so does not export {name}"
    out = subprocess.run(["nm", "-D", "--defined-only", picgb.library_path()], capture_output=True, text=True).stdout
    exported = sorted(set(re.findall(r"\bT (pgb_\w+)", out)))
    assert exported == header_functions(), "exports and header differ"


def test_params_default_matches_parameters_h(lib):
    """pgb_params_default (C) and make_params() (Python) restate the same
    parameters.h defaults (parameters.h:41-366)."""
    import picgb
    a = picgb.PgbParams()
    assert lib.pgb_params_default(C.byref(a)) == 0
    b = picgb.make_params()
    for name, _ in picgb.PgbParams._fields_:
        va, vb = getattr(a, name), getattr(b, name)
        if hasattr(va, "__len__"):
            assert list(va) == list(vb), name
        else:
            assert va == vb, name


def test_create_rejects_bad_grid(lib):
    import picgb
    p = picgb.make_params(X_NO_OF_CELLS=100)
    h = C.c_void_p()
    rc = lib.pgb_create(C.byref(p), C.byref(h))
    assert rc == -1 and not h.value
    assert b"power of 2" in lib.pgb_last_error(None)


def test_create_rejects_unknown_poisson_mode_and_pass_count(lib):
    import picgb
    for field, value, text in (("poisson_mode", 7, b"poisson_mode"), ("dc_max_iters", -1, b"dc_max_iters"),
                               ("dc_max_iters", 65, b"dc_max_iters")):
        p = picgb.make_params(X_NO_OF_CELLS=33)
        setattr(p, field, value)
        h = C.c_void_p()
        rc = lib.pgb_create(C.byref(p), C.byref(h))
        assert rc == -1 and not h.value, field
        assert text in lib.pgb_last_error(None), field


def test_no_silent_cpu_fallback_without_a_gpu(lib):
    """Without a usable GPU the library reports a CUDA error; it never
    computes on the host instead."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import picgb
    p = picgb.make_params(X_NO_OF_CELLS=33)
    h = C.c_void_p()
    rc = lib.pgb_create(C.byref(p), C.byref(h))
    assert rc == -2 and not h.value
    assert lib.pgb_last_error(None)


def test_datadump_text_format_matches_reference():
    """particle::dump_data writes each double with `ofstream <<` at the
    default precision (particle.cpp:1361-1382); write_datadump reproduces
    the reference's own dump byte for byte."""
    import tempfile
    import picgb
    from conftest import load_golden
    g = load_golden("core33")
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "dataDump_e.txt")
        picgb.write_datadump(path, g["e_out"])
        head = "".join(open(path).readlines()[:20])
        assert head == str(g["dump_e_head"])
        back = picgb.read_datadump(path)
        np.testing.assert_allclose(back, g["e_out"], rtol=5e-6)


def test_footprint_grows_with_particles_and_grid(lib):
    import picgb
    small = picgb.make_params(X_NO_OF_CELLS=65)
    big = picgb.make_params(X_NO_OF_CELLS=257)
    a = picgb.footprint(small, 1000, 1000)
    b = picgb.footprint(small, 1_000_000, 1_000_000)
    c = picgb.footprint(big, 1000, 1000)
    assert 0 < a < b and a < c
    # particles dominate: about 56 B per slot of capacity (2n + 65536) and species, plus lists
    assert b - a > 2 * 56 * 2 * (1_000_000 - 1000)


def test_server_rejects_a_run_larger_than_its_budget(lib):
    """Admission is by memory: a request that can never fit is refused at
    submission with PGB_ERR_CAPACITY (no GPU work is done)."""
    import picgb
    p = picgb.make_params(X_NO_OF_CELLS=65)
    e = np.zeros((10, 6))
    with picgb.Server(hbm_budget=1 << 20, round_steps=5, max_active=4) as srv:
        with pytest.raises(picgb.PicError, match="budget"):
            srv.submit(p, e, e, 10)
        assert srv.stats()["submitted"] == 0


def test_binary_datadump_round_trips_exactly(tmp_path):
    """The binary restart format keeps every double, NaN and infinities
    included, and rejects files that are not dumps or are cut short."""
    import picgb
    rng = np.random.default_rng(1)
    a = rng.standard_normal((1000, 6)) * 1e-3
    a[3, 2], a[5, 0], a[7, 4] = np.nan, np.inf, -0.0
    path = tmp_path / "dataDump_e.bin"
    picgb.write_datadump_bin(str(path), a)
    b = picgb.read_datadump_bin(str(path))
    assert b.shape == a.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))
    assert path.stat().st_size == 16 + 48 * 1000
    picgb.write_datadump_bin(str(path), np.empty((0, 6)))
    assert picgb.read_datadump_bin(str(path)).shape == (0, 6)
    (tmp_path / "bad.bin").write_bytes(b"NOTADUMP" + bytes(8))
    (tmp_path / "cut.bin").write_bytes(path.read_bytes()[:8] + np.array([5], "<i8").tobytes() + bytes(40))
    for bad in ("bad.bin", "cut.bin"):
        with pytest.raises(picgb.PicError):
            picgb.read_datadump_bin(str(tmp_path / bad))


def test_header_is_plain_c_and_a_c_caller_links(lib, tmp_path):
    """include/picgb.h compiles as strict C99, and a C program links against
    libpicgb.so and calls an entry point that needs no GPU."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    import picgb
    src = tmp_path / "caller.c"
    src.write_text('#include "picgb.h"\n'
                   "int main(void) {\n"
                   "    pgb_params p;\n"
                   "    pgb_launch_config c = {8, 32};\n"
                   "    (void)c;\n"
                   "    if (pgb_params_default(&p) != 0) return 2;\n"
                   "    return p.x_no_of_cells > 2 && p.poisson_mode == PGB_POISSON_FMG_REF ? 0 : 3;\n"
                   "}\n")
    exe = tmp_path / "caller"
    libdir = os.path.dirname(picgb.library_path())
    inc = os.path.join(REPO, "include")
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{inc}", str(src), "-o", str(exe),
                    f"-L{libdir}", "-lpicgb", f"-Wl,-rpath,{libdir}"], check=True)
    assert subprocess.run([str(exe)]).returncode == 0
