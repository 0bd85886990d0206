"""Failures made on the host, never on the GPU: restart files that are cut
short or corrupt, and a device allocation that fails.

- A text dataDump is read as particle::load_particles reads it
  (particle.cpp:385: `while (in >> x >> y >> vx >> vy >> vz >> weight)`):
  up to the first incomplete record or the first token that is not a
  number, by the Python reader and by the C++ driver alike.
- A binary dump with a wrong header or fewer records than it declares is
  refused with a message.
- PGB_FAULT_ALLOC=k makes a handle's k-th particle-storage growth fail as
  if the device were out of memory: the call returns PGB_ERR_NOMEM with a
  message, and the handle stays usable (the same load succeeds next time
  and the run then steps exactly like one that never failed).
"""
import os
import subprocess

import numpy as np
import pytest

import picgb
from conftest import load_golden


def _records(n, seed=1):
    rng = np.random.default_rng(seed)
    return np.column_stack([rng.uniform(1e-3, 2e-3, (n, 2)), rng.normal(0, 1e5, (n, 3)), np.ones(n)])


def test_text_dump_reader_stops_where_the_reference_stops(tmp_path):
    a = _records(5)
    path = tmp_path / "dataDump_e.txt"
    picgb.write_datadump(str(path), a)
    full = picgb.read_datadump(str(path))
    assert full.shape == (5, 6)
    text = path.read_text().splitlines()
    # cut in the middle of the fourth record: three complete records
    path.write_text("\n".join(text[:3]) + "\n" + " ".join(text[3].split()[:4]) + "\n")
    assert np.array_equal(picgb.read_datadump(str(path)), full[:3])
    # a token that is not a number in the third record stops the read there
    bad = text[2].split()
    bad[1] = "x1.0"
    path.write_text("\n".join(text[:2] + [" ".join(bad)] + text[3:]) + "\n")
    assert np.array_equal(picgb.read_datadump(str(path)), full[:2])
    path.write_text("")
    assert picgb.read_datadump(str(path)).shape == (0, 6)


def test_binary_dump_reader_rejects_bad_header_and_truncation(tmp_path):
    a = _records(4)
    path = tmp_path / "dataDump_e.bin"
    picgb.write_datadump_bin(str(path), a)
    assert np.array_equal(picgb.read_datadump_bin(str(path)), a)
    raw = path.read_bytes()
    path.write_bytes(b"PGBDUMP0" + raw[8:])
    with pytest.raises(picgb.PicError, match="not a binary particle dump"):
        picgb.read_datadump_bin(str(path))
    path.write_bytes(raw[:-8])
    with pytest.raises(picgb.PicError, match="truncated"):
        picgb.read_datadump_bin(str(path))


def _driver_dir(tmp_path):
    from test_host_driver import PARAMS_TEXT
    text = PARAMS_TEXT.replace("#define X_NO_OF_CELLS 129", "#define X_NO_OF_CELLS 65") \
                      .replace("#define Y_NO_OF_CELLS 129", "#define Y_NO_OF_CELLS 65")
    (tmp_path / "parameters.h").write_text(text)
    return os.path.join(os.path.dirname(picgb.library_path()), "picgb_run")


def _restart(exe, d, *extra):
    return subprocess.run([exe, str(d / "parameters.h"), str(d), "--steps", "0", "--restart", "--no-graphs", *extra],
                          capture_output=True, text=True, timeout=300)


@pytest.mark.gpu
def test_driver_restarts_from_cut_and_corrupt_text_dumps(tmp_path):
    g = load_golden("core65")
    exe = _driver_dir(tmp_path)
    picgb.write_datadump(str(tmp_path / "dataDump_e.txt"), g["e_in"])
    picgb.write_datadump(str(tmp_path / "dataDump_i1.txt"), g["i_in"])
    lines = (tmp_path / "dataDump_e.txt").read_text().splitlines()
    (tmp_path / "dataDump_e.txt").write_text("\n".join(lines[:700]) + "\n" + lines[700][:7] + "\n")
    ilines = (tmp_path / "dataDump_i1.txt").read_text().splitlines()
    bad = ilines[300].split()
    bad[3] = "--"
    (tmp_path / "dataDump_i1.txt").write_text("\n".join(ilines[:300] + [" ".join(bad)] + ilines[301:]) + "\n")
    out = _restart(exe, tmp_path)
    assert out.returncode == 0, out.stderr
    assert picgb.read_datadump(str(tmp_path / "dataDump_e.txt")).shape == (700, 6)
    assert picgb.read_datadump(str(tmp_path / "dataDump_i1.txt")).shape == (300, 6)


@pytest.mark.gpu
def test_driver_refuses_corrupt_binary_dumps(tmp_path):
    g = load_golden("core65")
    exe = _driver_dir(tmp_path)
    picgb.write_datadump_bin(str(tmp_path / "dataDump_e.bin"), g["e_in"])
    picgb.write_datadump_bin(str(tmp_path / "dataDump_i1.bin"), g["i_in"])
    raw = (tmp_path / "dataDump_e.bin").read_bytes()
    (tmp_path / "dataDump_e.bin").write_bytes(raw[:-48])
    out = _restart(exe, tmp_path, "--binary-dump")
    assert out.returncode != 0 and "truncated binary particle dump" in out.stderr
    (tmp_path / "dataDump_e.bin").write_bytes(b"XXXXXXXX" + raw[8:])
    out = _restart(exe, tmp_path, "--binary-dump")
    assert out.returncode != 0 and "not a binary particle dump" in out.stderr


@pytest.mark.gpu
def test_failed_allocation_leaves_the_handle_usable(monkeypatch):
    g = load_golden("arcoll33")
    p = g["p"]

    def run(fault):
        if fault:
            monkeypatch.setenv("PGB_FAULT_ALLOC", "1")
        else:
            monkeypatch.delenv("PGB_FAULT_ALLOC", raising=False)
        with picgb.Run(p) as r:
            monkeypatch.delenv("PGB_FAULT_ALLOC", raising=False)
            if fault:
                with pytest.raises(picgb.PicError, match="allocation of particle storage failed") as ei:
                    r.load_particles(0, g["e_in"])
                assert ei.value.code == picgb.PGB_ERR_NOMEM
            r.load_particles(0, g["e_in"])
            r.load_particles(1, g["i_in"])
            r.initial_boundary()
            r.step(int(g["nsteps"]))
            return r.get_particles(0), r.get_particles(1), r.get_grid("phi"), r.counters()

    a, b = run(True), run(False)
    assert np.array_equal(a[0], b[0], equal_nan=True) and np.array_equal(a[1], b[1], equal_nan=True)
    assert np.array_equal(a[2], b[2]) and a[3] == b[3]
