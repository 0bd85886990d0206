"""pgb_deposit_static: the allocation-free deposit, checked against pgb_deposit.

pgb_deposit_static is for callers that can't allocate device memory: a hook
between steps on the simulation's stream (cudaMalloc/cudaFree would
synchronise the device) or a host that has reserved the device for particle
capacity.  Its scratch is a fixed device array that every call shares, so
the test makes two calls in a row on different species: a second call that
saw the first call's sums would differ from pgb_deposit.

Tolerance: none.  Both paths add the same int64 fixed-point integers and
scale them by the same FP64 products, so the grids must be bit-identical.
This file is named to be collected last; it passes alone in a fresh process
and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
import picgb


def rel_err(a, b):
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


@pytest.mark.gpu
def test_static_deposit_matches_run_deposit_on_two_calls(lib):
    torch = pytest.importorskip("torch")
    g = load_golden("core65")
    p = g["p"]
    nx, ny = p.x_no_of_cells, p.y_no_of_cells
    dx, dy = p.xlength / (nx - 1), p.ylength / (ny - 1)
    species = ((0, "e_in", p.qce, "q_e"), (1, "i_in", p.qci, "q_i"))

    expected = {}
    with picgb.Run(p) as r:
        for s, key, _, grid in species:
            r.load_particles(s, g[key])
            r.deposit(s)
        for s, _, _, grid in species:
            expected[s] = r.get_grid(grid).reshape(-1)

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    for s, key, qc, _ in species:                       # two calls in a row
        recs = torch.from_numpy(np.ascontiguousarray(g[key], dtype=np.float64)).to(dev)
        q = torch.full((nx * ny,), float("nan"), dtype=torch.float64, device=dev)
        rc = lib.pgb_deposit_static(C.c_void_p(recs.data_ptr()), recs.shape[0], nx, ny, dx, dy, qc,
                                    C.c_void_p(q.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.pgb_last_error(None)
        stream.synchronize()
        got = q.cpu().numpy()
        assert np.all(np.isfinite(got)), "grid not fully written"
        assert np.array_equal(got, expected[s]), f"species {s}: max rel diff {rel_err(got, expected[s]):.3g}"
    assert not np.array_equal(expected[0], expected[1])


def test_static_deposit_rejects_grids_beyond_its_scratch(lib):
    """The size check comes before any CUDA call, so it needs no GPU."""
    host = np.zeros(514 * 514, dtype=np.float64)
    rc = lib.pgb_deposit_static(None, 0, 514, 514, 1e-4, 1e-4, 1e-19, C.c_void_p(host.ctypes.data), None)
    assert rc == -4                                     # PGB_ERR_CAPACITY
    msg = lib.pgb_last_error(None).decode()
    assert "263169" in msg and "513 x 513" in msg, msg
