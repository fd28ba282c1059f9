"""The allocation-free propagator step (adscf_propagate_step_noalloc).

It serves callers that cannot allocate device memory themselves (memory
pre-partitioned between tenants, a driver that owns every device buffer, hot
paths where an allocation's implicit synchronisation is not allowed).  This
test calls it through the C ABI on device buffers the test owns and checks it
against the context-based adscf_propagate_step and the FP64 oracle's
Propagate_Step on the same inputs, for two calls in a row (the scratch keeps
the previous call's contents, which must not leak into the next result).
Same FP64 tolerance as the other bulk tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_step(lib, torch, grid, size, ds, q, e):
    gx, gy, gz = grid
    dq = torch.tensor(q, device="cuda", dtype=torch.float64).contiguous()
    de = torch.tensor(e, device="cuda", dtype=torch.float64).contiguous()
    stream = torch.cuda.current_stream()
    rc = lib.adscf_propagate_step_noalloc(gx, gy, gz, size[0], size[1], size[2], ds,
                                          ctypes.c_void_p(dq.data_ptr()),
                                          ctypes.c_void_p(de.data_ptr()),
                                          ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    return rc, dq.cpu().numpy()


@pytest.mark.parametrize("grid,size,ds", [((16, 12, 20), (4.0, 3.5, 4.5), 0.01),
                                          ((32, 32, 32), (3.8, 3.8, 3.8), 0.005)])
def test_noalloc_step_matches_context_step(grid, size, ds):
    torch = pytest.importorskip("torch")
    from adscf_gb300 import BULK, FP64, Context, _lib
    from oracle import bulk as ob
    lib = _lib.load()
    gx, gy, gz = grid
    rng = np.random.default_rng(2024)
    explaplace = ob.calculate_laplace(grid, size, ds)
    with Context(BULK, grid=grid, size=size, ds=ds, precision=FP64) as ctx:
        for call in range(2):
            q = 1.0 + 0.3 * rng.standard_normal((gz, gy, gx))
            e = np.exp(-0.5 * ds * rng.standard_normal((gz, gy, gx)))
            ref = ctx.propagate_step(q, e)
            rc, out = _noalloc_step(lib, torch, grid, size, ds, q, e)
            assert rc == _lib.ADSCF_OK, (call, rc)
            assert np.max(np.abs(out - ref)) <= 1e-12 * np.max(np.abs(ref)), call
            want = ob.propagate_step(q, e, explaplace)
            assert np.max(np.abs(out - want)) <= 1e-12 * np.max(np.abs(want)), call


def test_noalloc_rebuild_refused_while_capturing():
    """A call that would rebuild the tables (new grid) synchronises its
    stream, so on a capturing stream it returns ADSCF_E_STATE instead of
    invalidating the caller's capture; the next ordinary call still works."""
    torch = pytest.importorskip("torch")
    from adscf_gb300 import _lib
    lib = _lib.load()
    d = torch.ones(10 * 8 * 6, device="cuda", dtype=torch.float64)
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
        rc = lib.adscf_propagate_step_noalloc(10, 8, 6, 1.0, 1.0, 1.0, 0.01,
                                              ctypes.c_void_p(d.data_ptr()),
                                              ctypes.c_void_p(d.data_ptr()),
                                              ctypes.c_void_p(s.cuda_stream))
    assert rc == _lib.ADSCF_E_STATE
    rc = lib.adscf_propagate_step_noalloc(10, 8, 6, 1.0, 1.0, 1.0, 0.01,
                                          ctypes.c_void_p(d.data_ptr()),
                                          ctypes.c_void_p(d.data_ptr()), None)
    torch.cuda.synchronize()
    assert rc == _lib.ADSCF_OK
    assert bool(torch.isfinite(d).all())


def test_noalloc_rejects_sizes_beyond_scratch():
    torch = pytest.importorskip("torch")
    from adscf_gb300 import _lib
    lib = _lib.load()
    d = torch.zeros(8, device="cuda", dtype=torch.float64)
    rc = lib.adscf_propagate_step_noalloc(128, 128, 128, 1.0, 1.0, 1.0, 0.01,
                                          ctypes.c_void_p(d.data_ptr()),
                                          ctypes.c_void_p(d.data_ptr()), None)
    assert rc == _lib.ADSCF_E_TOO_LARGE
    assert "fixed scratch" in lib.adscf_status_string(rc).decode()
