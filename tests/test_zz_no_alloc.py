"""The allocation-free 1-D density entry point.

Some callers cannot allocate device memory: their device memory belongs to
another framework's pool, or they run in a service that must not allocate
after start-up. ent_density_1d_noalloc serves them from one fixed device
array inside the library. This test calls it through the C ABI on two inputs
in a row (the second call reuses the array the first one left behind) and
checks each result against the allocating entry point, ent_densities_device,
at the density tolerance of the other tests (1e-5 relative per point). It
also checks the size limit. It lives in a file of its own that pytest
collects last, and it passes alone in a fresh process as well as after the
other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-5


def _noalloc(lib, dx, n, h, dout):
    return lib.ent_density_1d_noalloc(C.c_void_p(dx.data_ptr()), n, h,
                                      C.c_void_p(dout.data_ptr()), None)


def test_no_alloc_density_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    from entropical_gb300 import Context, workloads
    torch.cuda.set_device(0)
    ctx = Context(0)
    lib = ctx.lib
    cases = [(workloads.gmm_1d(20_000, seed=42), 0.1),
             (np.random.default_rng(8).standard_normal(65_536).astype(np.float32) * 3, 0.05)]
    for x, h in cases:
        n = x.size
        dx = torch.from_numpy(x).cuda()
        dout = torch.zeros(n, dtype=torch.float64, device="cuda")
        assert _noalloc(lib, dx, n, h, dout) == 0
        torch.cuda.synchronize()
        ref = torch.zeros(n, dtype=torch.float64, device="cuda")
        ctx.combined_densities_device(dx.data_ptr(), n, 1, [0], [h], None, ref.data_ptr())
        torch.cuda.synchronize()
        p, r = dout.cpu().numpy(), ref.cpu().numpy()
        assert np.max(np.abs(p - r) / r) < REL
    # beyond the fixed array: a clear error, nothing written
    big = torch.zeros(65_537, dtype=torch.float32, device="cuda")
    out = torch.zeros(65_537, dtype=torch.float64, device="cuda")
    assert _noalloc(lib, big, 65_537, 0.1, out) == 9  # ENT_ERR_TOO_LARGE
    ctx.close()


def test_no_alloc_errors_and_caller_stream():
    """Invalid input is refused with the library's status codes (a NaN in the
    column, a bandwidth that is not positive), the array left usable, and a
    call on the caller's own stream matches the allocating entry point."""
    torch = pytest.importorskip("torch")
    from entropical_gb300 import Context
    torch.cuda.set_device(0)
    ctx = Context(0)
    lib = ctx.lib
    x = np.random.default_rng(9).standard_normal(5000).astype(np.float32)
    dout = torch.zeros(5000, dtype=torch.float64, device="cuda")
    bad = x.copy()
    bad[123] = np.nan
    assert _noalloc(lib, torch.from_numpy(bad).cuda(), 5000, 0.2, dout) == 5  # ENT_ERR_NONFINITE
    dx = torch.from_numpy(x).cuda()
    assert _noalloc(lib, dx, 5000, 0.0, dout) == 4    # ENT_ERR_ARG
    assert _noalloc(lib, dx, 5000, -0.2, dout) == 4
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        rc = lib.ent_density_1d_noalloc(C.c_void_p(dx.data_ptr()), 5000, 0.2,
                                        C.c_void_p(dout.data_ptr()), C.c_void_p(s.cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    ref = torch.zeros(5000, dtype=torch.float64, device="cuda")
    ctx.combined_densities_device(dx.data_ptr(), 5000, 1, [0], [0.2], None, ref.data_ptr())
    torch.cuda.synchronize()
    p, r = dout.cpu().numpy(), ref.cpu().numpy()
    assert np.max(np.abs(p - r) / r) < REL
    ctx.close()
