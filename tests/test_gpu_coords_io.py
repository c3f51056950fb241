"""ent_load_coords_device: blocks of parsed rows copied into a column-major
device matrix with pinned, overlapped copies; bit-exact with the host
loader."""
import numpy as np
import pytest

from entropical_gb300 import read_coords

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("usecols,n", [(None, 40_000), ([0, 5, 63], 40_000), (None, 110_000)])
def test_device_loader_matches_host(ctx, tmp_path, usecols, n):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    # 8 MB blocks of rows: 2 blocks, 1 block, 4 blocks (both staging buffers reused)
    x = rng.standard_normal((64, n)).astype(np.float32)
    p = str(tmp_path / "c.txt")
    np.savetxt(p, x.T, fmt="%.8g")
    host = read_coords(p, usecols)
    dev = torch.zeros(host.shape, dtype=torch.float32, device="cuda")
    n_rows, n_cols = ctx.load_coords_device(p, dev.data_ptr(), usecols)
    torch.cuda.synchronize()
    assert (n_cols, n_rows) == host.shape
    assert np.array_equal(dev.cpu().numpy(), host)
    # the loaded matrix feeds the device entry points directly
    h = [0.3] * 2
    out = torch.zeros(n_rows, dtype=torch.float64, device="cuda")
    ctx.combined_densities_device(dev.data_ptr(), n_rows, n_cols, [0, 1], h, None,
                                  out.data_ptr())
    torch.cuda.synchronize()
    p_host = ctx.combined_densities(host, None, [0, 1], h)
    assert np.allclose(out.cpu().numpy(), p_host, rtol=1e-12)
