"""Data ingest (FFTGrid::fillInData's per-trace core) on the GPU against the oracle."""
import numpy as np
import pytest
import torch

from conftest import rel

pytestmark = pytest.mark.gpu


def _case(nxp, nyp, nzp, nz, n_data, seed, dz=4.0):
    from crava_gb300 import api
    _, rnxp = api.dims(nxp)
    ncol = rnxp * nyp
    rng = np.random.default_rng(seed)
    # band-limited traces with a linear trend, leading/trailing zeros on some, dead columns
    t = np.arange(n_data)
    tr = np.stack([np.sin(2 * np.pi * rng.uniform(0.01, 0.08) * t + rng.uniform(0, 6)) * rng.uniform(0.5, 2)
                   + rng.uniform(-1, 1) + 0.01 * rng.uniform(-1, 1) * t for _ in range(ncol)]).astype(np.float32)
    for c in rng.choice(ncol, ncol // 5, replace=False):
        tr[c, :rng.integers(1, 6)] = 0
        tr[c, n_data - rng.integers(1, 4):] = 0
    state = (rng.uniform(size=ncol) < 0.05).astype(np.uint8)
    z0_data = (1000.0 + rng.uniform(-8, 8, ncol)).astype(np.float32)
    z0_grid = (z0_data + rng.uniform(-6, 30, ncol)).astype(np.float32)   # some cells above/below the data
    dz_grid = rng.uniform(3.5, 4.5, ncol).astype(np.float32)
    return tr, state, z0_data, z0_grid, dz_grid, dz


@pytest.mark.parametrize("dims,n_data", [((20, 12, 40, 30), 37), ((64, 30, 64, 50), 75), ((45, 16, 80, 64), 96)])
@pytest.mark.parametrize("cubetype", ["DATA", "PARAMETER"])
def test_fill_in_data_matches_oracle(cuda, oracle, dims, n_data, cubetype):
    from crava_gb300 import api
    nxp, nyp, nzp, nz = dims
    ctype = api.DATA if cubetype == "DATA" else api.PARAMETER
    tr, state, z0d, z0g, dzg, dz = _case(nxp, nyp, nzp, nz, n_data, nxp + n_data)
    ref, ref_ext = oracle.fill_in_data(nxp, nyp, nzp, nz, cubetype == "DATA", tr, state, z0d, z0g, dzg, dz, 20.0)
    _, rnxp = api.dims(nxp)
    buf = torch.full((nzp, nyp, rnxp), 7.0, device="cuda")
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    ext = api.fill_in_data(buf, nxp, nz, ctype, dev(tr), dev(state), dev(z0d), dev(z0g), dev(dzg), dz, 20.0)
    got = buf.cpu().numpy()
    e = rel(got, ref)
    print(dims, n_data, cubetype, "fill_in_data vs oracle:", e, ext, ref_ext)
    assert e < 2e-6
    assert ext == ref_ext
    dead = np.nonzero(state)[0]
    assert np.all(got.reshape(nzp, -1)[:, dead] == 0)


def test_fill_in_data_rejects_bad_arguments(cuda, native):
    assert native.cg_fill_in_data(None, 8, 8, 8, 8, 1, None, 10, None, None, None, None, 4.0, 0.0, None, None) == -1
