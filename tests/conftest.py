import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


def golden(name):
    import numpy as np
    return np.load(os.path.join(REPO, "tests", "golden", name))


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build_oracle()
    return O


@pytest.fixture(scope="session")
def native():
    """The built libcravagpu.so (built here if stale)."""
    import crava_gb300
    crava_gb300.build()
    return crava_gb300.lib()


@pytest.fixture(scope="session")
def cuda(native):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")


def rel(a, b):
    import numpy as np
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def to_cube(spec):
    """complex (nzp, nyp, cnxp) numpy -> float32/64 CUDA cube (nzp, nyp, 2*cnxp)."""
    import numpy as np
    import torch
    real_dt = np.float32 if spec.dtype == np.complex64 else np.float64
    arr = np.ascontiguousarray(spec).view(real_dt)
    return torch.from_numpy(arr.copy()).cuda()


def from_cube(cube):
    import numpy as np
    a = cube.cpu().numpy()
    return a.view(np.complex64 if a.dtype == np.float32 else np.complex128)


def oracle_pipeline(O, sc, prec="d", nthreads=None, tables=None):
    """The whole inversion on the CPU oracle, from real-domain inputs.

    tables: the FP32 per-k operator tables to use (default: the oracle's own);
    pass the GPU path's tables to compare arithmetic on identical inputs."""
    import os
    import numpy as np
    nt = nthreads or os.cpu_count()
    # the operator tables are FP32 inputs on every path (fillErrMultVectors is float in the reference)
    if tables is None:
        tables = O.k_tables(sc.nxp, sc.wavelets, sc.A, sc.nz, sc.nzp, sc.dt_ms, sc.low_cut, sc.high_cut, prec="f")
    tables = dict(tables)
    tables["nxp"] = sc.nxp
    if prec == "d":
        tables = {k: (v.astype(np.complex128) if hasattr(v, "dtype") and v.dtype == np.complex64 else v)
                  for k, v in tables.items()}
    data = [O.fft3d_r2c(d, sc.nxp, O.DATA, prec, nt) for d in sc.data]
    mean = [O.fft3d_r2c(m, sc.nxp, O.PARAMETER, prec, nt) for m in sc.mean]
    covs = []
    gi, gj = getattr(sc, "corr_grad", (0.0, 0.0))
    for (p, q) in [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]:
        c = O.fill_param_corr(sc.nxp, sc.nyp, sc.nzp, sc.corr_xy, sc.circ_corr_t, gi, gj,
                              float(np.float32(sc.sigma0[p, q])), prec=prec)
        covs.append(O.fft3d_r2c(c, sc.nxp, O.COVARIANCE, prec, nt))
    ec = O.fft3d_r2c(O.fill_err_corr(sc.nxp, sc.nyp, sc.nzp, sc.corr_xy, gi, gj, prec=prec), sc.nxp, O.COVARIANCE,
                     prec, nt)
    s0 = np.asarray(sc.sigma0, dtype=np.float64).astype(np.float32).astype(np.float64)
    res, mu, cov, nf = O.invert_bins(data, mean, covs, ec, tables, sc.err_theta_cov, s0, sc.wnc, prec=prec,
                                     nthreads=nt)
    post = np.stack([O.fft3d_c2r(m, sc.nxp, O.PARAMETER, prec, nt)[:, :, :sc.nxp] for m in mu])
    return post, np.stack(res), np.stack(cov), nf
