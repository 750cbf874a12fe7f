"""Local-noise correction (Crava::correctAlphaBetaRho), CPU side: the oracle's per-trace matrices against a
numpy restatement of newPosteriorCovPointwise that uses LAPACK's geev like the reference, and the defining
property of computeG: with every local scale at its minimum the correction is the identity."""
import numpy as np
import pytest


def _model(n=5, seed=1):
    from crava_gb300 import synthetic as S
    sc = S.make_scenario(12, 10, 16, list(np.linspace(5, 40, n)), 28.0, nxp=16, nyp=12, nzp=20, seed=seed)
    Sm = sc.sigma0.astype(np.float64)
    # a posterior variance at the origin between 30 and 70 % of the prior, correlated
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((3, 3)) * 0.15
    Q = np.linalg.cholesky(Sm)
    F = np.eye(3) * 0.5 + (B + B.T) * 0.1
    Smd = Q @ F @ F.T @ Q.T
    return sc, Sm, 0.5 * (Smd + Smd.T)


def _numpy_pointwise(G, E, Sm, Smd, scales):
    """newPosteriorCovPointwise (src/crava.cpp:2345-2451) line by line with np.linalg.eig (LAPACK geev)."""
    from crava_gb300.api import _eig
    n = G.shape[0]
    D = np.diag(np.sqrt(scales))
    help_ = G @ Sm @ G.T + D @ E @ D
    w, V = _eig(help_)
    H = V @ np.diag(np.where(w > 0.00000001, 1.0 / w, 0.0)) @ V.T
    deltanew = Sm @ G.T @ H @ G @ Sm
    w, V = _eig(Sm - deltanew)
    smdnew = V @ np.diag(np.where(w > 0.0, np.sqrt(np.abs(w)), 0.0)) @ V.T
    w, V = _eig(deltanew)
    dsq = V @ np.diag(np.where(w > 0.0, np.sqrt(np.abs(w)), 0.0)) @ V.T
    w, V = _eig(Sm - Smd)
    sdinv = V @ np.diag(np.where(w > 0.0000001, 1.0 / np.sqrt(np.abs(w)), 0.0)) @ V.T
    assert n == E.shape[0]
    return dsq @ sdinv, smdnew


@pytest.mark.parametrize("n", [3, 5, 8])
def test_oracle_pointwise_matches_lapack_restatement(oracle, native, n):
    from crava_gb300 import api
    sc, Sm, Smd = _model(n)
    G = api.local_noise_g(sc.err_theta_cov, Sm, Smd)
    rng = np.random.default_rng(n)
    for _ in range(5):
        scales = rng.uniform(1.0, 3.0, n)
        a, b = oracle.new_posterior_cov_pointwise(G, sc.err_theta_cov, Sm, Smd, scales)
        ra, rb = _numpy_pointwise(G, sc.err_theta_cov, Sm, Smd, scales)
        assert np.abs(a - ra).max() < 1e-9 * max(1.0, np.abs(ra).max())
        assert np.abs(b - rb).max() < 1e-9 * max(1.0, np.abs(rb).max())


@pytest.mark.parametrize("n", [3, 5])
def test_unit_scales_leave_the_posterior_unchanged(oracle, native, n):
    """computeG is built so that Sm G^T (G Sm G^T + Se)^-1 G Sm = Sm - Spost: at the minimum scale everywhere
    the correction matrix is the identity."""
    from crava_gb300 import api
    sc, Sm, Smd = _model(n, seed=3)
    G = api.local_noise_g(sc.err_theta_cov, Sm, Smd)
    a, _ = oracle.new_posterior_cov_pointwise(G, sc.err_theta_cov, Sm, Smd, np.ones(n))
    assert np.abs(a - np.eye(3)).max() < 1e-8
    # a larger local noise shrinks the update towards the prior
    a2, _ = oracle.new_posterior_cov_pointwise(G, sc.err_theta_cov, Sm, Smd, np.full(n, 4.0))
    assert np.linalg.norm(a2, 2) < 1.0


def test_oracle_correction_trace_loop(oracle):
    sc, Sm, Smd = _model(3, seed=5)
    from crava_gb300 import api
    G = api.local_noise_g(sc.err_theta_cov, Sm, Smd)
    rng = np.random.default_rng(2)
    nx, ny, nz, nxp = sc.nx, sc.ny, sc.nz, sc.nxp
    scale = rng.uniform(1.0, 2.0, (3, ny, nx))
    scale[1, 2, 3] = -99999.0   # RMISSING is left out of the minimum
    post = [m + 0.01 * rng.standard_normal(m.shape).astype(np.float32) for m in sc.mean]
    out, smd = oracle.correct_alpha_beta_rho(post, sc.mean, nx, ny, nz, nxp, G, sc.err_theta_cov, Sm, Smd, scale,
                                             want_sigmamd=True)
    i, j, k = 4, 5, 7
    mins = [scale[l][scale[l] != -99999.0].min() for l in range(3)]
    sn, smdn = _numpy_pointwise(G, sc.err_theta_cov, Sm, Smd, np.array([scale[l, j, i] / mins[l] for l in range(3)]))
    d = np.array([post[p][k, j, i] - sc.mean[p][k, j, i] for p in range(3)], dtype=np.float32)
    want = np.array([sc.mean[p][k, j, i] for p in range(3)], dtype=np.float64) + sn @ d.astype(np.float64)
    got = np.array([out[p][k, j, i] for p in range(3)])
    assert np.abs(got - want.astype(np.float32)).max() <= 2e-7 * np.abs(want).max()
    w, V = np.linalg.eigh(Smd)
    assert np.abs(smd[j, i].reshape(3, 3) - smdn @ (V @ np.diag(1 / np.sqrt(w)) @ V.T)).max() < 1e-9
    # padding cells and cells below nz are untouched
    assert np.array_equal(out[0][nz:], post[0][nz:]) and np.array_equal(out[1][:, ny:], post[1][:, ny:])
