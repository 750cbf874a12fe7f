"""Local-noise correction on the GPU (cg_correct_alpha_beta_rho, cg_apply_trace_matrices) against the oracle."""
import numpy as np
import pytest
import torch

from conftest import rel

pytestmark = pytest.mark.gpu


def _case(n, dims, seed):
    from crava_gb300 import api, synthetic as S
    nx, ny, nz, nxp, nyp, nzp = dims
    sc = S.make_scenario(nx, ny, nz, list(np.linspace(5, 40, n)), 28.0, nxp=nxp, nyp=nyp, nzp=nzp, seed=seed)
    Sm = sc.sigma0.astype(np.float64)
    rng = np.random.default_rng(seed)
    Q = np.linalg.cholesky(Sm)
    B = rng.standard_normal((3, 3)) * 0.1
    F = np.eye(3) * 0.55 + (B + B.T) * 0.1
    Smd = Q @ F @ F.T @ Q.T
    Smd = 0.5 * (Smd + Smd.T)
    G = api.local_noise_g(sc.err_theta_cov, Sm, Smd)
    yy, xx = np.mgrid[0:ny, 0:nx]
    scale = np.stack([1.0 + 0.8 * (0.5 + 0.5 * np.sin(xx / 3.0 + l) * np.cos(yy / 4.0)) for l in range(n)])
    scale[0, 1, 1] = -99999.0
    post = [m + 0.02 * rng.standard_normal(m.shape).astype(np.float32) for m in sc.mean]
    return sc, Sm, Smd, G, scale, post


@pytest.mark.parametrize("n,dims", [(3, (20, 16, 24, 24, 20, 30)), (5, (37, 29, 40, 45, 36, 50)),
                                    (8, (16, 12, 20, 20, 15, 24))])
def test_correct_alpha_beta_rho_matches_oracle(cuda, oracle, n, dims):
    from crava_gb300 import api
    nx, ny, nz, nxp, nyp, nzp = dims
    sc, Sm, Smd, G, scale, post = _case(n, dims, 10 + n)
    ref, smd_ref = oracle.correct_alpha_beta_rho(post, sc.mean, nx, ny, nz, nxp, G, sc.err_theta_cov, Sm, Smd, scale,
                                                 want_sigmamd=True)
    P = [torch.from_numpy(p).cuda() for p in post]
    M = [torch.from_numpy(np.ascontiguousarray(m)).cuda() for m in sc.mean]
    ns = torch.from_numpy(np.ascontiguousarray(scale)).cuda()
    smd = torch.empty((ny, nx, 9), dtype=torch.float64, device="cuda")
    api.correct_alpha_beta_rho(P, M, nx, ny, nz, nxp, G, sc.err_theta_cov, Sm, Smd, ns, smd)
    torch.cuda.synchronize()
    got = [p.cpu().numpy() for p in P]
    for p in range(3):
        upd_ref = ref[p][:nz, :ny, :nx] - sc.mean[p][:nz, :ny, :nx]
        upd = got[p][:nz, :ny, :nx] - sc.mean[p][:nz, :ny, :nx]
        e = rel(upd, upd_ref)
        print(n, dims, p, "update vs oracle", e, "max abs", np.abs(got[p] - ref[p]).max())
        assert e < 1e-6
        assert np.array_equal(got[p][nz:], post[p][nz:]) and np.array_equal(got[p][:, :, nx:], post[p][:, :, nx:])
    assert np.abs(smd.cpu().numpy() - smd_ref).max() < 1e-9 * np.abs(smd_ref).max()


def test_apply_trace_matrices(cuda):
    from crava_gb300 import api
    rng = np.random.default_rng(4)
    nx, ny, nz, nxp, nyp, nzp = 13, 11, 17, 16, 14, 20
    _, rnxp = api.dims(nxp)
    f = [rng.standard_normal((nzp, nyp, rnxp)).astype(np.float32) for _ in range(3)]
    mu = [rng.standard_normal((nzp, nyp, rnxp)).astype(np.float32) for _ in range(3)]
    mats = rng.standard_normal((ny, nx, 9))
    F = [torch.from_numpy(x).cuda() for x in f]
    api.apply_trace_matrices(F, torch.from_numpy(mats).cuda(), nx, ny, nz, nxp,
                             mean=[torch.from_numpy(x).cuda() for x in mu])
    got = np.stack([x.cpu().numpy() for x in F])
    want = np.stack(f).astype(np.float64)
    x = want[:, :nz, :ny, :nx].copy()
    M = mats.reshape(ny, nx, 3, 3)
    want[:, :nz, :ny, :nx] = np.einsum("jipq,qkji->pkji", M, x).astype(np.float32)
    want = (want.astype(np.float32) + np.stack(mu))
    assert np.abs(got[:, :, :, :nxp] - want[:, :, :, :nxp]).max() < 1e-5


def test_local_noise_after_inversion(cuda, oracle):
    """The pipeline order of the reference: inversion, output grids (postVar0), correctAlphaBetaRho."""
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    # the reference makes the lateral correlation positive definite (makeCorr2DPositiveDefinite), so the
    # prior variance at the origin is Sigma0 and Sigma0 - postVar0 is positive semi-definite
    sc = S.make_scenario(24, 20, 32, [5.0, 15.0, 25.0, 35.0], 28.0, nxp=30, nyp=24, nzp=40, seed=21, pd_corr_xy=True)
    inv = Inversion(sc, forms=("mixed",))
    inv.restore("mixed")
    inv.run("mixed")
    pv0, _, _ = inv.outputs("mixed")
    pv0 = np.asarray(pv0, dtype=np.float64)
    post = [m.cpu().numpy().copy() for m in inv.mean]
    yy, xx = np.mgrid[0:sc.ny, 0:sc.nx]
    scale = np.stack([1.0 + 0.5 * (1 + np.sin(xx / 4.0 + l) * np.cos(yy / 5.0)) for l in range(sc.ntheta)])
    smd = inv.correct_local_noise("mixed", torch.from_numpy(scale).cuda(), pv0)
    torch.cuda.synchronize()
    from crava_gb300 import api
    G = api.local_noise_g(sc.err_theta_cov, sc.sigma0, pv0)
    ref, smd_ref = oracle.correct_alpha_beta_rho(post, sc.mean, sc.nx, sc.ny, sc.nz, sc.nxp, G, sc.err_theta_cov,
                                                 sc.sigma0, pv0, scale, want_sigmamd=True)
    for p in range(3):
        got = inv.mean[p].cpu().numpy()
        e = rel(got - sc.mean[p], ref[p] - sc.mean[p])
        print("pipeline local noise", p, e)
        assert e < 1e-6
    assert np.abs(smd.cpu().numpy() - smd_ref).max() < 1e-9 * np.abs(smd_ref).max()
