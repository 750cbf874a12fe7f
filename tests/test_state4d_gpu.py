"""4D time-lapse merge / invert / split on the GPU against the oracle (State4D restated)."""
import numpy as np
import pytest
import torch

from conftest import from_cube, rel, to_cube

pytestmark = pytest.mark.gpu


def random_state(nxp, nyp, nzp, seed):
    """A 6-parameter prior per bin: Hermitian positive definite 6x6 spectra and means."""
    rng = np.random.default_rng(seed)
    cnxp = nxp // 2 + 1
    shp = (nzp, nyp, cnxp)
    G = rng.standard_normal(shp + (6, 6)) + 1j * rng.standard_normal(shp + (6, 6))
    F = np.einsum("...ik,...jk->...ij", G, np.conj(G)) / 6 + 0.5 * np.eye(6)
    scale = np.array([0.10, 0.07, 0.05, 0.03, 0.02, 0.02])
    F = F * scale[:, None] * scale[None, :]
    ssi = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    sdi = [(0, 3), (0, 4), (0, 5), (1, 3), (1, 4), (1, 5), (2, 3), (2, 4), (2, 5)]
    ddi = [(3, 3), (3, 4), (3, 5), (4, 4), (4, 5), (5, 5)]
    ss = [F[..., i, j].astype(np.complex64) for i, j in ssi]
    sd = [F[..., i, j].astype(np.complex64) for i, j in sdi]
    dd = [F[..., i, j].astype(np.complex64) for i, j in ddi]
    mu = [(rng.standard_normal(shp) + 1j * rng.standard_normal(shp)).astype(np.complex64) * 0.1 for _ in range(6)]
    return mu[:3], mu[3:], ss, sd, dd


def test_merge_matches_oracle(cuda, oracle):
    from crava_gb300 import api
    nxp, nyp, nzp = 20, 12, 14
    mu_s, mu_d, ss, sd, dd = random_state(nxp, nyp, nzp, 1)
    ref_mu, ref_cov = oracle.state4d_merge(mu_s, mu_d, ss, sd, dd, prec="f")
    g = [[to_cube(x) for x in grp] for grp in (mu_s, mu_d, ss, sd, dd)]
    mu_cur = [torch.empty_like(g[0][0]) for _ in range(3)]
    cov_cur = [torch.empty_like(g[0][0]) for _ in range(6)]
    api.state4d_merge(*g, mu_cur, cov_cur, nxp)
    torch.cuda.synchronize()
    assert rel(np.stack([from_cube(x) for x in mu_cur]), np.stack(ref_mu)) == 0
    assert rel(np.stack([from_cube(x) for x in cov_cur]), np.stack(ref_cov)) < 1e-7


def test_split_matches_oracle(cuda, oracle):
    from crava_gb300 import api
    nxp, nyp, nzp = 20, 12, 14
    mu_s, mu_d, ss, sd, dd = random_state(nxp, nyp, nzp, 2)
    mu_cur, cov_cur = oracle.state4d_merge(mu_s, mu_d, ss, sd, dd, prec="d")
    # a posterior of the current state: shrink the prior covariance, move the mean
    cov_post = [(c * 0.6).astype(np.complex64) for c in cov_cur]
    mu_post = [(m + 0.01).astype(np.complex64) for m in mu_cur]
    (rs, rd, rss, rsd, rdd), nf = oracle.state4d_split(mu_s, mu_d, ss, sd, dd, mu_post, cov_post, prec="d")
    g = [[to_cube(x) for x in grp] for grp in (mu_s, mu_d, ss, sd, dd)]
    nfail = api.state4d_split(*g, [to_cube(x) for x in mu_post], [to_cube(x) for x in cov_post], nxp)
    torch.cuda.synchronize()
    got = [np.stack([from_cube(x) for x in grp]) for grp in g]
    ref = [np.stack(x) for x in (rs, rd, rss, rsd, rdd)]
    errs = [rel(a, b) for a, b in zip(got, ref)]
    print("split vs FP64 oracle:", errs, "fails", int(nfail.item()), nf)
    assert int(nfail.item()) == nf == 0
    assert max(errs) < 2e-5
