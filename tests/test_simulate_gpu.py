"""Posterior simulation on the GPU against the reference's RandomGen noise and lib_matr."""
import numpy as np
import pytest
import torch

from conftest import from_cube, golden, rel, to_cube

pytestmark = pytest.mark.gpu


def test_injected_noise_matches_reference(cuda):
    """The reference's own noise (RandomGen + fillInComplexNoise) through the GPU factor/apply/C2R."""
    from crava_gb300 import api
    inv = golden("inversion_c0small.npz")
    sim = golden("simulation_c0small.npz")
    nxp, nyp, nzp = int(inv["nxp"]), int(inv["nyp"]), int(inv["nzp"])
    cov = [to_cube(c) for c in inv["out_cov"]]
    chol, nfail = api.posterior_cholesky(cov, nxp)
    noise = [to_cube(n) for n in sim["noise"]]
    fields = [torch.empty_like(cov[0]) for _ in range(3)]
    api.simulate_fields(chol, fields, nxp, noise=noise)
    torch.cuda.synchronize()
    got = np.stack([f.cpu().numpy()[..., :nxp] for f in fields])
    e = rel(got, sim["sim_real"][..., :nxp])
    print("simulated fields vs reference:", e, "failed factors:", int(nfail.item()))
    assert e < 1e-5


def test_mean_is_added_and_spectra_match_oracle(cuda, oracle):
    from crava_gb300 import api
    inv = golden("inversion_c1small.npz")
    nxp, nyp, nzp = int(inv["nxp"]), int(inv["nyp"]), int(inv["nzp"])
    noise = oracle.fill_complex_noise(nxp, nyp, nzp, 777, 3)
    z = oracle.simulate_bins(list(inv["out_cov"]), list(noise), prec="d")
    ref = np.stack([oracle.fft3d_c2r(x, nxp, oracle.PARAMETER, "d")[..., :nxp] for x in z])
    ref += inv["out_mean_real"][..., :nxp]
    cov = [to_cube(c) for c in inv["out_cov"]]
    chol, _ = api.posterior_cholesky(cov, nxp)
    fields = [torch.empty_like(cov[0]) for _ in range(3)]
    mean = [torch.from_numpy(m.copy()).cuda() for m in inv["out_mean_real"]]
    api.simulate_fields(chol, fields, nxp, noise=[to_cube(n) for n in noise], post_mean=mean)
    torch.cuda.synchronize()
    got = np.stack([f.cpu().numpy()[..., :nxp] for f in fields])
    dev = got - inv["out_mean_real"][..., :nxp]
    e = rel(dev, ref - inv["out_mean_real"][..., :nxp])
    print("simulated deviations vs FP64 oracle:", e)
    assert e < 1e-5


def test_generated_noise_statistics_and_structure(cuda):
    """Counter-based noise: unit variance, zero mean, Hermitian x=0 plane, reproducible."""
    from crava_gb300 import api
    nxp, nyp, nzp = 64, 48, 40
    cnxp = nxp // 2 + 1
    # identity posterior covariance -> L = I, so the fields' spectra are the noise itself
    ones = torch.zeros((nzp, nyp, 2 * cnxp), device="cuda")
    ones.view(nzp, nyp, cnxp, 2)[..., 0] = 1.0
    zero = torch.zeros_like(ones)
    chol, nf = api.posterior_cholesky([ones, ones, ones, zero, zero, zero], nxp)
    assert int(nf.item()) == 0

    def noise_spectra(seed, r):
        f = [torch.empty_like(ones) for _ in range(3)]
        # reproduce the apply step only: run with the add disabled and read the spectra back by a forward transform
        api.simulate_fields(chol, f, nxp, seed=seed, real0=r)
        for x in f:
            api.fft_in_place(x, nxp, api.PARAMETER)
        return np.stack([from_cube(x) for x in f])

    a = noise_spectra(1234, 0)
    b = noise_spectra(1234, 0)
    c = noise_spectra(1234, 1)
    assert rel(a, b) < 1e-6          # same (seed, realisation) -> same field
    assert rel(a, c) > 0.5           # different realisation -> independent
    inner = a[:, :, :, 1:cnxp - 1]
    assert abs(float(np.mean(np.abs(inner) ** 2)) - 1.0) < 0.02
    assert abs(float(np.mean(inner.real))) < 0.01
    # x=0 plane is Hermitian in (j, k) after the round trip
    p0 = a[:, :, :, 0]
    jr = (-np.arange(nyp)) % nyp
    kr = (-np.arange(nzp)) % nzp
    mirror = np.conj(p0[:, kr][:, :, jr])
    assert rel(p0, mirror) < 1e-5


def test_many_realisations_batched_equal_single(cuda):
    from crava_gb300 import api
    inv = golden("inversion_c0small.npz")
    nxp = int(inv["nxp"])
    cov = [to_cube(c) for c in inv["out_cov"]]
    chol, _ = api.posterior_cholesky(cov, nxp)
    nreal = 7
    fields = [torch.empty_like(cov[0]) for _ in range(3 * nreal)]
    api.simulate_fields(chol, fields, nxp, seed=99, real0=0)
    for r in (0, 3, 6):
        single = [torch.empty_like(cov[0]) for _ in range(3)]
        api.simulate_fields(chol, single, nxp, seed=99, real0=r)
        for p in range(3):
            assert torch.equal(single[p], fields[3 * r + p])
