"""Output grids after the bin loop: covariance and residual grids back to the real domain, postVar0 and
postCov00, and exp() of the posterior means (fused into the inverse transform or stand-alone)."""
import numpy as np
import pytest
import torch

from conftest import rel

pytestmark = pytest.mark.gpu

EXP_TOL = 4e-7   # elementwise relative: expf is within 2 ulp of the correctly rounded exp


def test_inversion_outputs_match_oracle(cuda, oracle):
    from crava_gb300 import api, synthetic as S
    from crava_gb300.pipeline import Inversion
    sc = S.scaled_config1(48, 40, 64, seed=21)
    inv = Inversion(sc, forms=("mixed",))
    inv.restore("mixed")
    inv.run("mixed")
    torch.cuda.synchronize()
    cov_spec = [api.as_spectrum(c).cpu().numpy().copy() for c in inv.cov]
    res_spec = [api.as_spectrum(d).cpu().numpy().copy() for d in inv.data]
    mean = [m.cpu().numpy().copy() for m in inv.mean]
    v0, c00, elastic = inv.outputs("mixed")
    torch.cuda.synchronize()
    cov_real = [oracle.fft3d_c2r(c, sc.nxp, oracle.COVARIANCE, "d") for c in cov_spec]
    res_real = [oracle.fft3d_c2r(r, sc.nxp, oracle.DATA, "d") for r in res_spec]
    # covariance and residual grids in the real domain
    got_cov = np.stack([c[:, :, :sc.nxp].cpu().numpy() for c in inv.cov])
    assert rel(got_cov, np.stack([c[:, :, :sc.nxp] for c in cov_real])) < 2e-6
    got_res = np.stack([d[:, :, :sc.nxp].cpu().numpy() for d in inv.data])
    assert rel(got_res, np.stack([r[:, :, :sc.nxp] for r in res_real])) < 2e-6
    # postVar0 from the lag-0 values (order 00 11 22 01 02 12), postCov00 from (0,0,k)
    o = [c[0, 0, 0] for c in got_cov]
    ref_v0 = np.array([[o[0], o[3], o[4]], [o[3], o[1], o[5]], [o[4], o[5], o[2]]])
    np.testing.assert_array_equal(v0, ref_v0)
    np.testing.assert_array_equal(c00, got_cov[:3, :sc.nz, 0, 0])
    o64 = [c[0, 0, 0] for c in cov_real]
    ref64 = np.array([o64[i] for i in (0, 3, 4, 3, 1, 5, 4, 5, 2)]).reshape(3, 3)
    assert np.abs(v0 - ref64).max() < 1e-5 * np.abs(v0).max()
    # exp of the posterior means: every float of the cube (padding included), RMISSING kept
    for m, e in zip(mean, elastic):
        ref = np.exp(m.astype(np.float64))
        assert np.max(np.abs(e.cpu().numpy() - ref) / ref) < EXP_TOL


def test_fused_inverse_exp_equals_inverse_then_exp(cuda):
    from crava_gb300 import api
    for n in ((256, 64, 40), (90, 50, 36), (245, 21, 16)):   # four-step rows, generic even, generic odd
        nxp, nyp, nzp = n
        _, rnxp = api.dims(nxp)
        g = torch.Generator(device="cuda").manual_seed(nxp)
        x = torch.randn((nzp, nyp, rnxp), device="cuda", generator=g) * 0.1
        api.fft_in_place(x, nxp, api.PARAMETER)
        a, b = x.clone(), x.clone()
        api.inv_fft_in_place(a, nxp, api.PARAMETER)
        api.exp_transform(a)
        api.inv_fft_exp_batch([b], nxp, api.PARAMETER)
        torch.cuda.synchronize()
        A, B = a[..., :nxp].cpu().numpy(), b[..., :nxp].cpu().numpy()
        assert np.max(np.abs(A - B) / np.abs(A)) < 1e-6, n


def test_exp_log_transform_semantics(cuda):
    from crava_gb300 import api
    v = torch.tensor([0.0, 1.0, -2.5, -99999.0, 8.0, 3.0, -1.0, 0.5, 2.0], device="cuda")
    e = v.clone()
    api.exp_transform(e)
    ref = np.where(v.cpu().numpy() == -99999.0, -99999.0, np.exp(v.cpu().numpy().astype(np.float64)))
    assert np.max(np.abs(e.cpu().numpy() - ref) / np.abs(ref)) < EXP_TOL
    l = torch.tensor([1.0, 2.718281828, -3.0, 0.0, -99999.0, 10.0, 1e-3, 5.0, 7.0], device="cuda")
    lt = l.clone()
    api.log_transform(lt)
    lv = l.cpu().numpy()
    ref = np.where((lv == -99999.0) | (lv <= 0), 0.0, np.log(np.where(lv > 0, lv, 1.0)))
    assert np.max(np.abs(lt.cpu().numpy() - ref)) < 1e-6
