"""The GPU path against the reference's own compiled Crava and State4D code.

The fixtures were written by crava_o2 (oracle/o2_harness.cpp), which runs the
reference's Wavelet, SeismicParametersHolder, Crava::computePostMeanResidAndFFTCov
and State4D::merge / ::split compiled from its sources (tests/golden/make_golden.py).
The GPU starts from the same real-domain cubes, wavelets, correlation surfaces and
model parameters, builds its own tables and transforms, and is held to the
reference's outputs at FP32 tolerances.
"""
import numpy as np
import pytest
import torch

from conftest import from_cube, golden, rel, to_cube

pytestmark = pytest.mark.gpu

CASES = ["inversion_c0small.npz", "inversion_c1small.npz", "inversion_n8odd.npz", "inversion_grad.npz"]


def _scenario(g):
    from crava_gb300 import synthetic as S
    return S.Scenario(nx=int(g["nx"]), ny=int(g["ny"]), nz=int(g["nz"]), nxp=int(g["nxp"]), nyp=int(g["nyp"]),
                      nzp=int(g["nzp"]), dt_ms=float(g["dt_ms"]), theta_deg=list(g["theta_deg"]), A=g["A"],
                      wavelets=g["wavelets"], corr_xy=g["corr_xy"], circ_corr_t=g["circ_corr_t"],
                      sigma0=g["sigma0"], err_theta_cov=g["err_theta_cov"], data=list(g["data_real"]),
                      mean=list(g["mean_real"]), wnc=float(g["wnc"]), low_cut=float(g["low_cut"]),
                      high_cut=float(g["high_cut"]),
                      corr_grad=tuple(float(x) for x in g["corr_grad"]) if "corr_grad" in g else (0.0, 0.0))


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("form", ["plain", "fp32", "mixed", "mixed_cold"])
def test_gpu_inversion_matches_reference_crava(cuda, case, form):
    """Posterior mean (real cubes), residual and posterior covariance spectra of the GPU inversion from the
    real-domain inputs, against Crava::computePostMeanResidAndFFTCov run by the reference's own code.  The
    plain form is the reference's dataflow (covariance cubes filled and transformed); the fused forms
    rebuild the separable prior spectra; mixed_cold sets the model up inside the call."""
    from crava_gb300.pipeline import Inversion
    g = golden(case)
    sc = _scenario(g)
    base = "mixed" if form == "mixed_cold" else form
    inv = Inversion(sc, forms=(base,))
    inv.restore(base)
    inv.ws.reset_stats()
    if form == "mixed_cold":
        inv.run_cold("mixed")
    else:
        inv.run(base)
    torch.cuda.synchronize()
    pm, res, cov = inv.results(base)
    nxp = sc.nxp
    prior = g["mean_real"][..., :nxp]
    ref = g["crava_mean_real"][..., :nxp]
    e = (rel(pm, ref), rel(pm - prior, ref - prior), rel(res, g["crava_resid"]), rel(cov, g["crava_cov"]))
    print(case, form, "GPU vs reference Crava (mean, update, resid, cov):", e, inv.ws.stats())
    assert e[0] < 1e-6 and e[1] < 2e-4 and e[2] < 2e-5 and e[3] < 2e-5
    assert inv.ws.stats()["failed"] == int(g["nfail"])


def test_gpu_state4d_merge_and_split_match_reference(cuda):
    """cg_state4d_merge / cg_state4d_split against State4D::merge / ::split of the reference."""
    from crava_gb300 import api
    g = golden("state4d_n4.npz")
    nxp = int(g["nxp"])
    st = [to_cube(x) for x in g["state"]]
    grp = [st[0:3], st[3:6], st[6:12], st[12:21], st[21:27]]
    mu_cur = [torch.empty_like(st[0]) for _ in range(3)]
    cov_cur = [torch.empty_like(st[0]) for _ in range(6)]
    api.state4d_merge(*grp, mu_cur, cov_cur, nxp)
    torch.cuda.synchronize()
    merged = np.stack([from_cube(x) for x in mu_cur + cov_cur])
    e_merge = rel(merged, g["merged"])
    post = [to_cube(x) for x in g["post"]]
    nfail = api.state4d_split(*grp, post[:3], post[3:], nxp)
    torch.cuda.synchronize()
    split = np.stack([from_cube(x) for x in st])
    e_split = rel(split, g["split"])
    print("GPU State4D vs reference: merge", e_merge, "split", e_split, "kept prior", int(nfail.item()))
    assert e_merge < 1e-7
    assert e_split < 2e-5


def test_gpu_local_noise_correction_matches_reference(cuda):
    """cg_correct_alpha_beta_rho with the reference's G against Crava::correctAlphaBetaRho run by the reference's
    own code: every trace but the RMISSING one (NaN in the reference, the minimum scale here)."""
    from crava_gb300 import api
    g = golden("reference_localnoise.npz")
    nx, ny, nz, nxp = (int(g[k]) for k in ("nx", "ny", "nz", "nxp"))
    P = [torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in g["post"]]
    M = [torch.from_numpy(np.ascontiguousarray(m)).cuda() for m in g["mean"]]
    ns = torch.from_numpy(np.ascontiguousarray(g["scale"])).cuda()
    api.correct_alpha_beta_rho(P, M, nx, ny, nz, nxp, g["G"], g["err_theta_cov"], g["prior_var0"], g["post_var0"], ns)
    torch.cuda.synchronize()
    miss = np.zeros(g["out"][0].shape, bool)
    jj, ii = np.nonzero((g["scale"] == -99999.0).any(axis=0))
    miss[:nz, jj, ii] = True
    for p in range(3):
        got, ref, mean = P[p].cpu().numpy(), g["out"][p], g["mean"][p]
        e = rel(got[~miss] - mean[~miss], ref[~miss] - mean[~miss])
        print("local-noise correction vs reference, parameter", p, ": update rel", e,
              "max abs", np.abs(got[~miss] - ref[~miss]).max())
        assert e < 1e-6
        assert np.isfinite(got[miss]).all()


@pytest.mark.parametrize("kind", ["data", "param"])
def test_gpu_fill_in_data_matches_reference(cuda, kind):
    """cg_fill_in_data fed the per-column traces and geometry of the reference's own fillInData run (crava_o2)
    against the cube that run produced."""
    from crava_gb300 import api
    g = golden("reference_fillindata.npz")
    nx, ny, nz, nxp, nyp, nzp = (int(g[k]) for k in ("nx", "ny", "nz", "nxp", "nyp", "nzp"))
    st = g[f"{kind}_state"]
    dz_data = float(np.unique(g[f"{kind}_dz_data"][st == 0])[0])
    _, rnxp = api.dims(nxp)
    buf = torch.full((nzp, nyp, rnxp), 7.0, device="cuda")
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    api.fill_in_data(buf, nxp, nz, api.DATA if kind == "data" else api.PARAMETER, dev(g[f"{kind}_traces"]),
                     dev(st.astype(np.uint8)), dev(g[f"{kind}_z0_data"]), dev(g[f"{kind}_z0_grid"]),
                     dev(g[f"{kind}_dz_grid"]), dz_data, float(g["smooth_length"]))
    got = buf.cpu().numpy()
    e = rel(got, g[f"{kind}_cube"])
    print("fillInData", kind, "GPU vs reference:", e)
    assert e < 2e-6


@pytest.mark.parametrize("threshold", [0.0, 0.3])
def test_gpu_interpolate_seismic_bit_exact_vs_reference(cuda, threshold):
    """cg_interpolate_seismic against FFTGrid::interpolateSeismic run by the reference's own code: bit for bit."""
    from crava_gb300 import api
    g = golden("reference_interpolate.npz")
    nx, ny, nz, nxp = (int(g[k]) for k in ("nx", "ny", "nz", "nxp"))
    t = torch.from_numpy(np.ascontiguousarray(g["cube"])).cuda()
    api.interpolate_seismic(t, nx, ny, nz, nxp, threshold)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(t.cpu().numpy(), g[f"out_{threshold:g}"])


def test_gpu_scale_wavelet_division_matches_reference(cuda):
    """cg_scale_wavelet_tables + cg_divide_by_scale_wavelet (with interpolateSeismic) against
    Crava::divideDataByScaleWavelet run by the reference's own code on a simbox of non-constant thickness, with the
    wavelets and gain grids as the reference's Wavelet::setGainGrid leaves them."""
    from crava_gb300 import api
    g = golden("reference_divide.npz")
    nx, ny, nz, nxp = (int(g[k]) for k in ("nx", "ny", "nz", "nxp"))
    dt, lz = float(g["dt_ms"]), float(g["lz"])
    s0 = np.asarray(g["sigma0"]).astype(np.float32).astype(np.float64)
    tab = api.scale_wavelet_tables(g["wavelets"], g["A"], s0, g["corr_t_filtered"], g["err_theta_cov"], nz, dt, lz,
                                   float(g["low_cut"]), float(g["high_cut"]), float(g["wnc"]))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()  # noqa: E731
    cubes = [dev(x) for x in g["data"]]
    nbad = api.divide_by_scale_wavelet(cubes, nx, ny, nz, nxp, dev(tab), dev(g["rel_thick"]), dt, lz,
                                       float(g["low_cut"]), float(g["high_cut"]), 0.0, shift=dev(g["shift"]),
                                       gain=dev(g["gain_normalised"]))
    assert nbad == [2, 2, 2]
    for l, c in enumerate(cubes):
        e = rel(c.cpu().numpy()[..., :nxp], g["out"][l][..., :nxp])
        print("scale-wavelet division, angle", l, "GPU vs reference:", e)
        assert e < 2e-5


def test_gpu_scale_wavelet_multiply_matches_reference(cuda):
    """cg_multiply_by_scale_wavelet on the reference's divided cubes against the reference's own
    multiplyDataByScaleWaveletAndWriteToFile product (crava_o2, the same cubes after their forward transform)."""
    from crava_gb300 import api
    g = golden("reference_divide.npz")
    nx, ny, nz, nxp = (int(g[k]) for k in ("nx", "ny", "nz", "nxp"))
    dt, lz = float(g["dt_ms"]), float(g["lz"])
    s0 = np.asarray(g["sigma0"]).astype(np.float32).astype(np.float64)
    tab = api.scale_wavelet_tables(g["wavelets"], g["A"], s0, g["corr_t_filtered"], g["err_theta_cov"], nz, dt, lz,
                                   float(g["low_cut"]), float(g["high_cut"]), float(g["wnc"]))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()  # noqa: E731
    cubes = [dev(x) for x in g["out"]]
    api.multiply_by_scale_wavelet(cubes, nx, ny, nxp, dev(tab), dev(g["rel_thick"]), dt, shift=dev(g["shift"]),
                                  gain=dev(g["gain_normalised"]))
    torch.cuda.synchronize()
    for l, c in enumerate(cubes):
        e = rel(c.cpu().numpy()[..., :nxp], g["mult"][l][..., :nxp])
        print("scale-wavelet multiply, angle", l, "GPU vs reference:", e)
        assert e < 2e-5
