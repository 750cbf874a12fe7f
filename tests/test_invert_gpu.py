"""GPU per-bin posterior against the reference's own FP32 outputs and the FP64 oracle."""
import numpy as np
import pytest
import torch

from conftest import from_cube, golden, oracle_pipeline, rel, to_cube

pytestmark = pytest.mark.gpu


def _ws_from_golden(g, cond_threshold=0.0):
    from crava_gb300 import api
    n = len(g["theta_deg"])
    ws = api.Workspace(int(g["nxp"]), int(g["nyp"]), int(g["nzp"]), n)
    tab = {k: g[k] for k in ("K", "em1", "em2", "em3", "band")}
    ws.set_model(tab, g["err_theta_cov"], g["sigma0"], float(g["wnc"]), cond_threshold=cond_threshold)
    return ws


@pytest.mark.parametrize("case", ["inversion_c0small.npz", "inversion_c1small.npz", "inversion_n8odd.npz",
                                  "inversion_grad.npz"])
def test_plain_matches_reference_lib_matr(cuda, case):
    """Same input spectra as the reference run -> same posterior (FP32 vs FP32)."""
    g = golden(case)
    ws = _ws_from_golden(g)
    data = [to_cube(x) for x in g["data_spec"]]
    mean = [to_cube(x) for x in g["mean_spec"]]
    cov = [to_cube(x) for x in g["cov_spec"]]
    ec = to_cube(g["errcorr_spec"])
    ws.reset_stats()
    ws.invert_plain(data, mean, cov, ec)
    torch.cuda.synchronize()
    res = np.stack([from_cube(x) for x in data])
    mu = np.stack([from_cube(x) for x in mean])
    cv = np.stack([from_cube(x) for x in cov])
    upd, upd_ref = mu - g["mean_spec"], g["out_mean"] - g["mean_spec"]
    e_upd, e_res, e_cov = rel(upd, upd_ref), rel(res, g["out_resid"]), rel(cv, g["out_cov"])
    print(case, "plain vs reference: update", e_upd, "resid", e_res, "cov", e_cov)
    assert e_upd < 1e-4 and e_res < 1e-5 and e_cov < 1e-5
    assert ws.stats()["failed"] == int(g["nfail"])


@pytest.mark.parametrize("case", ["inversion_c0small.npz", "inversion_c1small.npz", "inversion_n8odd.npz",
                                  "inversion_grad.npz"])
@pytest.mark.parametrize("form", ["fp32", "mixed"])
def test_fused_matches_fp64_oracle_on_reference_inputs(cuda, oracle, case, form):
    """Fused kernel (prior regenerated from the separable spectra, or from the per-bin table when the
    correlation gradients are nonzero) vs the FP64 restatement."""
    from crava_gb300 import api
    g = golden(case)
    ws = _ws_from_golden(g)
    nxp, nyp, nzp = int(g["nxp"]), int(g["nyp"]), int(g["nzp"])
    gi, gj = (float(x) for x in g["corr_grad"]) if "corr_grad" in g else (0.0, 0.0)
    corr_xy = torch.from_numpy(g["corr_xy"].astype(np.float32)).cuda()
    circ = torch.from_numpy(g["circ_corr_t"].astype(np.float32)).cuda()
    ws.prior_spectra(corr_xy, circ, api.PREC_FP32, grad=(gi, gj))
    data = [to_cube(x) for x in g["data_spec"]]
    mean = [to_cube(x) for x in g["mean_spec"]]
    cov = [to_cube(np.zeros_like(x)) for x in g["cov_spec"]]
    ws.reset_stats()
    ws.invert_fused(data, mean, cov, api.PREC_MIXED if form == "mixed" else api.PREC_FP32)
    torch.cuda.synchronize()
    # FP64 oracle on the same input spectra, prior spectra from FP64 transforms of the filled cubes
    covs = []
    s0f = g["sigma0"].astype(np.float32).astype(np.float64)
    for (p, q) in [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]:
        c = oracle.fill_param_corr(nxp, nyp, nzp, g["corr_xy"], g["circ_corr_t"], gi, gj, float(s0f[p, q]),
                                   prec="d")
        covs.append(oracle.fft3d_r2c(c, nxp, oracle.COVARIANCE, "d"))
    ec = oracle.fft3d_r2c(oracle.fill_err_corr(nxp, nyp, nzp, g["corr_xy"], gi, gj, prec="d"), nxp,
                          oracle.COVARIANCE, "d")
    tab = {k: g[k].astype(np.complex128) if g[k].dtype == np.complex64 else g[k] for k in ("K", "em1", "em2", "em3", "band")}
    tab["nxp"] = nxp
    r64, m64, c64, _ = oracle.invert_bins(list(g["data_spec"].astype(np.complex128)),
                                          list(g["mean_spec"].astype(np.complex128)), covs, ec, tab,
                                          g["err_theta_cov"], s0f, float(g["wnc"]), prec="d")
    mu = np.stack([from_cube(x) for x in mean])
    res = np.stack([from_cube(x) for x in data])
    cv = np.stack([from_cube(x) for x in cov])
    e_upd = rel(mu - g["mean_spec"], np.stack(m64) - g["mean_spec"])
    e_res = rel(res, np.stack(r64))
    e_cov = rel(cv, np.stack(c64))
    print(case, form, "vs FP64 oracle: update", e_upd, "resid", e_res, "cov", e_cov, ws.stats())
    assert e_upd < 1e-4 and e_res < 1e-5 and e_cov < 1e-4


@pytest.mark.parametrize("form", ["plain", "fp32", "mixed", "fp64", "mixed_3pass"])
def test_pipeline_matches_fp64_oracle(cuda, oracle, form):
    """Whole inversion from real-domain cubes (config-1 physics on a 40x36x48 cube)."""
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    sc = S.scaled_config1(40, 36, 48, seed=21)
    inv = Inversion(sc, forms=(form,))
    inv.restore(form)
    inv.run(form)
    torch.cuda.synchronize()
    pm, res, cov = inv.results(form)
    post64, res64, cov64, _ = oracle_pipeline(oracle, sc, "d", tables=inv.tables)
    prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
    e_mean = rel(pm, post64)
    e_upd = rel(pm - prior, post64 - prior)
    e_res = rel(res, res64)
    e_cov = rel(cov, cov64)
    print(form, "pipeline vs FP64 oracle: mean", e_mean, "update", e_upd, "resid", e_res, "cov", e_cov)
    tol = 1e-10 if form == "fp64" else 1e-4
    assert e_mean < (1e-12 if form == "fp64" else 1e-6)
    assert e_upd < tol and e_res < tol and e_cov < tol


# y lengths with the fused y-transform + bin-loop kernel (cg_invert_cubes_fused), tail x tiles included
@pytest.mark.parametrize("dims,cond", [((64, 128, 48), 0.0), ((40, 200, 32), 0.0), ((48, 256, 24), 0.0),
                                       ((64, 128, 48), 1.0001), ((30, 256, 20), 1.0001)])
def test_fused_y_kernel_matches_fp64_oracle(cuda, oracle, dims, cond):
    """cond = 1.0001 sends almost every in-band bin through the in-kernel FP64 path."""
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    from crava_gb300 import _native
    nxp, nyp, nzp = dims
    sc = S.scaled_config1(nxp, nyp, nzp, seed=nyp + nzp)
    inv = Inversion(sc, forms=("mixed",), cond_threshold=cond)
    inv.restore("mixed")
    inv.ws.reset_stats()
    L = _native.lib()
    assert L.cg_tune_set(4, nyp, 1) == 0   # CG_TUNE_FUSED_Y on for this y length
    try:
        inv.run("mixed")
        torch.cuda.synchronize()
    finally:
        L.cg_tune_clear()
        _native._apply_tuning(L)
    st = inv.ws.stats()
    pm, res, cov = inv.results("mixed")
    post64, res64, cov64, _ = oracle_pipeline(oracle, sc, "d", tables=inv.tables)
    prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
    e = (rel(pm, post64), rel(pm - prior, post64 - prior), rel(res, res64), rel(cov, cov64))
    print(dims, cond, "fused y kernel vs FP64 oracle (mean, update, resid, cov):", e, st)
    assert e[0] < 1e-6 and e[1] < 1e-4 and e[2] < 1e-4 and e[3] < 1e-4
    inband = int(inv.tables["band"].sum()) * sc.cnxp * sc.nyp
    if cond > 0:
        assert st["flagged"] > inband // 2   # the FP64 path ran for most in-band bins
    else:
        assert st["flagged"] == 0


# forward y pass, bins and inverse y pass per chunk of z-planes (CG_TUNE_FUSED_Y = even chunk size), with a
# short last chunk and, at cond = 1.0001, a FP64 fix-up queue that grows over the chunks
@pytest.mark.parametrize("dims,chunk,cond,form", [((64, 128, 48), 16, 0.0, "fp32"), ((40, 200, 36), 16, 0.0, "mixed"),
                                                  ((48, 256, 24), 10, 1.0001, "mixed"),
                                                  ((30, 120, 20), 4, 1.0001, "mixed"),
                                                  ((64, 128, 48), 64, 0.0, "mixed")])
def test_chunked_y_pipeline_matches_fp64_oracle(cuda, oracle, dims, chunk, cond, form):
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    from crava_gb300 import _native
    nxp, nyp, nzp = dims
    sc = S.scaled_config1(nxp, nyp, nzp, seed=nyp + nzp + chunk)
    inv = Inversion(sc, forms=(form,), cond_threshold=cond)
    inv.restore(form)
    inv.ws.reset_stats()
    L = _native.lib()
    assert L.cg_tune_set(4, nyp, chunk) == 0
    try:
        inv.run(form)
        torch.cuda.synchronize()
    finally:
        L.cg_tune_clear()
        _native._apply_tuning(L)
    st = inv.ws.stats()
    pm, res, cov = inv.results(form)
    post64, res64, cov64, _ = oracle_pipeline(oracle, sc, "d", tables=inv.tables)
    prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
    e = (rel(pm, post64), rel(pm - prior, post64 - prior), rel(res, res64), rel(cov, cov64))
    print(dims, chunk, cond, form, "chunked y pipeline vs FP64 oracle (mean, update, resid, cov):", e, st)
    assert e[0] < 1e-6 and e[1] < 1e-4 and e[2] < 1e-4 and e[3] < 1e-4
    inband = int(inv.tables["band"].sum()) * sc.cnxp * sc.nyp
    if cond > 0:
        assert st["flagged"] > inband // 2
        # queued bins are written by the fix-up alone: a chunk whose entries it missed, or whose means it
        # rewrote after their inverse y pass, would fail the comparison above
        csize = sc.cnxp * sc.nyp * sc.nzp
        if min(csize, max(1 << 16, csize // 8)) == csize:   # the workspace's queue holds every bin
            assert st["overflow"] == 0


# the split y transform of the means (CG_TUNE_FUSED_Y = 2, nxp = nyp = 256): x + y stage 1 in the row
# kernels, y stage 2 in the bin kernel; in-band and out-of-band planes, in-kernel FP64 bins at cond 1.0001
@pytest.mark.parametrize("nzp,cond,form", [(24, 0.0, "mixed"), (20, 0.0, "fp32"), (16, 1.0001, "mixed")])
def test_split_y_pipeline_matches_fp64_oracle(cuda, oracle, nzp, cond, form):
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    from crava_gb300 import _native
    sc = S.scaled_config1(256, 256, nzp, seed=nzp + 7)
    inv = Inversion(sc, forms=(form,), cond_threshold=cond)
    inv.restore(form)
    inv.ws.reset_stats()
    L = _native.lib()
    assert L.cg_tune_set(4, 256, 2) == 0
    try:
        inv.run(form)
        torch.cuda.synchronize()
    finally:
        L.cg_tune_clear()
        _native._apply_tuning(L)
    st = inv.ws.stats()
    pm, res, cov = inv.results(form)
    post64, res64, cov64, _ = oracle_pipeline(oracle, sc, "d", tables=inv.tables)
    prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
    e = (rel(pm, post64), rel(pm - prior, post64 - prior), rel(res, res64), rel(cov, cov64))
    print(nzp, cond, form, "split y vs FP64 oracle (mean, update, resid, cov):", e, st)
    assert e[0] < 1e-6 and e[1] < 1e-4 and e[2] < 1e-4 and e[3] < 1e-4
    band = inv.tables["band"].astype(bool)
    assert band.any() and not band.all()
    if cond > 0:
        assert st["flagged"] > int(band.sum()) * sc.cnxp * sc.nyp // 2


# the information form of the fused bin solve (CG_TUNE_BIN_FORM = 1, the default): per-k eigen-decompositions of the error
# covariance, a 3 x 3 Cholesky per bin; guarded bins (cond 1.0001 flags most of them) go to the FP64 fix-up
# the 128^3 cases give every CTA two runs of bins of its plane (the grid keeps about four waves), for both forms
@pytest.mark.parametrize("dims,cond,form,nt,bin_form", [((64, 128, 48), 0.0, "mixed", 5, 1), ((40, 200, 36), 0.0, "fp32", 5, 1),
                                                        ((48, 64, 40), 1.0001, "mixed", 5, 1), ((36, 48, 30), 0.0, "mixed", 3, 1),
                                                        ((30, 40, 32), 0.0, "fp32", 8, 1),
                                                        ((128, 128, 128), 0.0, "mixed", 5, 1),
                                                        ((128, 128, 128), 1.0001, "mixed", 5, 1),
                                                        ((128, 128, 128), 0.0, "mixed", 5, 0)])
def test_information_form_matches_fp64_oracle(cuda, oracle, dims, cond, form, nt, bin_form):
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    from crava_gb300 import _native
    nxp, nyp, nzp = dims
    sc = S.make_scenario(int(nxp / 1.25), int(nyp / 1.25), int(nzp / 1.25), list(np.linspace(0.0, 40.0, nt)), 25.0,
                         nxp=nxp, nyp=nyp, nzp=nzp, sn=3.0, notches_hz=(2.0, 80.0), low_cut=1.0, high_cut=100.0,
                         seed=nxp + nzp + nt)
    L = _native.lib()
    assert L.cg_tune_set(5, 0, bin_form) == 0
    try:
        inv = Inversion(sc, forms=(form,), cond_threshold=cond)
        inv.restore(form)
        inv.ws.reset_stats()
        inv.run(form)
        torch.cuda.synchronize()
    finally:
        L.cg_tune_clear()
        _native._apply_tuning(L)
    st = inv.ws.stats()
    pm, res, cov = inv.results(form)
    post64, res64, cov64, _ = oracle_pipeline(oracle, sc, "d", tables=inv.tables)
    prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
    e = (rel(pm, post64), rel(pm - prior, post64 - prior), rel(res, res64), rel(cov, cov64))
    print(dims, cond, form, nt, bin_form, "fused form vs FP64 oracle (mean, update, resid, cov):", e, st)
    assert e[0] < 1e-6 and e[1] < 1e-4 and e[2] < 1e-4 and e[3] < 1e-4
    if cond > 0:
        assert st["flagged"] > 0


@pytest.mark.parametrize("bin_form,cond", [(0, 0.0), (1, 0.0), (0, 1.0001), (1, 1.0001)])
def test_bin_runs_per_cta_give_identical_results(cuda, bin_form, cond):
    """The runs one CTA solves per staged per-k table (CG_TUNE_BIN_RUNS) change only how bins are grouped into
    CTAs: every setting gives the same posterior bit for bit, in both bin forms, with and without the FP64 guard
    forced on every in-band bin (the cube's bins fit the fix-up queue, so no bin falls back on overflow, which
    would depend on the queue order)."""
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    from crava_gb300 import _native
    sc = S.make_scenario(38, 51, 32, list(np.linspace(0.0, 40.0, 5)), 25.0, nxp=48, nyp=64, nzp=40, sn=3.0,
                         notches_hz=(2.0, 80.0), low_cut=1.0, high_cut=100.0, seed=77)
    assert sc.nbins <= 65536
    L = _native.lib()
    out = []
    try:
        assert L.cg_tune_set(5, 0, bin_form) == 0
        inv = Inversion(sc, forms=("mixed",), cond_threshold=cond)
        for runs in (0, 1, 3, 8):
            assert L.cg_tune_set(8, 0, runs) == 0
            inv.restore("mixed")
            inv.run("mixed")
            torch.cuda.synchronize()
            out.append(inv.results("mixed"))
    finally:
        L.cg_tune_clear()
        _native._apply_tuning(L)
    for o in out[1:]:
        for a, b in zip(o, out[0]):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("nt", [1, 2, 3, 5, 8])
def test_cold_inversion_matches_repeated_model_and_fp64_oracle(cuda, oracle, nt):
    """run_cold (operator tables, cg_workspace_set_model_async and the per-k table kernel inside the call)
    gives bit-for-bit the three-pass mixed inversion of a workspace whose model was set synchronously, and
    stays within the FP64 oracle's tolerances; stack counts 1..8 cover the parallel Jacobi's even and odd
    index sets."""
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    sc = S.make_scenario(32, 28, 40, list(np.linspace(0.0, 40.0, nt)), 25.0, nxp=40, nyp=36, nzp=48, sn=3.0,
                         notches_hz=(2.0, 80.0), low_cut=1.0, high_cut=100.0, seed=31 + nt)
    inv = Inversion(sc, forms=("mixed",))
    inv.restore("mixed")
    inv.run("mixed_3pass")
    torch.cuda.synchronize()
    warm = inv.results("mixed")
    from crava_gb300 import api
    inv2 = Inversion(sc, forms=("mixed",))
    # a stale model in the workspace, which run_cold must replace
    bad = S.make_scenario(32, 28, 40, list(np.linspace(5.0, 35.0, nt)), 30.0, nxp=40, nyp=36, nzp=48, sn=4.0,
                          seed=99)
    bad_tab = api.operator_tables(bad.wavelets, bad.A, bad.nz, bad.nzp, bad.dt_ms, bad.low_cut, bad.high_cut)
    inv2.ws.set_model(bad_tab, bad.err_theta_cov, bad.sigma0, bad.wnc)
    inv2.restore("mixed")
    inv2.run_cold("mixed")
    torch.cuda.synchronize()
    cold = inv2.results("mixed")
    for a, b in zip(cold, warm):
        assert np.array_equal(a, b)
    post64, res64, cov64, _ = oracle_pipeline(oracle, sc, "d", tables=inv.tables)
    prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
    e = (rel(cold[0], post64), rel(cold[0] - prior, post64 - prior), rel(cold[1], res64), rel(cold[2], cov64))
    print(nt, "cold inversion vs FP64 oracle (mean, update, resid, cov):", e)
    assert e[0] < 1e-6 and e[1] < 1e-4 and e[2] < 1e-4 and e[3] < 1e-4


def test_condition_histogram_counts_every_inband_bin(cuda):
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    sc = S.scaled_config1(48, 40, 64, seed=8)
    inv = Inversion(sc, forms=("mixed",))
    inv.restore("mixed")
    inv.run("mixed")
    torch.cuda.synchronize()
    hc, hi = inv.ws.condition_histogram(16)
    inband = int(inv.tables["band"].sum()) * sc.cnxp * sc.nyp
    print("condition histograms (Cholesky FP64, information FP32):", hc, hi)
    assert sum(hc) == inband
    assert 0 < sum(hi) <= inband
    assert hc[-1] == 0  # no failed factorisation on this model
    # a forced guard flags the bins the histogram puts above the threshold
    inv2 = Inversion(sc, forms=("mixed",), cond_threshold=10.0)
    inv2.restore("mixed")
    inv2.ws.reset_stats()
    inv2.run("mixed")
    torch.cuda.synchronize()
    hc2, hi2 = inv2.ws.condition_histogram(16)
    assert hi2 == hi
    fl = inv2.ws.stats()["flagged"]
    assert sum(hi[2:]) <= fl <= sum(hi[1:])  # above the threshold of 10 (decade 1 holds 10 itself)


# nonzero correlation gradients: the prior is no longer separable (fillInParamCorr's shifted temporal
# correlation); the fused forms read the per-bin table of cg_prior_spectra_grad
@pytest.mark.parametrize("dims", [(40, 36, 48), (36, 128, 40)])
@pytest.mark.parametrize("form", ["plain", "fp32", "mixed", "fp64", "mixed_3pass"])
def test_correlation_gradients_match_fp64_oracle(cuda, oracle, dims, form):
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    grad = (0.37, -0.21)
    sc = S.scaled_config1(*dims, seed=23, corr_grad=grad)
    inv = Inversion(sc, forms=(form,))
    inv.restore(form)
    inv.run(form)
    torch.cuda.synchronize()
    pm, res, cov = inv.results(form)
    post64, res64, cov64, _ = oracle_pipeline(oracle, sc, "d", tables=inv.tables)
    prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
    e = (rel(pm, post64), rel(pm - prior, post64 - prior), rel(res, res64), rel(cov, cov64))
    print(dims, form, "gradients", grad, "vs FP64 oracle (mean, update, resid, cov):", e)
    tol = 1e-10 if form == "fp64" else 1e-4
    assert e[0] < (1e-12 if form == "fp64" else 1e-6)
    assert e[1] < tol and e[2] < tol and e[3] < tol
    # the gradients change the answer: the separable (zero-gradient) prior is far from the oracle's
    sc0 = S.scaled_config1(*dims, seed=23)
    post0, _, cov0, _ = oracle_pipeline(oracle, sc0, "d", tables=inv.tables)
    assert rel(post0 - prior, post64 - prior) > 1e-2 and rel(cov0, cov64) > 1e-2


def test_correlation_gradients_through_host_context(cuda):
    """The C++ host layer (cg_inversion_*) takes the gradients from its model struct and gives the
    pipeline's fused mixed answer bit for bit."""
    from crava_gb300 import api, synthetic as S
    from crava_gb300.pipeline import Inversion
    sc = S.scaled_config1(40, 128, 48, seed=24, corr_grad=(-0.3, 0.45))
    inv = Inversion(sc, forms=("mixed",))
    inv.restore("mixed")
    inv.run("mixed")
    torch.cuda.synchronize()
    pm, res, cov = inv.results("mixed")
    h = api.HostInversion(sc)
    data = [d.copy() for d in sc.data]
    mean = [m.copy() for m in sc.mean]
    cv = [np.zeros_like(sc.data[0]) for _ in range(6)]
    h.run(data, mean, cv, form="mixed")
    assert np.array_equal(np.stack([m[:, :, :sc.nxp] for m in mean]), pm)
    assert np.array_equal(np.stack([d.view(np.complex64) for d in data]), res)
    assert np.array_equal(np.stack([c.view(np.complex64) for c in cv]), cov)


@pytest.mark.parametrize("case", ["inversion_c0small.npz", "inversion_grad.npz"])
def test_correlation_fills_bit_exact_vs_reference(cuda, case):
    """cg_fill_param_corr / cg_fill_err_corr against the cubes the reference's fillInParamCorr (times
    priorVar0) and fillInErrCorr wrote, with zero and nonzero correlation gradients."""
    from crava_gb300 import api
    g = golden(case)
    nxp, nyp, nzp = int(g["nxp"]), int(g["nyp"]), int(g["nzp"])
    gi, gj = (float(x) for x in g["corr_grad"]) if "corr_grad" in g else (0.0, 0.0)
    corr_xy = torch.from_numpy(g["corr_xy"].astype(np.float32)).cuda()
    circ = torch.from_numpy(g["circ_corr_t"].astype(np.float32)).cuda()
    s0f = g["sigma0"].astype(np.float32)
    buf = torch.empty(g["errcorr_real"].shape, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream()
    for t, (p, q) in enumerate([(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]):
        api.check_call("cg_fill_param_corr", buf, nxp, nyp, nzp, corr_xy, circ, gi, gj, float(s0f[p, q]), st)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(buf.cpu().numpy(), g["prior_cov_real"][t])
    api.check_call("cg_fill_err_corr", buf, nxp, nyp, nzp, corr_xy, gi, gj, st)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(buf.cpu().numpy(), g["errcorr_real"])


@pytest.mark.parametrize("form", ["plain", "fp32", "mixed"])
def test_captured_step_replays_the_eager_inversion(cuda, form):
    """Inversion.capture: the step captured once as a CUDA graph gives, on every replay, the eager step's
    outputs bit for bit (the benchmark's headline step is this replay)."""
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    sc = S.scaled_config1(40, 36, 48, seed=27)
    inv = Inversion(sc, forms=(form,))
    inv.restore(form)
    inv.run(form)
    torch.cuda.synchronize()
    eager = inv.results(form)
    g = inv.capture(form)
    for _ in range(2):
        inv.restore(form)
        g.replay()
        torch.cuda.synchronize()
        for a, b in zip(inv.results(form), eager):
            assert np.array_equal(a, b)
