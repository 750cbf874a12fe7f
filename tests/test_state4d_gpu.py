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


def _oracle_timelapse_chain(oracle, tl, state, errc, tables, prec="d"):
    """merge -> bin loop (4D branch) -> split per vintage, all in the oracle."""
    from crava_gb300.pipeline import MERGE_TO_BIN
    mu_s, mu_d, ss, sd, dd = [list(g) for g in state]
    tab = dict(tables, nxp=tl.nxp)
    nfails = []
    for v in tl.vintages:
        mu_cur, cov_cur = oracle.state4d_merge(mu_s, mu_d, ss, sd, dd, prec=prec)
        data = [oracle.fft3d_r2c(d, tl.nxp, oracle.DATA, prec) for d in v["data"]]
        _, mu_post, cov_bin, _ = oracle.invert_bins(data, mu_cur, [cov_cur[t] for t in MERGE_TO_BIN], errc, tab,
                                                    v["err_theta_cov"], tl.sigma_current(), tl.wnc, is4d=True,
                                                    prec=prec)
        cov_post = [None] * 6
        for k, t in enumerate(MERGE_TO_BIN):
            cov_post[t] = cov_bin[k]
        (mu_s, mu_d, ss, sd, dd), nf = oracle.state4d_split(mu_s, mu_d, ss, sd, dd, mu_post, cov_post, prec=prec)
        nfails.append(nf)
    return (mu_s, mu_d, ss, sd, dd), nfails


def test_timelapse_two_vintages_matches_fp64_oracle_chain(cuda, oracle):
    """Two vintages x 4 stacks: merge -> forward transforms -> plain bin loop (4D branch) -> split on the GPU
    against the same chain in the FP64 oracle, from the same initial state spectra."""
    from crava_gb300 import api, synthetic as S
    from crava_gb300.pipeline import TimeLapse
    tl = S.make_timelapse(16, 12, 11, [0.0, 40.0 / 3, 80.0 / 3, 40.0], 25.0, nxp=20, nyp=15, nzp=14, seed=7)
    run = TimeLapse(tl)
    run.restore()
    state0 = run.state()
    errc = api.as_spectrum(run.errcorr).cpu().numpy()
    run.run()
    torch.cuda.synchronize()
    got = run.state()
    ref, ref_fails = _oracle_timelapse_chain(oracle, tl, state0, errc, run.tables)
    names = ["mu_s", "mu_d", "ss", "sd", "dd"]
    errs = {nm: rel(np.stack(a), np.stack(b)) for nm, a, b in zip(names, got, ref)}
    upd = rel(np.stack(got[1]) - np.stack(state0[1]), np.stack(ref[1]) - np.stack(state0[1]))
    print("timelapse vs FP64 oracle chain:", errs, "dynamic update", upd,
          "split fails", [int(x.item()) for x in run.nfail_split])
    # bins with a zero prior (the temporal spectrum is cut to zero at k <= lowIntCut) keep their prior in
    # split, exactly as in the reference; the counts agree
    assert [int(x.item()) for x in run.nfail_split] == ref_fails
    assert errs["mu_s"] < 1e-6 and errs["mu_d"] < 1e-4 and upd < 1e-4
    assert errs["ss"] < 1e-5 and errs["sd"] < 1e-5 and errs["dd"] < 1e-5
    # posterior variances (diagonal spectra of the static and dynamic blocks) never exceed the prior ones
    for blk in (2, 4):
        for t in (0, 3, 5):
            post, prior = got[blk][t].real, state0[blk][t].real
            assert np.all(post <= prior + 1e-6 * np.abs(prior).max())


def test_plain_4d_bin_loop_matches_reference_lib_matr(cuda):
    """The 4D branch of the plain bin loop against the reference's own lib_matr run on the same spectra."""
    from conftest import golden
    from crava_gb300 import api
    g = golden("inversion_4d_n4.npz")
    n = len(g["theta_deg"])
    ws = api.Workspace(int(g["nxp"]), int(g["nyp"]), int(g["nzp"]), n)
    tab = {k: g[k] for k in ("K", "em1", "em2", "em3", "band")}
    ws.set_model(tab, g["err_theta_cov"], g["sigma0"], float(g["wnc"]), is4d=True)
    data = [to_cube(x) for x in g["data_spec"]]
    mean = [to_cube(x) for x in g["mean_spec"]]
    cov = [to_cube(x) for x in g["cov_spec"]]
    ws.invert_plain(data, mean, cov, to_cube(g["errcorr_spec"]))
    torch.cuda.synchronize()
    res = np.stack([from_cube(x) for x in data])
    mu = np.stack([from_cube(x) for x in mean])
    cv = np.stack([from_cube(x) for x in cov])
    e_upd = rel(mu - g["mean_spec"], g["out_mean"] - g["mean_spec"])
    e_res, e_cov = rel(res, g["out_resid"]), rel(cv, g["out_cov"])
    print("4D plain vs reference: update", e_upd, "resid", e_res, "cov", e_cov)
    assert e_upd < 1e-4 and e_res < 1e-5 and e_cov < 1e-5
    assert ws.stats()["failed"] == int(g["nfail"])


def test_fused_vintage_fp32_bit_identical_to_three_passes(cuda):
    """cg_vintage4d in FP32 (merge, 4D bin solve and split per bin in one pass) gives bit for bit the
    state, residuals, posterior means and split-failure counts of the separate merge / bin-loop / split
    kernels, over two vintages."""
    from crava_gb300 import api, synthetic as S
    from crava_gb300.pipeline import TimeLapse
    tl = S.make_timelapse(16, 12, 11, [0.0, 40.0 / 3, 80.0 / 3, 40.0], 25.0, nxp=20, nyp=15, nzp=14, seed=7)
    out = {}
    for form in ("plain", "fp32"):
        run = TimeLapse(tl)
        run.restore()
        for v in range(len(tl.vintages)):
            run.run_vintage(v, form=form)
        torch.cuda.synchronize()
        out[form] = (run.state(), [from_cube(x) for x in run.data], [x.cpu().numpy() for x in run.post_mean],
                     [int(x.item()) for x in run.nfail_split])
    (s_p, d_p, m_p, f_p), (s_f, d_f, m_f, f_f) = out["plain"], out["fp32"]
    for a, b in zip(s_p, s_f):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
    for x, y in zip(d_p, d_f):
        np.testing.assert_array_equal(x, y)
    for x, y in zip(m_p, m_f):
        np.testing.assert_array_equal(x, y)
    assert f_p == f_f


@pytest.mark.parametrize("cond", [0.0, 1.0001])
def test_fused_vintage_mixed_matches_fp64_oracle_chain(cuda, oracle, cond):
    """cg_vintage4d in the MIXED form against the FP64 oracle chain; cond = 1.0001 sends (nearly) every
    in-band bin through the FP64 redo of merge, solve and split."""
    from crava_gb300 import api, synthetic as S
    from crava_gb300.pipeline import TimeLapse
    tl = S.make_timelapse(16, 12, 11, [0.0, 40.0 / 3, 80.0 / 3, 40.0], 25.0, nxp=20, nyp=15, nzp=14, seed=7)
    run = TimeLapse(tl)
    if cond > 0:
        for v, ws in enumerate(run.ws):
            ws.set_model(run.tables, tl.vintages[v]["err_theta_cov"], tl.sigma_current(), tl.wnc, is4d=True,
                         cond_threshold=cond)
    run.restore()
    state0 = run.state()
    errc = api.as_spectrum(run.errcorr).cpu().numpy()
    flagged = []
    for v in range(len(tl.vintages)):
        run.ws[v].reset_stats()
        run.run_vintage(v, form="mixed")
        flagged.append(run.ws[v].stats()["flagged"])
    torch.cuda.synchronize()
    got = run.state()
    ref, ref_fails = _oracle_timelapse_chain(oracle, tl, state0, errc, run.tables)
    names = ["mu_s", "mu_d", "ss", "sd", "dd"]
    errs = {nm: rel(np.stack(a), np.stack(b)) for nm, a, b in zip(names, got, ref)}
    upd = rel(np.stack(got[1]) - np.stack(state0[1]), np.stack(ref[1]) - np.stack(state0[1]))
    print("fused mixed vintage (cond", cond, ") vs FP64 oracle chain:", errs, "dynamic update", upd, "flagged",
          flagged, "split fails", [int(x.item()) for x in run.nfail_split], ref_fails)
    assert [int(x.item()) for x in run.nfail_split] == ref_fails
    assert errs["mu_s"] < 1e-6 and errs["mu_d"] < 1e-4 and upd < 1e-4
    assert errs["ss"] < 1e-5 and errs["sd"] < 1e-5 and errs["dd"] < 1e-5
    if cond > 0:
        assert min(flagged) > 0
        assert upd < 1e-5  # the FP64 redo: only the FP32 storage of state and data remains


def test_evolve_and_genexp_match_reference(cuda):
    """cg_fill_genexp_corr and cg_state4d_evolve against the reference's fillInGenExpCorr and
    State4D::evolve (crava_o2; products in FP32 here, FP64 there)."""
    from conftest import golden
    from crava_gb300 import api
    g = golden("state4d_evolve.npz")
    nx, ny, nxp = int(g["nx"]), int(g["ny"]), int(g["nxp"])
    st = g["state"]
    nzp, nyp, _ = st.shape[1:]
    buf = torch.empty(g["genexp_real"].shape, dtype=torch.float32, device="cuda")
    api.fill_genexp_corr(buf, nxp, nx / 3.0, ny / 3.0, 20.0)
    torch.cuda.synchronize()
    gr = buf.cpu().numpy()
    # exp of the device against the host library: equal but for the odd last-bit case
    assert np.abs(gr - g["genexp_real"]).max() <= 6e-8 * np.abs(g["genexp_real"][..., :nxp]).max()
    api.fft_in_place(buf, nxp, api.COVARIANCE)
    lam_gpu = from_cube(buf)
    assert rel(lam_gpu, g["genexp_spec"]) < 1e-6
    cubes = [to_cube(x) for x in st]
    grp = [cubes[0:3], cubes[3:6], cubes[6:12], cubes[12:21], cubes[21:27]]
    api.state4d_evolve(*grp, nxp, g["E"], g["c"], g["C"], lam=to_cube(g["genexp_spec"]))
    torch.cuda.synchronize()
    got = np.stack([from_cube(x) for x in cubes])
    e = rel(got, g["evolved"])
    worst = max(float(np.abs(got[t] - g["evolved"][t]).max() / np.abs(g["evolved"][t]).max()) for t in range(27))
    print("evolve vs reference: rel", e, "worst cube max-abs / max", worst)
    assert e < 1e-6 and worst < 1e-5


def test_timelapse_with_evolution_matches_fp64_oracle_chain(cuda, oracle):
    """Two vintages with State4D::evolve between them (as ModelGeneral::advanceTime calls it) on the GPU
    against merge -> bin loop -> split -> evolve -> merge -> bin loop -> split in the FP64 oracle."""
    from crava_gb300 import api, synthetic as S
    from crava_gb300.pipeline import TimeLapse, MERGE_TO_BIN
    E = np.block([[np.eye(3), np.zeros((3, 3))],
                  [0.1 * np.eye(3), 0.9 * np.eye(3) + 0.05 * (np.ones((3, 3)) - np.eye(3))]])
    c = np.array([0.0, 0.0, 0.0, 0.01, -0.02, 0.005])
    C = np.zeros((6, 6))
    C[3:, 3:] = 4e-4 * np.array([[1.0, 0.3, 0.2], [0.3, 1.0, 0.25], [0.2, 0.25, 1.0]])
    tl = S.make_timelapse(16, 12, 11, [0.0, 40.0 / 3, 80.0 / 3, 40.0], 25.0, nxp=20, nyp=15, nzp=14, seed=7)
    tl.evolution = [(E, c, C)]
    for form in ("plain", "mixed"):
        run = TimeLapse(tl)
        run.restore()
        state0 = run.state()
        errc = api.as_spectrum(run.errcorr).cpu().numpy()
        lam = api.as_spectrum(run.lam).cpu().numpy()
        run.run(form=form)
        torch.cuda.synchronize()
        got = run.state()
        mu_s, mu_d, ss, sd, dd = [list(x) for x in state0]
        tab = dict(run.tables, nxp=tl.nxp)
        for v, vin in enumerate(tl.vintages):
            if v > 0:
                st = oracle.state4d_evolve(mu_s + mu_d + ss + sd + dd, tl.nxp, tl.nyp, tl.nzp, E, c, C, lam=lam,
                                           prec="d")
                mu_s, mu_d, ss, sd, dd = st[0:3], st[3:6], st[6:12], st[12:21], st[21:27]
            mu_cur, cov_cur = oracle.state4d_merge(mu_s, mu_d, ss, sd, dd, prec="d")
            data = [oracle.fft3d_r2c(d, tl.nxp, oracle.DATA, "d") for d in vin["data"]]
            _, mu_post, cov_bin, _ = oracle.invert_bins(data, mu_cur, [cov_cur[t] for t in MERGE_TO_BIN], errc,
                                                        tab, vin["err_theta_cov"], tl.sigma_current(), tl.wnc,
                                                        is4d=True, prec="d")
            cov_post = [None] * 6
            for k, t in enumerate(MERGE_TO_BIN):
                cov_post[t] = cov_bin[k]
            (mu_s, mu_d, ss, sd, dd), _ = oracle.state4d_split(mu_s, mu_d, ss, sd, dd, mu_post, cov_post, prec="d")
        ref = (mu_s, mu_d, ss, sd, dd)
        names = ["mu_s", "mu_d", "ss", "sd", "dd"]
        errs = {nm: rel(np.stack(a), np.stack(b)) for nm, a, b in zip(names, got, ref)}
        print(form, "timelapse with evolution vs FP64 oracle chain:", errs)
        assert errs["mu_s"] < 1e-6 and errs["mu_d"] < 1e-4
        assert errs["ss"] < 1e-5 and errs["sd"] < 1e-5 and errs["dd"] < 1e-5
