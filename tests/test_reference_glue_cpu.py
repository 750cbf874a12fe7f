"""The code around the bin solve against the reference's own compiled classes.

The fixtures come from crava_o2 (oracle/o2_harness.cpp), which runs the
reference's Wavelet, SeismicParametersHolder, Crava and State4D code compiled
from its sources (tests/golden/make_golden.py): its Ricker wavelets and
resampling, computeCircCorrT, the prior and error correlation fills,
fillErrMultVectors for both thickness branches, the whole
computePostMeanResidAndFFTCov, computeAdjustmentFactor, State4D::merge and
::split and findClosestFactorableNumber.  Here the repo's restatements (the
synthetic-input generator, the C++ host tables, the CPU oracle) are held to
them; the GPU tests hold the GPU to the same fixtures.
"""
import numpy as np
import pytest

from conftest import golden, oracle_pipeline, rel

CASES = ["inversion_c0small.npz", "inversion_c1small.npz", "inversion_n8odd.npz", "inversion_grad.npz"]
TABLES = ("K", "em1", "em2", "em3")


def _scenario(g):
    """The fixture's inputs as a Scenario (the reference's circCorrT)."""
    from crava_gb300 import synthetic as S
    return S.Scenario(nx=int(g["nx"]), ny=int(g["ny"]), nz=int(g["nz"]), nxp=int(g["nxp"]), nyp=int(g["nyp"]),
                      nzp=int(g["nzp"]), dt_ms=float(g["dt_ms"]), theta_deg=list(g["theta_deg"]), A=g["A"],
                      wavelets=g["wavelets"], corr_xy=g["corr_xy"], circ_corr_t=g["circ_corr_t"],
                      sigma0=g["sigma0"], err_theta_cov=g["err_theta_cov"], data=list(g["data_real"]),
                      mean=list(g["mean_real"]), wnc=float(g["wnc"]), low_cut=float(g["low_cut"]),
                      high_cut=float(g["high_cut"]),
                      corr_grad=tuple(float(x) for x in g["corr_grad"]) if "corr_grad" in g else (0.0, 0.0))


def test_ricker_wavelets_match_reference():
    """synthetic.ricker_fft_order (Wavelet's Ricker, 239 taps at 1 ms, resampled onto the grid in FFT
    order, src/wavelet.cpp:130-186, :416-463) and the wavelet norm."""
    from crava_gb300 import synthetic as S
    g = golden("reference_wavelets.npz")
    for i in range(4):
        nzp, dt, f, _ = g[f"case{i}_grid"]
        w = S.ricker_fft_order(int(nzp), float(dt), float(f)).astype(np.float32)
        ref = g[f"case{i}_wavelets"]
        assert rel(w, ref[0]) < 1e-6 and rel(w, ref[1]) < 1e-6, i
        norm = np.sqrt(np.sum((w * w).astype(np.float64)))
        assert abs(norm - g[f"case{i}_norms"][0]) <= 1e-6 * norm


def test_circ_corr_t_matches_reference(oracle):
    """computeCircCorrT + makeCircCorrTPosDef (src/seismicparametersholder.cpp:430-501): the FP64
    restatement in the input generator and the oracle's FP32 one."""
    from crava_gb300 import synthetic as S
    g = golden("reference_wavelets.npz")
    for i in range(4):
        nzp = int(g[f"case{i}_grid"][0])
        ref = g[f"case{i}_circ_corr_t"]
        c = S.circ_corr_t(g[f"case{i}_corr_t"], int(g[f"case{i}_min_int_fq"]), nzp)
        assert rel(c, ref) < 1e-6, i
        assert rel(oracle.circ_corr_t(g[f"case{i}_corr_t"], int(g[f"case{i}_min_int_fq"]), nzp), ref) < 1e-6, i


@pytest.mark.parametrize("case", CASES)
def test_prior_and_error_correlation_fills_bit_exact(oracle, case):
    """FFTGrid::fillInParamCorr x priorVar0 (initializeCorrelations) and fillInErrCorr, with the fixture's
    correlation gradients (nonzero in inversion_grad.npz, where the error correlation's |lag| < 1 window
    depends on the last bit of the float lag)."""
    g = golden(case)
    nxp, nyp, nzp = int(g["nxp"]), int(g["nyp"]), int(g["nzp"])
    gi, gj = (float(x) for x in g["corr_grad"]) if "corr_grad" in g else (0.0, 0.0)
    s0 = np.asarray(g["sigma0"]).astype(np.float32)
    for t, (p, q) in enumerate([(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]):
        c = oracle.fill_param_corr(nxp, nyp, nzp, g["corr_xy"], g["circ_corr_t"], gi, gj, float(s0[p, q]))
        np.testing.assert_array_equal(c[..., :nxp], g["prior_cov_real"][t][..., :nxp])
    e = oracle.fill_err_corr(nxp, nyp, nzp, g["corr_xy"], gi, gj)
    np.testing.assert_array_equal(e[..., :nxp], g["errcorr_real"][..., :nxp])
    if gi or gj:  # the gradients matter: the separable fill differs
        c0 = oracle.fill_param_corr(nxp, nyp, nzp, g["corr_xy"], g["circ_corr_t"], 0, 0, float(s0[0, 0]))
        assert not np.array_equal(c0[..., :nxp], g["prior_cov_real"][0][..., :nxp])


@pytest.mark.parametrize("case", CASES)
def test_host_operator_tables_match_reference_both_branches(native, oracle, case):
    """cg_operator_tables / cg_operator_tables_ex (host C++) and the oracle's restatements against the
    reference's fillErrMultVectors, fillkW, fillkWNorm and fillInverseAbskWRobust (src/crava.cpp:1337-1519)
    on the same wavelets, both thickness branches.  In band, entries agree to FP32 rounding of the table's
    scale (the reference's spectra are FP32 FFTW transforms).  Out of band the non-constant branch's
    errMult3 at the Ricker's DC bin is 1/|W(0)| of a value that is zero up to rounding: it is huge on both
    sides and never used."""
    from crava_gb300 import api
    g = golden(case)
    args = (g["wavelets"], g["A"], int(g["nz"]), int(g["nzp"]), float(g["dt_ms"]), float(g["low_cut"]),
            float(g["high_cut"]))
    band = np.asarray(g["band"]).astype(bool)
    for branch, sfx in (("constant", ""), ("non-constant", "_nct")):
        if sfx:
            host = api.operator_tables_nct(*args, 1.0)
            orc = oracle.k_tables_nct(int(g["nxp"]), g["wavelets"], g["A"], int(g["nz"]), int(g["nzp"]),
                                      int(g["nz"]) * float(g["dt_ms"]), float(g["low_cut"]), float(g["high_cut"]), 1.0)
        else:
            host = api.operator_tables(*args)
            orc = oracle.k_tables(int(g["nxp"]), *args)
        for impl, t in (("host", host), ("oracle", orc)):
            np.testing.assert_array_equal(t["band"], g["band" + sfx])
            for k in TABLES:
                ref = g[k + sfx][band]
                got = t[k][band]
                if sfx and k == "em3":
                    # errMult3 = 1/max|W| (robust): compare the amplitudes, whose FP32 rounding is absolute;
                    # near the notches of a notched wavelet 1/|W| magnifies it
                    ref, got = 1.0 / ref.real, 1.0 / got.real
                assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max(), (branch, impl, k)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("prec", ["f", "d"])
def test_oracle_pipeline_matches_reference_crava(oracle, case, prec):
    """The whole inversion: the oracle in the reference's dataflow (its own transforms and bin loop) with
    the reference's tables against Crava::computePostMeanResidAndFFTCov itself (src/crava.cpp:975-1285),
    which also ran the reference's findParameterVariances, getNextErrorVariance, band test and
    lib_matr solves.  FP32 differences only: the update (posterior minus prior mean) is ~60x smaller than
    the mean, so its relative difference is correspondingly larger."""
    g = golden(case)
    sc = _scenario(g)
    tab = {k: g[k] for k in TABLES + ("band",)}
    post, res, cov, nf = oracle_pipeline(oracle, sc, prec, tables=tab)
    nxp = sc.nxp
    prior = g["mean_real"][..., :nxp]
    ref_mean = g["crava_mean_real"][..., :nxp]
    e = (rel(post, ref_mean), rel(post - prior, ref_mean - prior), rel(res, g["crava_resid"]),
         rel(cov, g["crava_cov"]))
    print(case, prec, "oracle vs reference Crava (mean, update, resid, cov):", e)
    assert e[0] < 1e-6 and e[1] < 1e-4 and e[2] < 2e-5 and e[3] < 2e-5
    assert nf == int(g["nfail"])


@pytest.mark.parametrize("case", CASES)
def test_bin_loop_glue_matches_reference_crava(case):
    """ref_harness.cpp's glue around the reference's lib_matr (the fixture's out_* arrays, which keep the
    posterior-mean spectra) reproduces the reference's own bin loop bit for bit."""
    g = golden(case)
    np.testing.assert_array_equal(g["out_resid"], g["crava_resid"])
    np.testing.assert_array_equal(g["out_cov"], g["crava_cov"])
    nxp = int(g["nxp"])
    np.testing.assert_array_equal(g["out_mean_real"][..., :nxp], g["crava_mean_real"][..., :nxp])


def test_state4d_merge_and_split_match_reference(oracle):
    """State4D::merge and State4D::split (src/state4d.cpp:140-580) against the FP32 oracle restatement."""
    g = golden("state4d_n4.npz")
    st = list(g["state"])
    mu_s, mu_d, ss, sd, dd = st[0:3], st[3:6], st[6:12], st[12:21], st[21:27]
    mu_cur, cov_cur = oracle.state4d_merge(mu_s, mu_d, ss, sd, dd, prec="f")
    merged = np.stack(list(mu_cur) + list(cov_cur))
    e_merge = rel(merged, g["merged"])
    post = list(g["post"])
    st_out, nfail = oracle.state4d_split(mu_s, mu_d, ss, sd, dd, post[:3], post[3:], prec="f")
    split = np.stack([x for grp in st_out for x in grp])
    e_split = rel(split, g["split"])
    print("State4D oracle vs reference: merge", e_merge, "split", e_split, "split failures", nfail)
    assert e_merge < 1e-7
    assert e_split < 1e-5


def test_adjustment_factor_matches_reference(oracle):
    """Crava::computeAdjustmentFactor (src/crava.cpp:807-903) for local time shifts, gains and relative
    thicknesses 0.6-1.3: the oracle's per-trace restatement that the GPU scale-wavelet division is held to.
    Compared on the bins divideDataByScaleWavelet uses (lowCut < f_k < highCut with the trace's stretched
    frequency step, src/crava.cpp:750-770); above highCut, near the Nyquist bin, the global wavelet's
    spectrum is zero up to FP32 rounding and the factor is that rounding magnified."""
    g = golden("reference_adjustment.npz")
    cases = g["cases"]
    nz, nzp, dt = int(g["nz"]), int(g["nzp"]), float(g["dt_ms"])
    s0 = np.asarray(g["sigma0"]).astype(np.float32).astype(np.float64)
    worst = 0.0
    for l in range(2):
        for c, (ts, gain, sf) in enumerate(cases):
            ref = g[f"adjust{l}"][c]
            got = oracle.adjustment_factor(g[f"wavelet{l}"], g[f"A{l}"], s0, g[f"corr_t_filtered{l}"], nz, dt,
                                           nz * dt, float(g["low_cut"]), float(g["high_cut"]), float(g["wnc"]),
                                           float(g[f"err_var{l}"]), float(ts), float(gain), float(sf))
            f = 1000.0 / (float(sf) * dt * nzp) * np.arange(nzp // 2 + 1)
            used = (f > float(g["low_cut"])) & (f < float(g["high_cut"]))
            e = rel(got[used], ref[used])
            worst = max(worst, e)
            assert e < 2e-5, (l, c, e)
    print("adjustment factor vs reference: worst rel err", worst)


def test_find_closest_factorable_matches_reference(native, oracle):
    """FFTGrid::findClosestFactorableNumber (src/fftgrid.cpp:2857-2885): the C-ABI, the oracle and the
    input generator."""
    from crava_gb300.synthetic import find_closest_factorable
    g = golden("reference_factorable.npz")
    for n, ref in zip(g["n"], g["closest"]):
        assert native.cg_find_closest_factorable(int(n)) == ref
        assert oracle.find_closest_factorable(int(n)) == ref
        assert find_closest_factorable(int(n)) == ref


def test_crava_file_bytes_and_reader_match_reference(native, tmp_path):
    """FFTGrid::writeCravaFile / readCravaFile (src/fftgrid.cpp:2410-2493): the library writes the same
    bytes as the reference for the same cube and geometry, and the reference's reader gets the cube back
    from the library's file (and the library reads the reference's file)."""
    from crava_gb300 import api
    g = golden("reference_file_formats.npz")
    p = tmp_path / "grid.crava"
    api.write_crava_file(p, g["cube"], list(g["geom"]), int(g["nx"]), int(g["ny"]))
    assert p.read_bytes() == bytes(g["crava_bytes"])
    np.testing.assert_array_equal(g["read_crava"], g["cube"])
    q = tmp_path / "ref.crava"
    q.write_bytes(bytes(g["crava_bytes"]))
    back, geom, nxny = api.read_crava_file(q, int(g["nxp"]), int(g["nyp"]), int(g["nzp"]))
    np.testing.assert_array_equal(back, g["cube"])
    assert list(geom) == list(g["geom"]) and nxny == (int(g["nx"]), int(g["ny"]))


def test_storm_file_bytes_and_reader_match_reference(native, tmp_path):
    """NRLib::StormContGrid::WriteToFile / ReadFromFile (libs/nrlib/stormgrid/stormcontgrid.cpp:72-205) with
    constant surfaces: same bytes as the reference's writer, and the reference's reader gets the values and
    the header back from the library's file."""
    from crava_gb300 import api
    g = golden("reference_file_formats.npz")
    hv = dict(zip(("zone", "missing", "x_min", "lx", "y_min", "ly", "z_top", "z_bot", "erosion_top", "erosion_bot",
                   "angle_deg"), g["storm_header"]))
    h = api.StormHeader()
    h.zone_number, h.model_file, h.missing_code, h.variable = int(hv["zone"]), b"ModelFile", hv["missing"], b"Vp"
    h.x_min, h.lx, h.y_min, h.ly = hv["x_min"], hv["lx"], hv["y_min"], hv["ly"]
    h.z_top, h.z_bot, h.erosion_top, h.erosion_bot = hv["z_top"], hv["z_bot"], hv["erosion_top"], hv["erosion_bot"]
    h.lz, h.angle_deg = hv["z_bot"] - hv["z_top"], hv["angle_deg"]
    p = tmp_path / "vp.storm"
    api.write_storm(p, g["values"], h)
    assert p.read_bytes() == bytes(g["storm_bytes"])
    np.testing.assert_array_equal(g["read_storm"], g["values"])
    rh = dict(zip([str(k) for k in g["read_storm_keys"]], g["read_storm_header"]))
    assert (rh["ni"], rh["nj"], rh["nk"]) == (5, 4, 3)
    assert rh["x_min"] == hv["x_min"] and rh["lx"] == hv["lx"] and rh["z_top"] == hv["z_top"]
    assert abs(rh["angle"] - np.pi * hv["angle_deg"] / 180.0) < 1e-15 and rh["lz"] == hv["z_bot"] - hv["z_top"]


def test_local_noise_correction_matches_reference(oracle):
    """Crava::computeG and Crava::correctAlphaBetaRho run by the reference's own code (crava_o2): computeG
    restated with LAPACK's geev reproduces the reference's G, and the oracle's correction with that G is bit for
    bit the reference's on every trace but the one whose scale is RMISSING, where the reference takes the square
    root of a negative ratio and writes NaN (here that trace counts at the minimum scale)."""
    from crava_gb300 import api
    g = golden("reference_localnoise.npz")
    nx, ny, nz, nxp = (int(g[k]) for k in ("nx", "ny", "nz", "nxp"))
    G = api.local_noise_g(g["err_theta_cov"], g["prior_var0"], g["post_var0"])
    assert np.abs(G - g["G"]).max() <= 1e-12 * np.abs(g["G"]).max()
    out, _ = oracle.correct_alpha_beta_rho(list(g["post"]), list(g["mean"]), nx, ny, nz, nxp, g["G"],
                                           g["err_theta_cov"], g["prior_var0"], g["post_var0"], g["scale"])
    miss = np.zeros(g["out"][0].shape, bool)
    jj, ii = np.nonzero((g["scale"] == -99999.0).any(axis=0))
    miss[:nz, jj, ii] = True
    for p in range(3):
        ref = g["out"][p]
        np.testing.assert_array_equal(out[p][~miss], ref[~miss])
        assert np.isnan(ref[miss]).all() and np.isfinite(out[p][miss]).all()


@pytest.mark.parametrize("kind", ["data", "param"])
def test_fill_in_data_matches_reference(oracle, kind):
    """FFTGrid::fillInData run by the reference's own code (crava_o2) from a STORM grid onto a simbox: fed the
    per-column traces and geometry the reference's lookups produced, the oracle's per-trace core (taper or
    extrapolation and trend, FFT resampling, interpolation onto the cells) gives the reference's cube."""
    g = golden("reference_fillindata.npz")
    nx, ny, nz, nxp, nyp, nzp = (int(g[k]) for k in ("nx", "ny", "nz", "nxp", "nyp", "nzp"))
    st = g[f"{kind}_state"]
    dz_data = np.unique(g[f"{kind}_dz_data"][st == 0])
    assert len(dz_data) == 1
    cube, ext = oracle.fill_in_data(nxp, nyp, nzp, nz, kind == "data", g[f"{kind}_traces"], st.astype(np.uint8),
                                    g[f"{kind}_z0_data"], g[f"{kind}_z0_grid"], g[f"{kind}_dz_grid"], float(dz_data[0]),
                                    float(g["smooth_length"]))
    ref = g[f"{kind}_cube"]
    assert rel(cube, ref) < 1e-6
    dead = np.nonzero(st)[0]
    assert np.all(cube.reshape(nzp, -1)[:, dead] == 0) and np.all(ref.reshape(nzp, -1)[:, dead] == 0)


@pytest.mark.parametrize("threshold", [0.0, 0.3])
def test_interpolate_seismic_bit_exact_vs_reference(oracle, threshold):
    """FFTGrid::interpolateSeismic run by the reference's own code (crava_o2): dead traces alone, in pairs, on the
    edge and in a corner, and low-energy traces; the oracle's restatement gives the same cube bit for bit."""
    g = golden("reference_interpolate.npz")
    nx, ny, nz, nxp = (int(g[k]) for k in ("nx", "ny", "nz", "nxp"))
    out, _ = oracle.interpolate_seismic(g["cube"], nx, ny, nz, nxp, threshold, prec="f")
    np.testing.assert_array_equal(out, g[f"out_{threshold:g}"])


def test_scale_wavelet_division_matches_reference(oracle):
    """Crava::divideDataByScaleWavelet (then interpolateSeismic) run by the reference's own code (crava_o2) on a
    simbox of non-constant thickness with local wavelet shifts and gains and two dead traces.  The wavelet and the
    gain grid are taken as the reference's Wavelet::setGainGrid leaves them (grid over its geometric mean, wavelet
    times it): the oracle's division and interpolation are then within 1e-6 of the reference's cubes."""
    g = golden("reference_divide.npz")
    nx, ny, nz, nxp = (int(g[k]) for k in ("nx", "ny", "nz", "nxp"))
    s0 = np.asarray(g["sigma0"]).astype(np.float32).astype(np.float64)
    for l in range(len(g["A"])):
        d = oracle.divide_scale_wavelet(g["data"][l], nx, ny, nz, g["wavelets"][l], g["A"][l], s0, g["corr_t_filtered"],
                                        float(g["dt_ms"]), float(g["lz"]), float(g["low_cut"]), float(g["high_cut"]),
                                        float(g["wnc"]), float(g["err_theta_cov"][l, l]), g["rel_thick"], g["shift"][l],
                                        g["gain_normalised"][l], prec="f")
        d, nbad = oracle.interpolate_seismic(d, nx, ny, nz, nxp, 0.0, prec="f")
        assert nbad == 2
        ref = g["out"][l]
        assert rel(d[..., :nxp], ref[..., :nxp]) < 1e-6, l


def test_scale_wavelet_multiply_matches_reference(oracle):
    """Crava::multiplyDataByScaleWaveletAndWriteToFile (src/crava.cpp:906-968) run by the reference's own code
    (crava_o2) on its divided cubes after their forward transform (the state the bin loop leaves the residuals
    in): the oracle's per-trace product on the divided cubes against the reference's result.  The reference
    round-trips each cube through its 3D transforms first and transforms its global wavelet back and forth
    once per trace (createLocalWavelet1D, getCAmp), so the two agree to FP32 rounding of those steps."""
    g = golden("reference_divide.npz")
    nx, ny, nxp = (int(g[k]) for k in ("nx", "ny", "nxp"))
    for l in range(len(g["A"])):
        m = oracle.multiply_scale_wavelet(g["out"][l], nx, ny, g["wavelets"][l], float(g["dt_ms"]), g["rel_thick"],
                                          g["shift"][l], g["gain_normalised"][l], prec="f")
        e = rel(m[..., :nxp], g["mult"][l][..., :nxp])
        print("multiply, angle", l, "oracle vs reference:", e)
        assert e < 2e-6, l


def test_storm_surface_files_match_reference(native, tmp_path):
    """A STORM grid whose top and bottom surfaces are regular surfaces in files beside it
    (Volume::WriteVolumeToFile / ReadVolumeFromFile, WriteStormBinarySurf / ReadStormBinarySurf): the
    library writes the reference's bytes for the grid and both surface files (lz given as the reference
    computed it), reads the reference's files back, and the reference read the library's files."""
    from crava_gb300 import api
    g = golden("reference_storm_surfaces.npz")
    hv = dict(zip(("zone", "missing", "x_min", "lx", "y_min", "ly", "z_top", "z_bot", "erosion_top", "erosion_bot",
                   "angle_deg"), g["header"]))
    ref = {str(n): bytes(g[f"ref_file{i}"]) for i, n in enumerate(g["ref_names"])}
    head = ref["out.storm"].split(b"\n")
    lz = float(head[7].split()[0])  # Volume::RecalculateLZ's sampled maximum thickness
    h = api.StormHeader()
    h.zone_number, h.model_file, h.missing_code, h.variable = int(hv["zone"]), b"ModelFile", hv["missing"], b"Vp"
    h.x_min, h.lx, h.y_min, h.ly = hv["x_min"], hv["lx"], hv["y_min"], hv["ly"]
    h.erosion_top, h.erosion_bot, h.lz, h.angle_deg = hv["erosion_top"], hv["erosion_bot"], lz, hv["angle_deg"]
    sg = g["surf_geom"]
    surfs = {"z_top_file": api.StormSurface(g["top"], *sg), "z_bot_file": api.StormSurface(g["bot"], *sg)}
    p = tmp_path / "out.storm"
    api.write_storm(p, g["values"], h, surfaces=surfs)
    for name, raw in ref.items():
        assert (tmp_path / name).read_bytes() == raw, name
    # the library reads the reference's files
    d = tmp_path / "ref"
    d.mkdir()
    for name, raw in ref.items():
        (d / name).write_bytes(raw)
    v, rh = api.read_storm(d / "out.storm")
    np.testing.assert_array_equal(v, g["values"])
    assert rh.z_top_file == b"out.storm_top" and rh.z_bot_file == b"out.storm_bot" and rh.lz == lz
    assert rh.erosion_top == hv["erosion_top"] and rh.erosion_bot == hv["erosion_bot"]
    s = api.read_storm_surfaces(d / "out.storm", rh)
    assert set(s) == {"z_top_file", "z_bot_file"}
    np.testing.assert_array_equal(s["z_top_file"].z, g["top"])
    np.testing.assert_array_equal(s["z_bot_file"].z, g["bot"])
    assert (s["z_top_file"].x_min, s["z_top_file"].y_min) == (sg[0], sg[1])
    assert abs(s["z_top_file"].lx - sg[2]) < 1e-9 and abs(s["z_top_file"].ly - sg[3]) < 1e-9
    # the reference read the library's files (written with its own lz) back exactly
    np.testing.assert_array_equal(g["read_values"].reshape(g["values"].shape), g["values"])
    np.testing.assert_array_equal(g["read_top"], g["top"])
    np.testing.assert_array_equal(g["read_bot"], g["bot"])


def test_state4d_evolve_matches_reference(oracle):
    """State4D::evolve (src/state4d.cpp:800-996) run by the reference's own code (crava_o2) with one time step
    of a time evolution: the oracle's GenExp correlation fill is bit for bit the reference's
    fillInGenExpCorr, and its evolved state (FP64 products, as the reference forms them) agrees to the
    reference's FP32 storage."""
    g = golden("state4d_evolve.npz")
    nx, ny, nxp = int(g["nx"]), int(g["ny"]), int(g["nxp"])
    st = g["state"]
    nzp, nyp, _ = st.shape[1:]
    gr = oracle.fill_genexp(nxp, nyp, nzp, nx / 3.0, ny / 3.0, 20.0)
    np.testing.assert_array_equal(gr, g["genexp_real"])
    ev = np.stack(oracle.state4d_evolve(list(st), nxp, nyp, nzp, g["E"], g["c"], g["C"], lam=g["genexp_spec"]))
    assert rel(ev, g["evolved"]) < 1e-8
    for t in range(27):
        assert np.abs(ev[t] - g["evolved"][t]).max() <= 4e-7 * np.abs(g["evolved"][t]).max(), t
    # the increment and the mean shift are both visible in the fixture
    ev0 = np.stack(oracle.state4d_evolve(list(st), nxp, nyp, nzp, g["E"], g["c"], g["C"], lam=None))
    assert rel(ev0, g["evolved"]) > 1e-5
    assert g["evolved"][3][0, 0, 0] != st[3][0, 0, 0]
