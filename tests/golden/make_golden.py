"""Generate the golden fixtures in this directory from the reference build.

Run where the CRAVA reference checkout exists, naming it:

    CRAVA_REFERENCE_SRC=<reference checkout> python tests/golden/make_golden.py

It builds oracle/_ref from the reference's own sources: the FFTW 2.1.2,
lib_matr.c and random.cpp pieces with ref_harness.cpp (oracle/Makefile.ref),
and crava_o2, the reference's whole Crava / Wavelet / SeismicParametersHolder
/ State4D code with o2_harness.cpp (oracle/Makefile.o2).  Every output array
comes from the reference's compiled code; the inputs are seeded synthetic
cubes.  The fixtures are small so the CPU suite stays fast, and they travel to
machines without the reference checkout, where they are the only
reference-generated vectors.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import o2  # noqa: E402
from oracle import oracle as O  # noqa: E402
from crava_gb300 import synthetic as S  # noqa: E402

NCT = ("K", "em1", "em2", "em3", "band")


def reference_tables(wavelets, A, theta_deg, nz, nzp, dt_ms, low_cut, high_cut, wnc=0.1):
    """The per-k tables of the reference's Crava::fillErrMultVectors for given resampled wavelets (both
    thickness branches), from a crava_o2 run on a 2 x 1 lateral grid (the tables depend on the wavelets,
    A, nz, nzp, dt and the band only)."""
    n = len(theta_deg)
    rnxp = 4  # 2 * (nxp//2 + 1) for nxp = 2
    zero = np.zeros((nzp, 1, rnxp), np.float32)
    sc = S.Scenario(nx=2, ny=1, nz=nz, nxp=2, nyp=1, nzp=nzp, dt_ms=dt_ms, theta_deg=list(theta_deg), A=A,
                    wavelets=wavelets, corr_xy=np.ones((1, 2), np.float32), circ_corr_t=None,
                    sigma0=np.diag([0.01, 0.005, 0.0025]), err_theta_cov=np.eye(n) * 1e-3, data=[zero] * n,
                    mean=[zero] * 3, wnc=wnc, low_cut=low_cut, high_cut=high_cut,
                    corr_t=S.genexp_corr_t(max(nz, 2), dt_ms, 20.0, 1.5),
                    min_int_fq=int(np.floor(low_cut * (nzp * 0.001 * dt_ms))))
    r = o2.inversion(sc, sc.corr_t, sc.min_int_fq, 30.0, wavelets=wavelets)
    return {k: r[k] for k in NCT}, {k: r[k + "_nct"] for k in NCT}


def fft_case(name, nxp, nyp, nzp, seed):
    rng = np.random.default_rng(seed)
    cnxp, rnxp = O.dims(nxp)
    x = np.zeros((nzp, nyp, rnxp), np.float32)
    x[:, :, :nxp] = rng.standard_normal((nzp, nyp, nxp)).astype(np.float32)
    spec = (rng.standard_normal((nzp, nyp, cnxp)) + 1j * rng.standard_normal((nzp, nyp, cnxp))).astype(np.complex64)
    out = {"nxp": nxp, "nyp": nyp, "nzp": nzp, "real_in": x, "spec_in": spec}
    out["r2c_data"] = O.ref_fft3d_r2c(x, nxp, O.DATA)
    out["r2c_cov"] = O.ref_fft3d_r2c(x, nxp, O.COVARIANCE)
    out["c2r_param"] = O.ref_fft3d_c2r(spec, nxp, O.PARAMETER)
    out["c2r_cov"] = O.ref_fft3d_c2r(spec, nxp, O.COVARIANCE)
    np.savez_compressed(os.path.join(HERE, name), **out)


def inversion_case(name, sc, f_peak):
    """One inversion by the reference's own Crava::computePostMeanResidAndFFTCov (crava_*) on the scenario's
    inputs, with the scenario's resampled wavelets in the reference's Wavelet objects; the per-k tables
    (both thickness branches), the prior / error correlation cubes and circCorrT are the reference's.  The
    bin loop is also run by ref_harness.cpp's glue around the reference's lib_matr on the same spectra
    (out_*), which keeps the posterior-mean spectra before the inverse transform."""
    r = o2.inversion(sc, sc.corr_t, sc.min_int_fq, f_peak, wavelets=sc.wavelets)
    tab = {k: r[k] for k in NCT}
    data = list(r["data_spec"])
    mean = list(r["mean_spec"])
    covs = [O.ref_fft3d_r2c(c, sc.nxp, O.COVARIANCE) for c in r["prior_cov_real"]]
    ec = O.ref_fft3d_r2c(r["errcorr_real"], sc.nxp, O.COVARIANCE)
    res, mu, cov, nfail = O.ref_invert_bins(data, mean, covs, ec, dict(tab, nxp=sc.nxp), sc.err_theta_cov,
                                            sc.sigma0, sc.wnc)
    post_real = [O.ref_fft3d_c2r(m, sc.nxp, O.PARAMETER) for m in mu]
    out = dict(nx=sc.nx, ny=sc.ny, nz=sc.nz, nxp=sc.nxp, nyp=sc.nyp, nzp=sc.nzp, dt_ms=sc.dt_ms,
               theta_deg=np.array(sc.theta_deg), A=sc.A, wavelets=sc.wavelets, corr_xy=sc.corr_xy,
               corr_t=sc.corr_t, min_int_fq=sc.min_int_fq, circ_corr_t=r["circ_corr_t"], sigma0=sc.sigma0,
               err_theta_cov=sc.err_theta_cov, wnc=sc.wnc, low_cut=sc.low_cut, high_cut=sc.high_cut,
               data_real=np.stack(sc.data), mean_real=np.stack(sc.mean),
               prior_cov_real=r["prior_cov_real"], errcorr_real=r["errcorr_real"],
               wavelet_norms=r["wavelet_norms"],
               data_spec=np.stack(data), mean_spec=np.stack(mean), cov_spec=np.stack(covs), errcorr_spec=ec,
               out_resid=np.stack(res), out_mean=np.stack(mu), out_cov=np.stack(cov), out_mean_real=np.stack(post_real),
               nfail=nfail, is4d=0, corr_grad=np.array(getattr(sc, "corr_grad", (0.0, 0.0)), np.float32),
               crava_mean_real=r["out_mean_real"], crava_resid=r["out_resid"], crava_cov=r["out_cov"],
               **tab, **{k + "_nct": r[k + "_nct"] for k in NCT})
    np.savez_compressed(os.path.join(HERE, name), **out)
    return out


def gradient_case(name):
    """An inversion whose prior and error correlation carry nonzero correlation gradients (corrGradI/J): the
    reference's fillInParamCorr / fillInErrCorr with the gradients and its bin loop on the resulting
    non-separable spectra."""
    sc = S.make_scenario(18, 14, 22, [0.0, 15.0, 30.0, 40.0], 25.0, nxp=24, nyp=18, nzp=28, sn=3.0,
                         notches_hz=(2.0, 80.0), low_cut=1.0, high_cut=100.0, seed=6, corr_grad=(0.37, -0.21))
    return inversion_case(name, sc, 25.0)


def wavelet_case(name):
    """The reference's own Ricker wavelets (Wavelet1D + Wavelet::resample) on a few grids."""
    out = {}
    for i, (nzp, dt, f) in enumerate([(30, 4.0, 30.0), (64, 2.0, 25.0), (45, 4.0, 45.0), (128, 4.0, 15.0)]):
        sc = S.make_scenario(4, 3, max(2, int(nzp / 1.25)), [0.0, 20.0], f, nxp=4, nyp=3, nzp=nzp, dt_ms=dt, seed=i)
        r = o2.inversion(sc, sc.corr_t, sc.min_int_fq, f)
        out[f"case{i}_grid"] = np.array([nzp, dt, f, sc.nz])
        out[f"case{i}_wavelets"] = r["wavelets"]
        out[f"case{i}_norms"] = r["wavelet_norms"]
        out[f"case{i}_corr_t"] = sc.corr_t
        out[f"case{i}_min_int_fq"] = sc.min_int_fq
        out[f"case{i}_circ_corr_t"] = r["circ_corr_t"]
    np.savez_compressed(os.path.join(HERE, name), **out)


def adjustment_case(name):
    """Crava::computeAdjustmentFactor for a grid of local time shifts, gains and relative thicknesses."""
    sc = S.make_scenario(16, 12, 40, [10.0, 30.0], 30.0, nxp=20, nyp=15, nzp=50, seed=9)
    cases = np.array([(0.0, 1.0, 1.0), (0.0, 1.0, 0.7), (0.0, 1.0, 1.3), (3.0, 1.2, 0.85), (-2.5, 0.8, 1.15),
                      (7.0, 1.0, 1.0), (0.0, 0.5, 0.6)], np.float32)
    out = dict(nz=sc.nz, nzp=sc.nzp, dt_ms=sc.dt_ms, low_cut=sc.low_cut, high_cut=sc.high_cut, wnc=sc.wnc,
               sigma0=sc.sigma0, cases=cases)
    for l in range(sc.ntheta):
        ev = float(sc.err_theta_cov[l, l])
        wav, ctf, adj = o2.adjustment(sc, l, sc.corr_t, sc.min_int_fq, 30.0, cases, ev)
        out[f"A{l}"] = sc.A[l]
        out[f"err_var{l}"] = ev
        out[f"wavelet{l}"] = wav
        out[f"corr_t_filtered{l}"] = ctf
        out[f"adjust{l}"] = adj
    np.savez_compressed(os.path.join(HERE, name), **out)


def file_format_case(name):
    """The reference's FFTGrid::writeCravaFile and StormContGrid::WriteToFile bytes for seeded cubes, and
    its readers' view of the files the library writes (crava_gb300.api.write_crava_file / write_storm)."""
    from crava_gb300 import api
    rng = np.random.default_rng(17)
    nx, ny, nxp, nyp, nzp = 8, 5, 10, 6, 4
    _, rnxp = api.dims(nxp)
    cube = rng.standard_normal((nzp, nyp, rnxp)).astype(np.float32)
    geom = np.array([1000.5, 2000.25, 25.0, 12.5, 100.0, 200.0, 0.5, -0.5, 0.25, 0.75, 0.1])
    crava_bytes = o2.crava_write(cube, nx, ny, nxp, geom)
    hdr = dict(zone=0, missing=-999.25, x_min=456000.0, lx=1600.0, y_min=6780000.0, ly=1200.0, z_top=1800.0,
               z_bot=2400.0, erosion_top=1800.0, erosion_bot=2400.0, angle_deg=30.0)
    values = rng.standard_normal((3, 4, 5)).astype(np.float32)
    storm_bytes = o2.storm_write(values, **hdr)
    # the library's own files, read back by the reference
    tmp = os.path.join(HERE, "_tmp_grid")
    api.write_crava_file(tmp + ".crava", cube, list(geom), nx, ny)
    with open(tmp + ".crava", "rb") as f:
        ours_crava = f.read()
    h = api.StormHeader()
    h.zone_number, h.model_file, h.missing_code, h.variable = 0, b"ModelFile", -999.25, b"Vp"
    h.x_min, h.lx, h.y_min, h.ly = hdr["x_min"], hdr["lx"], hdr["y_min"], hdr["ly"]
    h.z_top, h.z_bot, h.erosion_top, h.erosion_bot = hdr["z_top"], hdr["z_bot"], hdr["erosion_top"], hdr["erosion_bot"]
    h.lz, h.angle_deg = hdr["z_bot"] - hdr["z_top"], hdr["angle_deg"]
    api.write_storm(tmp + ".storm", values, h)
    with open(tmp + ".storm", "rb") as f:
        ours_storm = f.read()
    os.remove(tmp + ".crava")
    os.remove(tmp + ".storm")
    read_crava = o2.crava_read(ours_crava, nxp, nyp, nzp)
    read_storm, read_hdr = o2.storm_read(ours_storm)
    np.savez_compressed(os.path.join(HERE, name), cube=cube, geom=geom, nx=nx, ny=ny, nxp=nxp, nyp=nyp, nzp=nzp,
                        crava_bytes=np.frombuffer(crava_bytes, np.uint8), values=values,
                        storm_header=np.array([hdr[k] for k in o2.STORM_PARAMS]),
                        storm_bytes=np.frombuffer(storm_bytes, np.uint8), read_crava=read_crava,
                        read_storm=read_storm, read_storm_header=np.array([read_hdr[k] for k in sorted(read_hdr)]),
                        read_storm_keys=np.array(sorted(read_hdr)))


def storm_surface_case(name):
    """A STORM grid whose top and bottom surfaces are regular surfaces written to files beside it: the
    reference's StormContGrid::WriteToFile output (grid and surface files) and its ReadFromFile view of the
    library's files."""
    from crava_gb300 import api
    rng = np.random.default_rng(19)
    hdr = dict(zone=2, missing=-999.25, x_min=456000.0, lx=1600.0, y_min=6780000.0, ly=1200.0, z_top=0.0,
               z_bot=0.0, erosion_top=1750.0, erosion_bot=2450.5, angle_deg=12.5)
    values = rng.standard_normal((3, 4, 5)).astype(np.float32)
    surf_geom = np.array([455700.0, 6779950.0, 1900.0, 1600.0])  # covers the rotated volume
    yy, xx = np.mgrid[0:4, 0:6]
    top = 1800.0 + 3.25 * xx - 1.5 * yy + rng.uniform(-2, 2, (4, 6))
    bot = top + 600.0 + 0.125 * xx * yy
    top[2, 3] = -999.0  # a missing node
    ref = o2.storm_write_surf(values, top, bot, surf_geom, **hdr)
    tmpdir = os.path.join(HERE, "_tmp_surf")
    os.makedirs(tmpdir, exist_ok=True)
    h = api.StormHeader()
    h.zone_number, h.model_file, h.missing_code, h.variable = 2, b"ModelFile", -999.25, b"Vp"
    h.x_min, h.lx, h.y_min, h.ly = hdr["x_min"], hdr["lx"], hdr["y_min"], hdr["ly"]
    h.erosion_top, h.erosion_bot = hdr["erosion_top"], hdr["erosion_bot"]
    h.lz, h.angle_deg = float(np.max(bot) - np.min(top[top > -999])), hdr["angle_deg"]
    surfs = {"z_top_file": api.StormSurface(top, *surf_geom), "z_bot_file": api.StormSurface(bot, *surf_geom)}
    api.write_storm(os.path.join(tmpdir, "out.storm"), values, h, surfaces=surfs)
    ours = {}
    for n in sorted(os.listdir(tmpdir)):
        with open(os.path.join(tmpdir, n), "rb") as f:
            ours[n] = f.read()
        os.remove(os.path.join(tmpdir, n))
    os.rmdir(tmpdir)
    files = dict(ours)
    files["in.storm"] = files.pop("out.storm")
    read_values, read_surf = o2.storm_read_surf(files)
    out = dict(values=values, top=top, bot=bot, surf_geom=surf_geom, header=np.array([hdr[k] for k in o2.STORM_PARAMS]),
               ref_names=np.array(sorted(ref)), read_values=read_values, read_top=read_surf["top"][0],
               read_top_geom=read_surf["top"][1], read_bot=read_surf["bot"][0], read_bot_geom=read_surf["bot"][1])
    for i, n in enumerate(sorted(ref)):
        out[f"ref_file{i}"] = np.frombuffer(ref[n], np.uint8)
    np.savez_compressed(os.path.join(HERE, name), **out)


def factorable_case(name):
    ns = np.array(list(range(1, 260)) + [341, 343, 500, 511, 625, 1000, 1023, 1025, 2047, 4097, 10000], np.int32)
    np.savez_compressed(os.path.join(HERE, name), n=ns, closest=o2.closest_factorable(ns))


def inversion_4d_case(name, tl, vintage=0):
    """The 4D branch of the bin loop (findParameterVariances, src/seismicparametersholder.cpp:366-373) on
    the merged current-state spectra of a time-lapse prior (State4D::merge restated in the oracle)."""
    from crava_gb300.pipeline import SS_PAIRS, SD_PAIRS, DD_PAIRS, MERGE_TO_BIN
    F = tl.sigma_full

    def spec(i, j):
        c = O.fill_param_corr(tl.nxp, tl.nyp, tl.nzp, tl.corr_xy, tl.circ_corr_t, 0, 0, np.float32(F[i, j]))
        return O.ref_fft3d_r2c(c, tl.nxp, O.COVARIANCE)
    ss = [spec(i, j) for i, j in SS_PAIRS]
    sd = [spec(i, j) for i, j in SD_PAIRS]
    dd = [spec(i, j) for i, j in DD_PAIRS]
    _, rnxp = O.dims(tl.nxp)
    mu_s = []
    for p in range(3):
        m = np.zeros((tl.nzp, tl.nyp, rnxp), np.float32)
        m[:, :, :tl.nxp] = np.float32(tl.mu_static[p])
        mu_s.append(O.ref_fft3d_r2c(m, tl.nxp, O.PARAMETER))
    mu_d = [np.zeros_like(mu_s[0]) for _ in range(3)]
    mu_cur, cov_cur = O.state4d_merge(mu_s, mu_d, ss, sd, dd, prec="f")
    cov_bin = [cov_cur[t] for t in MERGE_TO_BIN]
    v = tl.vintages[vintage]
    tab, _ = reference_tables(tl.wavelets, tl.A, tl.theta_deg, tl.nz, tl.nzp, tl.dt_ms, tl.low_cut, tl.high_cut)
    data = [O.ref_fft3d_r2c(d, tl.nxp, O.DATA) for d in v["data"]]
    ec = O.ref_fft3d_r2c(O.fill_err_corr(tl.nxp, tl.nyp, tl.nzp, tl.corr_xy), tl.nxp, O.COVARIANCE)
    s0 = tl.sigma_current()
    res, mu, cov, nfail = O.ref_invert_bins(data, mu_cur, cov_bin, ec, dict(tab, nxp=tl.nxp), v["err_theta_cov"], s0,
                                            tl.wnc,
                                            is4d=True)
    out = dict(nxp=tl.nxp, nyp=tl.nyp, nzp=tl.nzp, theta_deg=np.array(tl.theta_deg), sigma0=s0,
               err_theta_cov=v["err_theta_cov"], wnc=tl.wnc, K=tab["K"], em1=tab["em1"], em2=tab["em2"],
               em3=tab["em3"], band=tab["band"], data_spec=np.stack(data), mean_spec=np.stack(mu_cur),
               cov_spec=np.stack(cov_bin), errcorr_spec=ec, out_resid=np.stack(res), out_mean=np.stack(mu),
               out_cov=np.stack(cov), nfail=nfail, is4d=1)
    np.savez_compressed(os.path.join(HERE, name), **out)
    # State4D::merge and State4D::split by the reference's own code on this state and posterior
    state27 = np.stack(mu_s + mu_d + ss + sd + dd)
    bin_to_merge = [0, 3, 4, 1, 5, 2]
    post9 = np.stack(list(mu) + [cov[t] for t in bin_to_merge])
    merged, split = o2.state4d(state27, post9, tl.nxp)
    np.savez_compressed(os.path.join(HERE, "state4d_n4.npz"), nxp=tl.nxp, state=state27, post=post9,
                        merged=merged, split=split)


EVOLVE_E = np.block([[np.eye(3), np.zeros((3, 3))],
                     [0.1 * np.eye(3), 0.9 * np.eye(3) + 0.05 * (np.ones((3, 3)) - np.eye(3))]])
EVOLVE_C_MEAN = np.array([0.0, 0.0, 0.0, 0.01, -0.02, 0.005])
EVOLVE_C_COV = np.block([[np.zeros((3, 3)), np.zeros((3, 3))],
                         [np.zeros((3, 3)), 4e-4 * np.array([[1.0, 0.3, 0.2], [0.3, 1.0, 0.25], [0.2, 0.25, 1.0]])]])


def evolve_case(name):
    """State4D::evolve by the reference's own code (crava_o2) with one time step of a time evolution (the
    dynamic part decays, couples to the static part, gains a mean shift and a covariance increment) on the
    split state of state4d_n4.npz, and the increment's correlation cube evolve builds (fillInGenExpCorr)."""
    g = np.load(os.path.join(HERE, "state4d_n4.npz"))
    state = g["split"]
    nx, ny, nz, nxp = 16, 12, 11, int(g["nxp"])
    ev, gr, gs = o2.state4d_evolve(state, nx, ny, nz, nxp, EVOLVE_E, EVOLVE_C_MEAN, EVOLVE_C_COV)
    np.savez_compressed(os.path.join(HERE, name), nx=nx, ny=ny, nz=nz, nxp=nxp, state=state, E=EVOLVE_E,
                        c=EVOLVE_C_MEAN, C=EVOLVE_C_COV, evolved=ev, genexp_real=gr, genexp_spec=gs)


def local_noise_case(name, n, dims, seed):
    """Crava::computeG + Crava::correctAlphaBetaRho by the reference's own code (crava_o2) on a posterior that
    differs from the prior mean by noise, local noise scales that vary over the traces (one RMISSING cell),
    and posterior variances at the origin between 30 and 70 % of the prior."""
    nx, ny, nz, nxp, nyp, nzp = dims
    sc = S.make_scenario(nx, ny, nz, list(np.linspace(5, 40, n)), 28.0, nxp=nxp, nyp=nyp, nzp=nzp, seed=seed)
    Sm = sc.sigma0.astype(np.float64)
    rng = np.random.default_rng(seed)
    Q = np.linalg.cholesky(Sm)
    B = rng.standard_normal((3, 3)) * 0.1
    F = np.eye(3) * 0.55 + (B + B.T) * 0.1
    Smd = Q @ F @ F.T @ Q.T
    Smd = 0.5 * (Smd + Smd.T)
    yy, xx = np.mgrid[0:ny, 0:nx]
    scale = np.stack([1.0 + 0.8 * (0.5 + 0.5 * np.sin(xx / 3.0 + l) * np.cos(yy / 4.0)) for l in range(n)])
    scale[0, 1, 1] = -99999.0
    post = [m + 0.02 * rng.standard_normal(m.shape).astype(np.float32) for m in sc.mean]
    G, out = o2.local_noise(post, sc.mean, nx, ny, nz, nxp, sc.err_theta_cov, Sm, Smd, scale)
    np.savez_compressed(os.path.join(HERE, name), nx=nx, ny=ny, nz=nz, nxp=nxp, nyp=nyp, nzp=nzp,
                        err_theta_cov=sc.err_theta_cov, prior_var0=Sm, post_var0=Smd, scale=scale,
                        post=np.stack(post), mean=np.stack(sc.mean), G=G, out=np.stack(out))


def fill_in_data_case(name, seed):
    """FFTGrid::fillInData by the reference's own code (crava_o2) from a STORM grid onto a constant-thickness
    simbox, for a DATA cube (guard-zone taper) and a PARAMETER cube (end extrapolation and trend): the grid starts
    80 ms above the simbox and ends 48 ms below it, and covers 80 % of it along x, so the columns beyond are
    outside; the parameter traces have leading and trailing zeros."""
    rng = np.random.default_rng(seed)
    nx, ny, nz, nxp, nyp, nzp = 18, 14, 40, 24, 20, 50
    dx = dy = 25.0
    dz = 4.0
    sbox = (0.0, 0.0, 1000.0, nx * dx, ny * dy, nz * dz, 0.0, dx, dy, dz)
    gnx, gny, gnk = 15, ny, nz + 32
    gbox = (0.0, 0.0, 1000.0 - 80.0, gnx * dx, gny * dy, gnk * dz)
    t = np.arange(gnk)
    out = {}
    for kind, ctype in (("data", O.DATA), ("param", O.PARAMETER)):
        v = np.zeros((gnk, gny, gnx), np.float32)
        for j in range(gny):
            for i in range(gnx):
                if kind == "data":
                    tr = sum(rng.uniform(0.3, 1.0) * np.sin(2 * np.pi * rng.uniform(0.02, 0.12) * t + rng.uniform(0, 6))
                             for _ in range(3))
                else:
                    tr = 8.0 + 0.002 * t + 0.05 * np.sin(2 * np.pi * 0.03 * t + 0.1 * i + 0.2 * j)
                    tr[:int(rng.integers(0, 6))] = 0.0
                    tr[gnk - int(rng.integers(0, 5)):] = 0.0
                v[:, j, i] = tr
        cube, traces, state, z0d, dzd, z0g, dzg, counts = o2.fill_in_data(v, gbox, nx, ny, nz, nxp, nyp, nzp, sbox,
                                                                         ctype, 20.0)
        out.update({f"{kind}_values": v, f"{kind}_cube": cube, f"{kind}_traces": traces, f"{kind}_state": state,
                    f"{kind}_z0_data": z0d, f"{kind}_dz_data": dzd, f"{kind}_z0_grid": z0g,
                    f"{kind}_dz_grid": dzg, f"{kind}_counts": counts})
    np.savez_compressed(os.path.join(HERE, name), nx=nx, ny=ny, nz=nz, nxp=nxp, nyp=nyp, nzp=nzp,
                        smooth_length=20.0, **out)


def interpolate_case(name, seed):
    """FFTGrid::interpolateSeismic by the reference's own code (crava_o2): dead traces alone, in pairs, on the
    simbox edge and at a corner, and traces of low energy, with energy thresholds 0 and 0.3."""
    rng = np.random.default_rng(seed)
    nx, ny, nz, nxp, nyp, nzp = 14, 11, 20, 18, 15, 25
    rnxp = 2 * (nxp // 2 + 1)
    cube = rng.uniform(-1.5, 1.5, (nzp, nyp, rnxp)).astype(np.float32)
    for (j, i) in ((2, 3), (5, 5), (5, 6), (0, 0), (0, 1), (1, 0), (10, 13), (7, 0), (4, 13)):
        cube[:, j, i] = 0.0
    for (j, i) in ((8, 8), (3, 10)):
        cube[:, j, i] *= 0.2
    outs = {f"out_{t:g}": o2.interpolate_seismic(cube, nx, ny, nz, nxp, t) for t in (0.0, 0.3)}
    np.savez_compressed(os.path.join(HERE, name), nx=nx, ny=ny, nz=nz, nxp=nxp, nyp=nyp, nzp=nzp, cube=cube,
                        thresholds=np.array([0.0, 0.3]), **outs)


def divide_case(name, seed):
    """Crava::divideDataByScaleWavelet by the reference's own code (crava_o2): 3 stacks over a simbox whose
    relative thickness varies from 0.7 to 1 (a bottom surface on 4 x 3 nodes), local wavelet shifts of up to 4 ms
    and gains 0.85-1.2, two dead traces, energy threshold 0 (interpolateSeismic after the division); then the
    reference's multiplyDataByScaleWaveletAndWriteToFile on the divided cubes (mult)."""
    sc = S.make_scenario(14, 10, 30, [10.0, 20.0, 30.0], 30.0, nxp=18, nyp=14, nzp=40, seed=seed)
    rng = np.random.default_rng(seed)
    data = [d.copy() for d in sc.data]
    for (j, i) in ((3, 4), (7, 11)):
        for dd in data:
            dd[:, j, i] = 0.0
    from dataclasses import replace
    sc = replace(sc, data=data)
    thick = np.array([[1.0, 0.9, 0.8, 0.85], [0.95, 0.75, 0.7, 0.8], [0.9, 0.85, 0.9, 1.0]])
    shift = rng.uniform(-4.0, 4.0, (sc.ntheta, sc.ny, sc.nx)).astype(np.float32)
    gain = rng.uniform(0.85, 1.2, (sc.ntheta, sc.ny, sc.nx)).astype(np.float32)
    out, rel, lz, wav, gn, ctf, mult = o2.divide_scale_wavelet(sc, sc.corr_t, sc.min_int_fq, 30.0, thick, shift, gain,
                                                               0.0)
    np.savez_compressed(os.path.join(HERE, name), nx=sc.nx, ny=sc.ny, nz=sc.nz, nxp=sc.nxp, nyp=sc.nyp, nzp=sc.nzp,
                        dt_ms=sc.dt_ms, low_cut=sc.low_cut, high_cut=sc.high_cut, wnc=sc.wnc, A=sc.A,
                        sigma0=sc.sigma0, err_theta_cov=sc.err_theta_cov, data=np.stack(data), shift=shift,
                        gain=gain, gain_normalised=gn, rel_thick=rel, lz=lz, wavelets=wav, corr_t_filtered=ctf,
                        out=np.stack(out), mult=np.stack(mult))


def simulation_case(name, inv, seed):
    nxp, nyp, nzp = int(inv["nxp"]), int(inv["nyp"]), int(inv["nzp"])
    noise = O.ref_fill_complex_noise(nxp, nyp, nzp, seed, 3)
    z = O.ref_simulate_bins(list(inv["out_cov"]), list(noise))
    fields = [O.ref_fft3d_c2r(s, nxp, O.PARAMETER) for s in z]
    np.savez_compressed(os.path.join(HERE, name), seed=seed, noise=noise, sim_spec=np.stack(z),
                        sim_real=np.stack(fields))


def main():
    src = os.environ.get("CRAVA_REFERENCE_SRC")
    if not src:
        raise SystemExit("set CRAVA_REFERENCE_SRC to the reference checkout")
    O.build_ref()
    o2.build(src)
    only = set(sys.argv[1:])  # fixture names to (re)write; all when none are given
    if only:
        if "reference_localnoise.npz" in only:
            local_noise_case("reference_localnoise.npz", 5, (21, 17, 24, 24, 20, 30), 15)
        if "reference_fillindata.npz" in only:
            fill_in_data_case("reference_fillindata.npz", 16)
        if "reference_interpolate.npz" in only:
            interpolate_case("reference_interpolate.npz", 17)
        if "reference_divide.npz" in only:
            divide_case("reference_divide.npz", 18)
        if "inversion_grad.npz" in only:
            gradient_case("inversion_grad.npz")
        if "reference_storm_surfaces.npz" in only:
            storm_surface_case("reference_storm_surfaces.npz")
        if "state4d_evolve.npz" in only:
            evolve_case("state4d_evolve.npz")
        print("fixtures written to", HERE)
        return
    fft_case("fft_even.npz", 16, 12, 20, 11)
    fft_case("fft_odd.npz", 15, 9, 7, 12)
    fft_case("fft_mixed.npz", 40, 21, 25, 13)
    sc = S.make_scenario(16, 12, 20, [10.0, 20.0, 30.0], 30.0, nxp=20, nyp=15, nzp=24, seed=3)
    inv = inversion_case("inversion_c0small.npz", sc, 30.0)
    sc5 = S.make_scenario(20, 16, 26, [0.0, 10.0, 20.0, 30.0, 40.0], 25.0, nxp=24, nyp=20, nzp=32, sn=3.0,
                          notches_hz=(2.0, 80.0), low_cut=1.0, high_cut=100.0, seed=4)
    inversion_case("inversion_c1small.npz", sc5, 25.0)
    sc8 = S.make_scenario(9, 10, 12, [5.0 * i for i in range(8)], 35.0, nxp=12, nyp=14, nzp=15, sn=2.5, seed=5)
    inversion_case("inversion_n8odd.npz", sc8, 35.0)
    wavelet_case("reference_wavelets.npz")
    adjustment_case("reference_adjustment.npz")
    factorable_case("reference_factorable.npz")
    file_format_case("reference_file_formats.npz")
    simulation_case("simulation_c0small.npz", inv, 231171)
    tl = S.make_timelapse(16, 12, 11, [0.0, 40.0 / 3, 80.0 / 3, 40.0], 25.0, nxp=20, nyp=15, nzp=14, seed=8)
    inversion_4d_case("inversion_4d_n4.npz", tl)
    local_noise_case("reference_localnoise.npz", 5, (21, 17, 24, 24, 20, 30), 15)
    fill_in_data_case("reference_fillindata.npz", 16)
    interpolate_case("reference_interpolate.npz", 17)
    divide_case("reference_divide.npz", 18)
    gradient_case("inversion_grad.npz")
    storm_surface_case("reference_storm_surfaces.npz")
    evolve_case("state4d_evolve.npz")
    r = O.ref_rnorm01_seq(231171, 4096)
    np.savez_compressed(os.path.join(HERE, "rnorm01.npz"), seed=231171, draws=r)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
