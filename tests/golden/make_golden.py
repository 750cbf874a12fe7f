"""Generate the golden fixtures in this directory from the reference build.

Run where the CRAVA reference checkout exists (it builds oracle/_ref from the
reference's own FFTW 2.1.2, lib_matr.c and random.cpp):

    python tests/golden/make_golden.py

Every output array comes from the reference's compiled code (see
oracle/ref_harness.cpp); the inputs are seeded synthetic cubes.  The fixtures
are small so the CPU suite stays fast, and they travel to machines without the
reference checkout, where they are the only reference-generated vectors.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import oracle as O  # noqa: E402
from crava_gb300 import synthetic as S  # noqa: E402


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


def inversion_case(name, sc, is4d=False):
    tab = O.k_tables(sc.nxp, sc.wavelets, sc.A, sc.nz, sc.nzp, sc.dt_ms, sc.low_cut, sc.high_cut)
    data = [O.ref_fft3d_r2c(d, sc.nxp, O.DATA) for d in sc.data]
    mean = [O.ref_fft3d_r2c(m, sc.nxp, O.PARAMETER) for m in sc.mean]
    covs = []
    for (p, q) in [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]:
        c = O.fill_param_corr(sc.nxp, sc.nyp, sc.nzp, sc.corr_xy, sc.circ_corr_t, 0, 0, np.float32(sc.sigma0[p, q]))
        covs.append(O.ref_fft3d_r2c(c, sc.nxp, O.COVARIANCE))
    ec = O.ref_fft3d_r2c(O.fill_err_corr(sc.nxp, sc.nyp, sc.nzp, sc.corr_xy), sc.nxp, O.COVARIANCE)
    res, mu, cov, nfail = O.ref_invert_bins(data, mean, covs, ec, tab, sc.err_theta_cov, sc.sigma0, sc.wnc,
                                            is4d=is4d)
    post_real = [O.ref_fft3d_c2r(m, sc.nxp, O.PARAMETER) for m in mu]
    out = dict(nx=sc.nx, ny=sc.ny, nz=sc.nz, nxp=sc.nxp, nyp=sc.nyp, nzp=sc.nzp, dt_ms=sc.dt_ms,
               theta_deg=np.array(sc.theta_deg), A=sc.A, wavelets=sc.wavelets, corr_xy=sc.corr_xy,
               circ_corr_t=sc.circ_corr_t, sigma0=sc.sigma0, err_theta_cov=sc.err_theta_cov, wnc=sc.wnc,
               low_cut=sc.low_cut, high_cut=sc.high_cut,
               data_real=np.stack(sc.data), mean_real=np.stack(sc.mean),
               K=tab["K"], em1=tab["em1"], em2=tab["em2"], em3=tab["em3"], band=tab["band"],
               data_spec=np.stack(data), mean_spec=np.stack(mean), cov_spec=np.stack(covs), errcorr_spec=ec,
               out_resid=np.stack(res), out_mean=np.stack(mu), out_cov=np.stack(cov), out_mean_real=np.stack(post_real),
               nfail=nfail, is4d=int(is4d))
    np.savez_compressed(os.path.join(HERE, name), **out)
    return out


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
    tab = O.k_tables(tl.nxp, tl.wavelets, tl.A, tl.nz, tl.nzp, tl.dt_ms, tl.low_cut, tl.high_cut)
    data = [O.ref_fft3d_r2c(d, tl.nxp, O.DATA) for d in v["data"]]
    ec = O.ref_fft3d_r2c(O.fill_err_corr(tl.nxp, tl.nyp, tl.nzp, tl.corr_xy), tl.nxp, O.COVARIANCE)
    s0 = tl.sigma_current()
    res, mu, cov, nfail = O.ref_invert_bins(data, mu_cur, cov_bin, ec, tab, v["err_theta_cov"], s0, tl.wnc,
                                            is4d=True)
    out = dict(nxp=tl.nxp, nyp=tl.nyp, nzp=tl.nzp, theta_deg=np.array(tl.theta_deg), sigma0=s0,
               err_theta_cov=v["err_theta_cov"], wnc=tl.wnc, K=tab["K"], em1=tab["em1"], em2=tab["em2"],
               em3=tab["em3"], band=tab["band"], data_spec=np.stack(data), mean_spec=np.stack(mu_cur),
               cov_spec=np.stack(cov_bin), errcorr_spec=ec, out_resid=np.stack(res), out_mean=np.stack(mu),
               out_cov=np.stack(cov), nfail=nfail, is4d=1)
    np.savez_compressed(os.path.join(HERE, name), **out)


def simulation_case(name, inv, seed):
    nxp, nyp, nzp = int(inv["nxp"]), int(inv["nyp"]), int(inv["nzp"])
    noise = O.ref_fill_complex_noise(nxp, nyp, nzp, seed, 3)
    z = O.ref_simulate_bins(list(inv["out_cov"]), list(noise))
    fields = [O.ref_fft3d_c2r(s, nxp, O.PARAMETER) for s in z]
    np.savez_compressed(os.path.join(HERE, name), seed=seed, noise=noise, sim_spec=np.stack(z),
                        sim_real=np.stack(fields))


def main():
    O.build_ref()
    fft_case("fft_even.npz", 16, 12, 20, 11)
    fft_case("fft_odd.npz", 15, 9, 7, 12)
    fft_case("fft_mixed.npz", 40, 21, 25, 13)
    sc = S.make_scenario(16, 12, 20, [10.0, 20.0, 30.0], 30.0, nxp=20, nyp=15, nzp=24, seed=3)
    inv = inversion_case("inversion_c0small.npz", sc)
    sc5 = S.make_scenario(20, 16, 26, [0.0, 10.0, 20.0, 30.0, 40.0], 25.0, nxp=24, nyp=20, nzp=32, sn=3.0,
                          notches_hz=(2.0, 80.0), low_cut=1.0, high_cut=100.0, seed=4)
    inversion_case("inversion_c1small.npz", sc5)
    sc8 = S.make_scenario(9, 10, 12, [5.0 * i for i in range(8)], 35.0, nxp=12, nyp=14, nzp=15, sn=2.5, seed=5)
    inversion_case("inversion_n8odd.npz", sc8)
    simulation_case("simulation_c0small.npz", inv, 231171)
    tl = S.make_timelapse(16, 12, 11, [0.0, 40.0 / 3, 80.0 / 3, 40.0], 25.0, nxp=20, nyp=15, nzp=14, seed=8)
    inversion_4d_case("inversion_4d_n4.npz", tl)
    r = O.ref_rnorm01_seq(231171, 4096)
    np.savez_compressed(os.path.join(HERE, "rnorm01.npz"), seed=231171, draws=r)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
