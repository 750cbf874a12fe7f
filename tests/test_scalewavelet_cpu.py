"""Non-constant simbox thickness, CPU side: the oracle's FP32 and FP64 restatements agree, the host
tables (C++) match the oracle and numpy, and the interpolation oracle gives the hand-computed answers."""
import numpy as np
import pytest

from conftest import rel


def _scenario(seed=5):
    from crava_gb300 import synthetic as S
    sc = S.make_scenario(20, 16, 24, [10.0, 20.0, 30.0], 30.0, nxp=24, nyp=20, nzp=30, seed=seed)
    yy, xx = np.mgrid[0:sc.nyp, 0:sc.nxp]
    rt = (1.0 + 0.25 * np.sin(xx / 5.0) * np.cos(yy / 4.0)).astype(np.float32)
    return sc, rt


@pytest.mark.parametrize("surfaces", [False, True])
def test_oracle_divide_and_multiply_fp32_vs_fp64(oracle, surfaces):
    sc, rt = _scenario()
    shift = gain = None
    if surfaces:
        shift = (2.0 * np.sin(np.arange(sc.nx * sc.ny) / 7.0)).astype(np.float32).reshape(sc.ny, sc.nx)
        gain = (1.0 + 0.1 * np.cos(np.arange(sc.nx * sc.ny) / 5.0)).astype(np.float32).reshape(sc.ny, sc.nx)
    lz = sc.nz * sc.dt_ms
    out = {p: oracle.divide_scale_wavelet(sc.data[0], sc.nx, sc.ny, sc.nz, sc.wavelets[0], sc.A[0], sc.sigma0,
                                          sc.circ_corr_t, sc.dt_ms, lz, sc.low_cut, sc.high_cut, sc.wnc,
                                          float(sc.err_theta_cov[0, 0]), rt, shift, gain, prec=p) for p in "fd"}
    assert rel(out["f"][:, :, :sc.nxp], out["d"][:, :, :sc.nxp]) < 1e-6
    m = {p: oracle.multiply_scale_wavelet(out["d"], sc.nx, sc.ny, sc.wavelets[0], sc.dt_ms, rt, shift, gain, prec=p)
         for p in "fd"}
    assert rel(m["f"][:, :, :sc.nxp], m["d"][:, :, :sc.nxp]) < 1e-6
    # a unit relative thickness without surfaces leaves the local wavelet equal to the global one: the
    # multiply of a divided cube is then a band-limited filter of the data, not the identity, but the
    # divide of an all-zero cube is exactly zero
    z = np.zeros_like(sc.data[0])
    zo = oracle.divide_scale_wavelet(z, sc.nx, sc.ny, sc.nz, sc.wavelets[0], sc.A[0], sc.sigma0, sc.circ_corr_t,
                                     sc.dt_ms, lz, sc.low_cut, sc.high_cut, sc.wnc, float(sc.err_theta_cov[0, 0]), rt,
                                     prec="f")
    assert not zo.any()


def test_host_operator_tables_non_constant_thickness(oracle, native):
    from crava_gb300 import api
    sc, rt = _scenario()
    lz = sc.nz * sc.dt_ms
    mrt = float(rt.min())
    t = api.operator_tables_nct(sc.wavelets, sc.A, sc.nz, sc.nzp, sc.dt_ms, sc.low_cut, sc.high_cut, mrt)
    o = oracle.k_tables_nct(sc.nxp, sc.wavelets.astype(np.float64), sc.A, sc.nz, sc.nzp, lz, sc.low_cut, sc.high_cut,
                            mrt, prec="d")
    assert np.array_equal(t["band"], o["band"])
    bd = o["band"].astype(bool)
    for k in ("K", "em1", "em2", "em3"):
        assert rel(t[k][bd], o[k][bd]) < 1e-6, k
    # K = kD * A: no wavelet in the forward operator of this branch
    kD = np.fft.fft(np.r_[-1.0, np.zeros(sc.nzp - 2), 1.0])
    assert rel(t["K"][:, 0, 1], kD * sc.A[0, 1]) < 1e-6
    # a lower minimum thickness widens the band at the low end only
    t2 = api.operator_tables_nct(sc.wavelets, sc.A, sc.nz, sc.nzp, sc.dt_ms, sc.low_cut, sc.high_cut, 0.3)
    assert t2["band"].sum() >= t["band"].sum()


def test_scale_wavelet_tables_against_numpy(native):
    from crava_gb300 import api
    sc, _ = _scenario()
    lz = sc.nz * sc.dt_ms
    nzp, c = sc.nzp, sc.nzp // 2 + 1
    tab = api.scale_wavelet_tables(sc.wavelets, sc.A, sc.sigma0, sc.circ_corr_t, sc.err_theta_cov, sc.nz, sc.dt_ms,
                                   lz, sc.low_cut, sc.high_cut, sc.wnc)
    assert tab.shape[1] == native.cg_scale_wavelet_table_size(nzp) and tab.shape[1] % 4 == 0
    for l in range(sc.ntheta):
        w = sc.wavelets[l].astype(np.float64)
        W = tab[l, :2 * c].view(np.complex64)
        assert rel(W, np.fft.rfft(w)) < 1e-6
        # E3 has unit norm within the band (findNormWithinFrequencyBand)
        E = tab[l, 2 * c:4 * c].view(np.complex64).astype(np.complex128)
        dOmega = np.float32(1.0) / (np.float32(nzp) * np.float32(sc.dt_ms) * np.float32(0.001))
        lo = max(0, int(np.floor(np.float32(sc.low_cut) / dOmega)))
        hi = min(c, int(np.ceil(np.float32(sc.high_cut) / dOmega)))
        n2 = sum(2.0 / nzp * abs(E[i]) ** 2 for i in range(lo, hi)) - (abs(E[0]) ** 2 / nzp if lo == 0 else 0.0)
        assert abs(n2 - 1.0) < 1e-5
        # tau2 = |Re FFT(2 c_i - c_{i+1} - c_{i-1})| of eiVar * corrT filtered to lags < nz
        eiv = float(sc.A[l] @ sc.sigma0 @ sc.A[l])
        refk = np.minimum(np.arange(nzp), nzp - np.arange(nzp))
        ct = np.where(refk < sc.nz, sc.circ_corr_t.astype(np.float64)[refk], 0.0) * eiv
        rc = 2 * ct - np.roll(ct, -1) - np.roll(ct, 1)
        assert rel(tab[l, 4 * c:5 * c], np.abs(np.fft.rfft(rc).real)) < 1e-5
        assert abs(tab[l, 5 * c] - np.float32(np.sqrt((w * w).sum())) ** 2) < 1e-5 * tab[l, 5 * c]
        assert tab[l, 5 * c + 2] == np.float32(sc.err_theta_cov[l, l]) and tab[l, 5 * c + 3] == np.float32(sc.wnc)


def test_interpolation_oracle_known_answers(oracle):
    nx, ny, nz, nxp, nyp, nzp = 6, 5, 4, 8, 6, 6
    rnxp = 2 * (nxp // 2 + 1)
    rng = np.random.default_rng(3)
    cube = rng.uniform(0.5, 1.5, (nzp, nyp, rnxp)).astype(np.float32)
    cube[:, 2, 3] = 0.0                              # one dead trace inside
    out, n = oracle.interpolate_seismic(cube, nx, ny, nz, nxp, 0.0, prec="f")
    assert n == 1
    nb = cube[:, 2, 2] + cube[:, 2, 4] + cube[:, 1, 3] + cube[:, 3, 3]
    assert np.array_equal(out[:, 2, 3], nb / np.float32(4.0))
    # the box of good traces is the whole simbox: padding traces are the tapered edge traces
    # (extrapolateSeismic), simbox traces other than the dead one are unchanged
    keep = np.ones((ny, nx), bool)
    keep[2, 3] = False
    assert np.array_equal(out[:, :ny, :nx][:, keep], cube[:, :ny, :nx][:, keep])
    i, j, k = 6, 1, 2                                # x padding: refi = getFillNumber(6, 6, 8) = 4
    dx = np.float32(np.float32(1) / np.float32(min(nx, nxp - nx) / 2.1))
    mult = np.float32(max(1.0 - float(dx * dx), 0.0) ** 3)
    assert out[k, j, i] == mult * cube[k, j, 4]
    # a dead corner with one good neighbour at its turn of the scan is not revisited once its right
    # neighbour is interpolated (the backtrack stops at a flag below 2): it stays zero
    cube2 = cube.copy()
    cube2[:, 0, 0] = 0.0
    cube2[:, 0, 1] = 0.0
    out2, n2 = oracle.interpolate_seismic(cube2, nx, ny, nz, nxp, 0.0, prec="f")
    assert n2 == 3
    assert np.array_equal(out2[:, 0, 1], (cube2[:, 0, 2] + cube2[:, 1, 1]) / np.float32(2.0))
    assert not out2[:, 0, 0].any()
    # a dead trace after a bad one is revisited by the backtrack: (1, 0) with (0, 0) good, (1, 1) bad
    cube3 = cube.copy()
    cube3[:, 1, 0] = 0.0
    cube3[:, 1, 1] = 0.0
    cube3[:, 0, 1] = 0.0
    out3, n3 = oracle.interpolate_seismic(cube3, nx, ny, nz, nxp, 0.0, prec="f")
    assert n3 == 4
    assert out3[:, 1, 0].all() and out3[:, 1, 1].all() and out3[:, 0, 1].all()
