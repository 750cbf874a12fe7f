"""The CPU oracle against vectors produced by the reference's own compiled code.

The fixtures in tests/golden were generated by tests/golden/make_golden.py from
the reference's FFTW 2.1.2, lib_matr.c and RandomGen.  These tests pin the C
restatement (oracle/cravaoracle.c) that every GPU parity test uses.
"""
import numpy as np
import pytest

from conftest import golden

FFT_TOL = 1e-6     # FP32 transforms, different factorisations: relative L2


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.mark.parametrize("case", ["fft_even.npz", "fft_odd.npz", "fft_mixed.npz"])
def test_fft_matches_reference_fftw(oracle, case):
    g = golden(case)
    nxp = int(g["nxp"])
    for prec, tol in (("f", FFT_TOL), ("d", FFT_TOL)):
        a = oracle.fft3d_r2c(g["real_in"], nxp, oracle.DATA, prec)
        assert rel(a, g["r2c_data"]) < tol
        a = oracle.fft3d_r2c(g["real_in"], nxp, oracle.COVARIANCE, prec)
        assert rel(a, g["r2c_cov"]) < tol
        # complex-to-real of a spectrum that is not Hermitian on the x=0 / Nyquist planes:
        # the reference keeps only Re of those bins after the y/z transforms.
        r = oracle.fft3d_c2r(g["spec_in"], nxp, oracle.PARAMETER, prec)
        assert rel(r[:, :, :nxp], g["c2r_param"][:, :, :nxp]) < tol
        r = oracle.fft3d_c2r(g["spec_in"], nxp, oracle.COVARIANCE, prec)
        assert rel(r[:, :, :nxp], g["c2r_cov"][:, :, :nxp]) < tol


@pytest.mark.parametrize("case", ["inversion_c0small.npz", "inversion_c1small.npz", "inversion_n8odd.npz",
                                  "inversion_4d_n4.npz", "inversion_grad.npz"])
def test_bin_loop_bit_exact_vs_reference(oracle, case):
    """Same spectra in -> the FP32 restatement reproduces lib_matr bit for bit (3D and 4D branches)."""
    g = golden(case)
    tab = {k: g[k] for k in ("K", "em1", "em2", "em3", "band")}
    tab["nxp"] = int(g["nxp"])
    res, mu, cov, nf = oracle.invert_bins(list(g["data_spec"]), list(g["mean_spec"]), list(g["cov_spec"]),
                                          g["errcorr_spec"], tab, g["err_theta_cov"], g["sigma0"], float(g["wnc"]),
                                          is4d=bool(int(g["is4d"])), prec="f")
    assert nf == int(g["nfail"])
    np.testing.assert_array_equal(np.stack(res), g["out_resid"])
    np.testing.assert_array_equal(np.stack(mu), g["out_mean"])
    np.testing.assert_array_equal(np.stack(cov), g["out_cov"])


@pytest.mark.parametrize("case", ["inversion_c0small.npz", "inversion_c1small.npz"])
def test_fp64_oracle_close_to_reference(oracle, case):
    g = golden(case)
    tab = {k: g[k].astype(np.complex128) if g[k].dtype == np.complex64 else g[k]
           for k in ("K", "em1", "em2", "em3", "band")}
    tab["nxp"] = int(g["nxp"])
    res, mu, cov, nf = oracle.invert_bins(list(g["data_spec"]), list(g["mean_spec"]), list(g["cov_spec"]),
                                          g["errcorr_spec"], tab, g["err_theta_cov"], g["sigma0"], float(g["wnc"]),
                                          prec="d")
    upd_ref = g["out_mean"] - g["mean_spec"]
    upd = np.stack(mu) - g["mean_spec"]
    assert rel(upd, upd_ref) < 1e-3
    assert rel(np.stack(cov), g["out_cov"]) < 1e-4


@pytest.mark.parametrize("case", ["inversion_c0small.npz", "inversion_c1small.npz", "inversion_n8odd.npz"])
def test_k_tables_match_reference_fill_err_mult_vectors(oracle, case):
    """The oracle's restatement of the per-k tables against the reference's own Crava::fillErrMultVectors
    (constant-thickness branch) on the same resampled wavelets.  The reference transforms the wavelets in
    FP32 (FFTW 2.1.2 float), the restatement in FP64 before rounding: entries agree to FP32 rounding of
    the table's scale."""
    g = golden(case)
    tab = oracle.k_tables(int(g["nxp"]), g["wavelets"], g["A"], int(g["nz"]), int(g["nzp"]), float(g["dt_ms"]),
                          float(g["low_cut"]), float(g["high_cut"]))
    np.testing.assert_array_equal(tab["band"], g["band"])
    for k in ("K", "em1", "em2", "em3"):
        assert np.abs(tab[k] - g[k]).max() <= 1e-6 * np.abs(g[k]).max(), k


def test_noise_generator_bit_exact(oracle):
    g = golden("rnorm01.npz")
    np.testing.assert_array_equal(oracle.rnorm01_seq(int(g["seed"]), g["draws"].size), g["draws"])
    s = golden("simulation_c0small.npz")
    inv = golden("inversion_c0small.npz")
    noise = oracle.fill_complex_noise(int(inv["nxp"]), int(inv["nyp"]), int(inv["nzp"]), int(s["seed"]), 3)
    np.testing.assert_array_equal(noise, s["noise"])


def test_simulation_bins_bit_exact(oracle):
    s = golden("simulation_c0small.npz")
    inv = golden("inversion_c0small.npz")
    z = oracle.simulate_bins(list(inv["out_cov"]), list(s["noise"]), prec="f")
    np.testing.assert_array_equal(np.stack(z), s["sim_spec"])
    nxp = int(inv["nxp"])
    f = [oracle.fft3d_c2r(x, nxp, oracle.PARAMETER) for x in z]
    assert rel(np.stack(f)[..., :nxp], s["sim_real"][..., :nxp]) < FFT_TOL


def test_find_closest_factorable(oracle):
    from crava_gb300.synthetic import find_closest_factorable
    for n in [1, 2, 7, 8, 11, 13, 49, 80, 81, 100, 121, 143, 200, 240, 256, 257, 511, 1000]:
        assert oracle.find_closest_factorable(n) == find_closest_factorable(n)
