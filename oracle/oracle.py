"""CPU oracle for the FFT-domain AVO inversion path -- TEST INFRASTRUCTURE ONLY.

This module is the checker: tests, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` leg of ``bench.py`` call it to produce the answer the GPU
path is compared against, and to time the CPU baseline.  Nothing in the
product package imports it.

Two native libraries sit behind it:

* ``oracle/_build/libcravaoracle.so`` -- ``cravaoracle.c``, a plain-C
  restatement of the reference algorithm in FP32 (reference operation order)
  and FP64 (the FP64 oracle).  Built here and on any test machine.
* ``oracle/_ref/libcrava_ref.so`` -- the reference's own FFTW 2.1.2,
  ``lib_matr.c`` and ``RandomGen`` compiled from the reference sources by
  ``Makefile.ref`` plus ``ref_harness.cpp``.  Only buildable where the
  reference checkout exists; used to pin the restatement and to generate the
  golden fixtures in ``tests/golden``.

Array conventions follow ``FFTGrid`` (src/fftgrid.cpp:40-70): a real cube is a
``(nzp, nyp, rnxp)`` array with ``rnxp = 2*(nxp//2+1)``; its spectrum is the
same buffer viewed as ``(nzp, nyp, cnxp)`` complex.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
ORACLE_SO = os.path.join(BUILD_DIR, "libcravaoracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libcrava_ref.so")
# the reference checkout, when this machine has one: named by the caller, never assumed
REFERENCE_SRC = os.environ.get("CRAVA_REFERENCE_SRC", "")

DATA, PARAMETER, COVARIANCE, OPERATOR = 1, 2, 3, 5

_lib = None
_ref = None


def build_oracle(force: bool = False) -> str:
    """Compile cravaoracle.c (portable C, OpenMP) into oracle/_build."""
    src = [os.path.join(HERE, "cravaoracle.c"), os.path.join(HERE, "oracle_impl.inc")]
    if not force and os.path.exists(ORACLE_SO) and all(
        os.path.getmtime(ORACLE_SO) >= os.path.getmtime(s) for s in src
    ):
        return ORACLE_SO
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = ORACLE_SO + f".tmp{os.getpid()}"
    subprocess.check_call(
        ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-w",
         src[0], "-lm", "-o", tmp]
    )
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref() -> str | None:
    """Build oracle/_ref from the reference sources when they are present."""
    if not REFERENCE_SRC or not os.path.isdir(os.path.join(REFERENCE_SRC, "libs", "fft")):
        return None
    repo = os.path.dirname(HERE)
    subprocess.check_call(
        ["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"), f"REF={REFERENCE_SRC}",
         f"-j{os.cpu_count() or 4}"],
        cwd=repo,
    )
    return REF_SO


def _P(dt):
    return np.ctypeslib.ndpointer(dtype=dt, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = ct.CDLL(ORACLE_SO)
        for sfx, R in (("_f", ct.c_float), ("_d", ct.c_double)):
            PR = ct.POINTER(R)
            PPR = ct.POINTER(PR)
            getattr(L, "or_fft3d_r2c" + sfx).argtypes = [PR, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int]
            getattr(L, "or_fft3d_c2r" + sfx).argtypes = [PR, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int]
            getattr(L, "or_fft1d_c2c" + sfx).argtypes = [PR, ct.c_int, ct.c_int]
            getattr(L, "or_invert_bins" + sfx).argtypes = [
                ct.c_int, ct.c_int, ct.c_int, ct.c_int, PPR, PPR, PPR, PR, PR, PR, PR, PR,
                ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_float, ct.c_int, ct.POINTER(ct.c_int), ct.c_int]
            getattr(L, "or_simulate_bins" + sfx).argtypes = [ct.c_size_t, PPR, PPR, ct.c_int]
            getattr(L, "or_fill_in_data" + sfx).argtypes = [PR, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int,
                                                            PR, ct.c_int, ct.c_void_p, PR, PR, PR, R, R,
                                                            ct.POINTER(ct.c_int), ct.c_int]
            getattr(L, "or_state4d_merge" + sfx).argtypes = [ct.c_size_t, PPR, PPR, PPR, PPR, PPR, PPR, PPR, ct.c_int]
            getattr(L, "or_state4d_split" + sfx).argtypes = [ct.c_size_t, PPR, PPR, PPR, PPR, PPR, PPR, PPR,
                                                             ct.POINTER(ct.c_int), ct.c_int]
            getattr(L, "or_fill_param_corr" + sfx).argtypes = [PR, ct.c_int, ct.c_int, ct.c_int, PR, PR,
                                                               ct.c_float, ct.c_float, R]
            getattr(L, "or_state4d_evolve" + sfx).argtypes = [ct.c_size_t, PPR, PPR, PPR, PPR, PPR, PR,
                                                              ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int,
                                                              ct.c_int, ct.c_int, ct.c_int]
            getattr(L, "or_fill_genexp" + sfx).argtypes = [PR, ct.c_int, ct.c_int, ct.c_int, ct.c_double,
                                                           ct.c_double, ct.c_double, ct.c_float, ct.c_float]
            getattr(L, "or_fill_err_corr" + sfx).argtypes = [PR, ct.c_int, ct.c_int, ct.c_int, PR,
                                                             ct.c_float, ct.c_float]
            getattr(L, "or_k_tables" + sfx).argtypes = [
                ct.c_int, ct.c_int, ct.c_int, PR, ct.c_void_p, ct.c_float, ct.c_float, ct.c_float, ct.c_float,
                ct.c_float, PR, PR, PR, PR, ct.c_void_p]
            getattr(L, "or_circ_corr_t" + sfx).argtypes = [ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, PR]
            getattr(L, "or_k_tables_nct" + sfx).argtypes = [
                ct.c_int, ct.c_int, ct.c_int, PR, ct.c_void_p, ct.c_float, ct.c_float, ct.c_float, ct.c_float,
                PR, PR, PR, PR, ct.c_void_p]
            FP = ct.POINTER(ct.c_float)
            getattr(L, "or_divide_scale_wavelet" + sfx).argtypes = [
                PR, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, PR, FP, ct.POINTER(ct.c_double), PR,
                ct.c_float, ct.c_float, ct.c_float, ct.c_float, ct.c_float, ct.c_float, FP, FP, FP, ct.c_int]
            getattr(L, "or_adjustment_factor" + sfx).argtypes = [
                PR, PR, FP, ct.POINTER(ct.c_double), PR, ct.c_int, ct.c_int, ct.c_float, ct.c_float, ct.c_float,
                ct.c_float, ct.c_float, ct.c_float, ct.c_float, ct.c_float, ct.c_float]
            getattr(L, "or_multiply_scale_wavelet" + sfx).argtypes = [
                PR, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, PR, ct.c_float, FP, FP, FP, ct.c_int]
            getattr(L, "or_interpolate_seismic" + sfx).argtypes = [
                PR, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_float]
            getattr(L, "or_interpolate_seismic" + sfx).restype = ct.c_int
            getattr(L, "or_circ_corr_t" + sfx).restype = ct.c_int
        L.or_fill_complex_noise.argtypes = [ct.POINTER(ct.c_float), ct.c_int, ct.c_int, ct.c_int,
                                            ct.POINTER(ct.c_uint)]
        L.or_rnorm01.argtypes = [ct.POINTER(ct.c_uint)]
        L.or_rnorm01.restype = ct.c_double
        L.or_find_closest_factorable.argtypes = [ct.c_int]
        PD = ct.POINTER(ct.c_double)
        L.or_new_posterior_cov_pointwise.argtypes = [ct.c_int, PD, PD, PD, PD, PD, PD, PD]
        L.or_correct_alpha_beta_rho.argtypes = [ct.POINTER(ct.POINTER(ct.c_float)), ct.POINTER(ct.POINTER(ct.c_float)),
                                                ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, PD, PD, PD,
                                                PD, PD, PD]
        L.or_find_closest_factorable.restype = ct.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO) or bool(REFERENCE_SRC) and os.path.isdir(os.path.join(REFERENCE_SRC, "libs", "fft"))


def ref():
    """The reference build (FFTW 2.1.2 + lib_matr + RandomGen).  x86 host only."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            build_ref()
        L = ct.CDLL(REF_SO)
        PF = ct.POINTER(ct.c_float)
        PPF = ct.POINTER(PF)
        L.ref_fft3d_r2c.argtypes = [PF, ct.c_int, ct.c_int, ct.c_int, ct.c_int]
        L.ref_fft3d_c2r.argtypes = [PF, ct.c_int, ct.c_int, ct.c_int, ct.c_int]
        L.ref_fft1d_r2c.argtypes = [PF, ct.c_int]
        L.ref_chol_cpx.argtypes = [ct.c_int, PF]
        L.ref_chol_cpx.restype = ct.c_int
        L.ref_invert_bins.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_int, PPF, PPF, PPF, PF, PF, PF, PF, PF,
                                      ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_float, ct.c_int, ct.c_int]
        L.ref_invert_bins.restype = ct.c_int
        L.ref_simulate_bins.argtypes = [ct.c_long, PPF, PPF]
        L.ref_rnorm01_seq.argtypes = [ct.c_uint, ct.c_int, ct.POINTER(ct.c_double)]
        L.ref_fill_complex_noise.argtypes = [PF, ct.c_int, ct.c_int, ct.c_int, ct.c_uint, ct.c_int]
        _ref = L
    return _ref


# ----------------------------------------------------------------------------
# helpers
# ----------------------------------------------------------------------------

def dims(nxp):
    cnxp = nxp // 2 + 1
    return cnxp, 2 * cnxp


def _rdt(prec):
    return np.float32 if prec == "f" else np.float64


def _ptr(a, R):
    return a.ctypes.data_as(ct.POINTER(R))


def _pp(arrs, R):
    P = ct.POINTER(R)
    return (P * len(arrs))(*[a.ctypes.data_as(P) for a in arrs])


def _real_view(c):
    """complex (.., cnxp) -> float view of the same memory"""
    return c.view(np.float32 if c.dtype == np.complex64 else np.float64)


def pad_real(cube, nxp):
    """(nzp, nyp, nxp) real -> (nzp, nyp, rnxp) padded FFTGrid layout (pad = 0)."""
    nzp, nyp, _ = cube.shape
    _, rnxp = dims(nxp)
    out = np.zeros((nzp, nyp, rnxp), dtype=cube.dtype)
    out[:, :, :nxp] = cube
    return out


def fft3d_r2c(real_padded, nxp, cubetype, prec="f", nthreads=1):
    """FFTGrid::fftInPlace on a copy; returns the (nzp, nyp, cnxp) spectrum."""
    R = ct.c_float if prec == "f" else ct.c_double
    a = np.ascontiguousarray(real_padded, dtype=_rdt(prec)).copy()
    nzp, nyp, _ = a.shape
    getattr(lib(), "or_fft3d_r2c_" + prec)(_ptr(a, R), nxp, nyp, nzp, cubetype, nthreads)
    return a.view(np.complex64 if prec == "f" else np.complex128)


def fft3d_c2r(spec, nxp, cubetype, prec="f", nthreads=1):
    """FFTGrid::invFFTInPlace on a copy; returns the (nzp, nyp, rnxp) real cube."""
    R = ct.c_float if prec == "f" else ct.c_double
    a = np.ascontiguousarray(spec, dtype=np.complex64 if prec == "f" else np.complex128).copy()
    nzp, nyp, _ = a.shape
    r = _real_view(a)
    getattr(lib(), "or_fft3d_c2r_" + prec)(_ptr(r, R), nxp, nyp, nzp, cubetype, nthreads)
    return r


def invert_bins(data, mean, cov, errcorr, tables, errThetaCov, sigma0, wnc, is4d=False, prec="f",
                nthreads=1):
    """Bin loop of Crava::computePostMeanResidAndFFTCov on copies.

    data: list of n spectra; mean: 3; cov: 6 (00,11,22,01,02,12); errcorr: 1.
    tables: dict with K (nzp,n,3), em1/em2/em3 (nzp,n) complex and band (nzp,) uint8.
    Returns (residuals, post_mean, post_cov, n_failed_cholesky).
    """
    R = ct.c_float if prec == "f" else ct.c_double
    cdt = np.complex64 if prec == "f" else np.complex128
    d = [np.ascontiguousarray(x, dtype=cdt).copy() for x in data]
    m = [np.ascontiguousarray(x, dtype=cdt).copy() for x in mean]
    c = [np.ascontiguousarray(x, dtype=cdt).copy() for x in cov]
    e = np.ascontiguousarray(errcorr, dtype=cdt)
    nzp, nyp, cnxp = d[0].shape
    nxp = tables["nxp"]
    n = len(d)
    K = np.ascontiguousarray(tables["K"], dtype=cdt)
    e1 = np.ascontiguousarray(tables["em1"], dtype=cdt)
    e2 = np.ascontiguousarray(tables["em2"], dtype=cdt)
    e3 = np.ascontiguousarray(tables["em3"], dtype=cdt)
    band = np.ascontiguousarray(tables["band"], dtype=np.uint8)
    etc = np.ascontiguousarray(errThetaCov, dtype=np.float64)
    s0 = np.ascontiguousarray(sigma0, dtype=np.float64)
    nf = ct.c_int(0)
    rv = lambda a: _ptr(_real_view(a), R)  # noqa: E731
    getattr(lib(), "or_invert_bins_" + prec)(
        nxp, nyp, nzp, n, _pp([_real_view(x) for x in d], R), _pp([_real_view(x) for x in m], R),
        _pp([_real_view(x) for x in c], R), rv(e), rv(K), rv(e1), rv(e2), rv(e3),
        band.ctypes.data, etc.ctypes.data, s0.ctypes.data, float(wnc), int(is4d), ct.byref(nf), nthreads)
    return d, m, c, nf.value


def ref_invert_bins(data, mean, cov, errcorr, tables, errThetaCov, sigma0, wnc, is4d=False, nthreads=1):
    """Same contract as invert_bins, computed with the reference's lib_matr (FP32)."""
    R = ct.c_float
    d = [np.ascontiguousarray(x, dtype=np.complex64).copy() for x in data]
    m = [np.ascontiguousarray(x, dtype=np.complex64).copy() for x in mean]
    c = [np.ascontiguousarray(x, dtype=np.complex64).copy() for x in cov]
    e = np.ascontiguousarray(errcorr, dtype=np.complex64)
    nzp, nyp, cnxp = d[0].shape
    n = len(d)
    K = np.ascontiguousarray(tables["K"], dtype=np.complex64)
    e1 = np.ascontiguousarray(tables["em1"], dtype=np.complex64)
    e2 = np.ascontiguousarray(tables["em2"], dtype=np.complex64)
    e3 = np.ascontiguousarray(tables["em3"], dtype=np.complex64)
    band = np.ascontiguousarray(tables["band"], dtype=np.uint8)
    etc = np.ascontiguousarray(errThetaCov, dtype=np.float64)
    s0 = np.ascontiguousarray(sigma0, dtype=np.float64)
    rv = lambda a: _ptr(_real_view(a), R)  # noqa: E731
    nf = ref().ref_invert_bins(
        tables["nxp"], nyp, nzp, n, _pp([_real_view(x) for x in d], R), _pp([_real_view(x) for x in m], R),
        _pp([_real_view(x) for x in c], R), rv(e), rv(K), rv(e1), rv(e2), rv(e3),
        band.ctypes.data, etc.ctypes.data, s0.ctypes.data, float(wnc), int(is4d), nthreads)
    return d, m, c, nf


def ref_fft3d_r2c(real_padded, nxp, cubetype):
    a = np.ascontiguousarray(real_padded, dtype=np.float32).copy()
    nzp, nyp, _ = a.shape
    ref().ref_fft3d_r2c(_ptr(a, ct.c_float), nxp, nyp, nzp, cubetype)
    return a.view(np.complex64)


def ref_fft3d_c2r(spec, nxp, cubetype):
    a = np.ascontiguousarray(spec, dtype=np.complex64).copy()
    nzp, nyp, _ = a.shape
    r = a.view(np.float32)
    ref().ref_fft3d_c2r(_ptr(r, ct.c_float), nxp, nyp, nzp, cubetype)
    return r


def simulate_bins(cov6, seeds3, prec="f", nthreads=1):
    R = ct.c_float if prec == "f" else ct.c_double
    cdt = np.complex64 if prec == "f" else np.complex128
    c = [np.ascontiguousarray(x, dtype=cdt) for x in cov6]
    s = [np.ascontiguousarray(x, dtype=cdt).copy() for x in seeds3]
    getattr(lib(), "or_simulate_bins_" + prec)(c[0].size, _pp([_real_view(x) for x in c], R),
                                               _pp([_real_view(x) for x in s], R), nthreads)
    return s


def ref_simulate_bins(cov6, seeds3):
    R = ct.c_float
    c = [np.ascontiguousarray(x, dtype=np.complex64) for x in cov6]
    s = [np.ascontiguousarray(x, dtype=np.complex64).copy() for x in seeds3]
    ref().ref_simulate_bins(c[0].size, _pp([_real_view(x) for x in c], R), _pp([_real_view(x) for x in s], R))
    return s


def state4d_merge(mu_s, mu_d, ss, sd, dd, prec="f", nthreads=1):
    R = ct.c_float if prec == "f" else ct.c_double
    cdt = np.complex64 if prec == "f" else np.complex128
    args = [[np.ascontiguousarray(x, dtype=cdt) for x in grp] for grp in (mu_s, mu_d, ss, sd, dd)]
    mu_cur = [np.zeros_like(args[0][0]) for _ in range(3)]
    cov_cur = [np.zeros_like(args[0][0]) for _ in range(6)]
    pp = [_pp([_real_view(x) for x in grp], R) for grp in args + [mu_cur, cov_cur]]
    getattr(lib(), "or_state4d_merge_" + prec)(args[0][0].size, *pp, nthreads)
    return mu_cur, cov_cur


def state4d_split(mu_s, mu_d, ss, sd, dd, mu_post, cov_post6, prec="f", nthreads=1):
    R = ct.c_float if prec == "f" else ct.c_double
    cdt = np.complex64 if prec == "f" else np.complex128
    st = [[np.ascontiguousarray(x, dtype=cdt).copy() for x in grp] for grp in (mu_s, mu_d, ss, sd, dd)]
    post = [[np.ascontiguousarray(x, dtype=cdt) for x in grp] for grp in (mu_post, cov_post6)]
    nf = ct.c_int(0)
    pp = [_pp([_real_view(x) for x in grp], R) for grp in st + post]
    getattr(lib(), "or_state4d_split_" + prec)(st[0][0].size, *pp, ct.byref(nf), nthreads)
    return st, nf.value


def state4d_evolve(state27, nxp, nyp, nzp, E, c, C, lam=None, prec="f", nthreads=None):
    """State4D::evolve on the 27 state spectra (mu_s 3, mu_d 3, ss 6, sd 9, dd 6; (nzp, nyp, cnxp) complex
    each): returns the evolved copies.  E, C (6, 6), c (6,); lam the transformed increment correlation or None."""
    cdt = np.complex64 if prec == "f" else np.complex128
    R = ct.c_float if prec == "f" else ct.c_double
    st = [np.ascontiguousarray(x, dtype=cdt).copy() for x in state27]
    grp = [st[0:3], st[3:6], st[6:12], st[12:21], st[21:27]]
    pp = [_pp([_real_view(x) for x in g], R) for g in grp]
    lm = np.ascontiguousarray(lam, dtype=cdt) if lam is not None else None
    Ed, cd, Cd = (np.ascontiguousarray(x, dtype=np.float64) for x in (E, c, C))
    getattr(lib(), "or_state4d_evolve_" + prec)(st[0].size, pp[0], pp[1], pp[2], pp[3], pp[4],
                                                _ptr(_real_view(lm), R) if lm is not None else None,
                                                Ed.ctypes.data, cd.ctypes.data, Cd.ctypes.data, nxp, nyp, nzp,
                                                nthreads or os.cpu_count())
    return st


def fill_genexp(nxp, nyp, nzp, rx, ry, rz, gradI=0.0, gradJ=0.0, prec="f"):
    """FFTGrid::fillInGenExpCorr: real padded cube (nzp, nyp, rnxp)."""
    R = ct.c_float if prec == "f" else ct.c_double
    _, rnxp = dims(nxp)
    buf = np.zeros((nzp, nyp, rnxp), dtype=_rdt(prec))
    getattr(lib(), "or_fill_genexp_" + prec)(_ptr(buf, R), nxp, nyp, nzp, float(rx), float(ry), float(rz), gradI,
                                             gradJ)
    return buf


def fill_param_corr(nxp, nyp, nzp, corrXY, circCorrT, gradI=0.0, gradJ=0.0, scalar=1.0, prec="f"):
    R = ct.c_float if prec == "f" else ct.c_double
    _, rnxp = dims(nxp)
    buf = np.zeros((nzp, nyp, rnxp), dtype=_rdt(prec))
    cxy = np.ascontiguousarray(corrXY, dtype=_rdt(prec))
    ct_ = np.ascontiguousarray(circCorrT, dtype=_rdt(prec))
    getattr(lib(), "or_fill_param_corr_" + prec)(_ptr(buf, R), nxp, nyp, nzp, _ptr(cxy, R), _ptr(ct_, R),
                                                 gradI, gradJ, scalar)
    return buf


def fill_in_data(nxp, nyp, nzp, nz, is_data, traces, state, z0_data, z0_grid, dz_grid, dz_data, smooth_length,
                 prec="f", nthreads=None):
    """FFTGrid::fillInData's per-trace core: traces (nyp*rnxp, n_data), one per column i + rnxp*j.
    Returns (padded real cube (nzp, nyp, rnxp), [max leading, max trailing extrapolation])."""
    import os
    R = ct.c_float if prec == "f" else ct.c_double
    _, rnxp = dims(nxp)
    tr = np.ascontiguousarray(traces, dtype=_rdt(prec))
    ncol, n_data = tr.shape
    assert ncol == rnxp * nyp
    st = np.ascontiguousarray(state, dtype=np.uint8)
    z0d, z0g, dzg = (np.ascontiguousarray(x, dtype=_rdt(prec)) for x in (z0_data, z0_grid, dz_grid))
    buf = np.zeros((nzp, nyp, rnxp), dtype=_rdt(prec))
    ext = (ct.c_int * 2)()
    getattr(lib(), "or_fill_in_data_" + prec)(_ptr(buf, R), nxp, nyp, nzp, nz, int(is_data), _ptr(tr, R), n_data,
                                              st.ctypes.data, _ptr(z0d, R), _ptr(z0g, R), _ptr(dzg, R),
                                              dz_data, smooth_length, ext, nthreads or os.cpu_count())
    return buf, [ext[0], ext[1]]


def fill_err_corr(nxp, nyp, nzp, corrXY, gradI=0.0, gradJ=0.0, prec="f"):
    R = ct.c_float if prec == "f" else ct.c_double
    _, rnxp = dims(nxp)
    buf = np.zeros((nzp, nyp, rnxp), dtype=_rdt(prec))
    cxy = np.ascontiguousarray(corrXY, dtype=_rdt(prec))
    getattr(lib(), "or_fill_err_corr_" + prec)(_ptr(buf, R), nxp, nyp, nzp, _ptr(cxy, R), gradI, gradJ)
    return buf


def k_tables(nxp, wavelets, A, nz, nzp, dt_ms, lowCut, highCut, minRelThick=1.0, prec="f"):
    """fillErrMultVectors for every k (constant-thickness branch)."""
    R = ct.c_float if prec == "f" else ct.c_double
    cdt = np.complex64 if prec == "f" else np.complex128
    w = np.ascontiguousarray(wavelets, dtype=_rdt(prec))
    n = w.shape[0]
    A32 = np.ascontiguousarray(A, dtype=np.float32)
    K = np.zeros((nzp, n, 3), dtype=cdt)
    e1 = np.zeros((nzp, n), dtype=cdt)
    e2 = np.zeros((nzp, n), dtype=cdt)
    e3 = np.zeros((nzp, n), dtype=cdt)
    band = np.zeros(nzp, dtype=np.uint8)
    lz = nz * dt_ms
    getattr(lib(), "or_k_tables_" + prec)(n, nz, nzp, _ptr(w, R), A32.ctypes.data, dt_ms, lz, minRelThick,
                                          lowCut, highCut, _ptr(_real_view(K), R), _ptr(_real_view(e1), R),
                                          _ptr(_real_view(e2), R), _ptr(_real_view(e3), R), band.ctypes.data)
    return {"K": K, "em1": e1, "em2": e2, "em3": e3, "band": band, "nxp": nxp}


def k_tables_nct(nxp, wavelets, A, nz, nzp, lz, lowCut, highCut, minRelThick, prec="f"):
    """fillErrMultVectors for every k, non-constant-thickness branch (K = kD*A, errMult1 = 1/||w||,
    errMult2 = kD3/||e3||, errMult3 = 1/|W| robust)."""
    R = ct.c_float if prec == "f" else ct.c_double
    cdt = np.complex64 if prec == "f" else np.complex128
    w = np.ascontiguousarray(wavelets, dtype=_rdt(prec))
    n = w.shape[0]
    A32 = np.ascontiguousarray(A, dtype=np.float32)
    K = np.zeros((nzp, n, 3), dtype=cdt)
    e1 = np.zeros((nzp, n), dtype=cdt)
    e2 = np.zeros((nzp, n), dtype=cdt)
    e3 = np.zeros((nzp, n), dtype=cdt)
    band = np.zeros(nzp, dtype=np.uint8)
    getattr(lib(), "or_k_tables_nct_" + prec)(n, nz, nzp, _ptr(w, R), A32.ctypes.data, lz, minRelThick, lowCut,
                                              highCut, _ptr(_real_view(K), R), _ptr(_real_view(e1), R),
                                              _ptr(_real_view(e2), R), _ptr(_real_view(e3), R), band.ctypes.data)
    return {"K": K, "em1": e1, "em2": e2, "em3": e3, "band": band, "nxp": nxp}


def _fptr(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32).ctypes.data_as(ct.POINTER(ct.c_float))


def divide_scale_wavelet(buf, nx, ny, nz, wavelet, A, prior_var0, circ_corr_t, dz, lz, low_cut, high_cut, wnc,
                         err_var, rel_thick, shift=None, gain=None, prec="f", nthreads=None):
    """Crava::divideDataByScaleWavelet on one real padded angle cube (returns a new cube; the
    interpolateSeismic step is separate)."""
    R = ct.c_float if prec == "f" else ct.c_double
    nzp, nyp, rnxp = buf.shape
    nxp = rel_thick.shape[1]
    out = np.array(buf, dtype=_rdt(prec), order="C")
    w = np.ascontiguousarray(wavelet, dtype=_rdt(prec))
    cc = np.ascontiguousarray(circ_corr_t, dtype=_rdt(prec))
    A32 = np.ascontiguousarray(A, dtype=np.float32)
    pv = np.ascontiguousarray(prior_var0, dtype=np.float64)
    rt = np.ascontiguousarray(rel_thick, dtype=np.float32)
    keep = [np.ascontiguousarray(x, dtype=np.float32) if x is not None else None for x in (shift, gain)]
    getattr(lib(), "or_divide_scale_wavelet_" + prec)(
        _ptr(out, R), nx, ny, nz, nxp, nyp, nzp, _ptr(w, R), A32.ctypes.data_as(ct.POINTER(ct.c_float)),
        pv.ctypes.data_as(ct.POINTER(ct.c_double)), _ptr(cc, R), dz, lz, low_cut, high_cut, wnc, err_var,
        rt.ctypes.data_as(ct.POINTER(ct.c_float)), _fptr(keep[0]), _fptr(keep[1]), nthreads or os.cpu_count())
    return out


def adjustment_factor(wavelet, A, prior_var0, circ_corr_t, nz, dz, lz, low_cut, high_cut, wnc, err_var, ts, gain, sf,
                      prec="f"):
    """Crava::computeAdjustmentFactor for one local wavelet (the global one shifted by ts ms, scaled by gain,
    stretched by sf): (nzp/2+1,) complex."""
    R = ct.c_float if prec == "f" else ct.c_double
    nzp = len(wavelet)
    out = np.zeros(2 * (nzp // 2 + 1), dtype=_rdt(prec))
    w = np.ascontiguousarray(wavelet, dtype=_rdt(prec))
    cc = np.ascontiguousarray(circ_corr_t, dtype=_rdt(prec))
    A32 = np.ascontiguousarray(A, dtype=np.float32)
    pv = np.ascontiguousarray(prior_var0, dtype=np.float64)
    getattr(lib(), "or_adjustment_factor_" + prec)(
        _ptr(out, R), _ptr(w, R), A32.ctypes.data_as(ct.POINTER(ct.c_float)), pv.ctypes.data_as(ct.POINTER(ct.c_double)),
        _ptr(cc, R), nz, nzp, dz, lz, low_cut, high_cut, wnc, err_var, ts, gain, sf)
    return out.view(np.complex64 if prec == "f" else np.complex128)


def multiply_scale_wavelet(buf, nx, ny, wavelet, dz, rel_thick, shift=None, gain=None, prec="f", nthreads=None):
    """Crava::multiplyDataByScaleWaveletAndWriteToFile's per-trace product on one real padded cube."""
    R = ct.c_float if prec == "f" else ct.c_double
    nzp, nyp, rnxp = buf.shape
    nxp = rel_thick.shape[1]
    out = np.array(buf, dtype=_rdt(prec), order="C")
    w = np.ascontiguousarray(wavelet, dtype=_rdt(prec))
    rt = np.ascontiguousarray(rel_thick, dtype=np.float32)
    keep = [np.ascontiguousarray(x, dtype=np.float32) if x is not None else None for x in (shift, gain)]
    getattr(lib(), "or_multiply_scale_wavelet_" + prec)(
        _ptr(out, R), nx, ny, nxp, nyp, nzp, _ptr(w, R), dz, rt.ctypes.data_as(ct.POINTER(ct.c_float)),
        _fptr(keep[0]), _fptr(keep[1]), nthreads or os.cpu_count())
    return out


def interpolate_seismic(buf, nx, ny, nz, nxp, energy_threshold=0.0, prec="f"):
    """FFTGrid::interpolateSeismic + extrapolateSeismic on one real padded cube; returns (cube, n_bad)."""
    R = ct.c_float if prec == "f" else ct.c_double
    nzp, nyp, rnxp = buf.shape
    out = np.array(buf, dtype=_rdt(prec), order="C")
    n = getattr(lib(), "or_interpolate_seismic_" + prec)(_ptr(out, R), nx, ny, nz, nxp, nyp, nzp, energy_threshold)
    return out, n


def _dp(a):
    return None if a is None else a.ctypes.data_as(ct.POINTER(ct.c_double))


def new_posterior_cov_pointwise(G, err_theta_cov, prior_var0, post_var0, scales):
    """Crava::newPosteriorCovPointwise for one trace: (sigmanew, sigmamdnew), 3x3 each."""
    G = np.ascontiguousarray(G, dtype=np.float64)
    n = G.shape[0]
    e = np.ascontiguousarray(err_theta_cov, dtype=np.float64)
    sm = np.ascontiguousarray(prior_var0, dtype=np.float64)
    smd = np.ascontiguousarray(post_var0, dtype=np.float64)
    sc = np.ascontiguousarray(scales, dtype=np.float64)
    out1 = np.zeros((3, 3))
    out2 = np.zeros((3, 3))
    lib().or_new_posterior_cov_pointwise(n, _dp(G), _dp(e), _dp(sm), _dp(smd), _dp(sc), _dp(out1), _dp(out2))
    return out1, out2


def correct_alpha_beta_rho(post, mean, nx, ny, nz, nxp, G, err_theta_cov, prior_var0, post_var0, noise_scale,
                           want_sigmamd=False):
    """Crava::correctAlphaBetaRho on copies of 3 real padded posterior-mean cubes; returns (cubes, sigmamd)."""
    P = [np.array(c, dtype=np.float32, order="C") for c in post]
    M = [np.ascontiguousarray(c, dtype=np.float32) for c in mean]
    nzp, nyp, _ = P[0].shape
    G = np.ascontiguousarray(G, dtype=np.float64)
    n = G.shape[0]
    PF = ct.POINTER(ct.c_float)
    pp = (PF * 3)(*[c.ctypes.data_as(PF) for c in P])
    mp = (PF * 3)(*[c.ctypes.data_as(PF) for c in M])
    arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (err_theta_cov, prior_var0, post_var0, noise_scale)]
    smd = np.zeros((ny, nx, 9)) if want_sigmamd else None
    lib().or_correct_alpha_beta_rho(pp, mp, nx, ny, nz, nxp, nyp, n, _dp(G), _dp(arrs[0]), _dp(arrs[1]), _dp(arrs[2]),
                                    _dp(arrs[3]), _dp(smd))
    return P, smd


def circ_corr_t(priorCorrT, minIntFq, nzp, prec="f"):
    R = ct.c_float if prec == "f" else ct.c_double
    pc = np.ascontiguousarray(priorCorrT, dtype=np.float32)
    out = np.zeros(nzp, dtype=_rdt(prec))
    rc = getattr(lib(), "or_circ_corr_t_" + prec)(pc.ctypes.data, pc.size, minIntFq, nzp, _ptr(out, R))
    if rc:
        raise ValueError("circular temporal correlation undefined (CircCorrT[0] <= 1e-5)")
    return out


def fill_complex_noise(nxp, nyp, nzp, seed, ncubes=1):
    """FFTGrid::fillInComplexNoise x ncubes with a RandomGen seeded by `seed`."""
    cnxp, _ = dims(nxp)
    out = np.zeros((ncubes, nzp, nyp, cnxp), dtype=np.complex64)
    st = ct.c_uint(seed)
    for c in range(ncubes):
        lib().or_fill_complex_noise(_ptr(out[c].view(np.float32), ct.c_float), nxp, nyp, nzp, ct.byref(st))
    return out


def ref_fill_complex_noise(nxp, nyp, nzp, seed, ncubes=1):
    cnxp, _ = dims(nxp)
    out = np.zeros((ncubes, nzp, nyp, cnxp), dtype=np.complex64)
    ref().ref_fill_complex_noise(_ptr(out.view(np.float32), ct.c_float), nxp, nyp, nzp, seed, ncubes)
    return out


def rnorm01_seq(seed, n):
    st = ct.c_uint(seed)
    return np.array([lib().or_rnorm01(ct.byref(st)) for _ in range(n)])


def ref_rnorm01_seq(seed, n):
    out = np.zeros(n, dtype=np.float64)
    ref().ref_rnorm01_seq(seed, n, out.ctypes.data_as(ct.POINTER(ct.c_double)))
    return out


def find_closest_factorable(n):
    return lib().or_find_closest_factorable(int(n))
