"""Python mirror of the reference's FFTGrid / Crava surface over the C-ABI.

torch provides device memory and streams; every transform and every per-bin
solve runs in libcravagpu.so.  Names follow the reference:

* ``fft_in_place`` / ``inv_fft_in_place``  -- FFTGrid::fftInPlace / invFFTInPlace
  (src/fftgrid.cpp:1783-1842) on a padded cube tensor of shape
  ``(nzp, nyp, rnxp)`` (float32 or float64), in place.
* ``Workspace``  -- per-model device state; ``invert_plain`` / ``invert_fused``
  run the bin loop of Crava::computePostMeanResidAndFFTCov
  (src/crava.cpp:1084-1247).
* ``operator_tables`` -- the per-k tables of Crava::fillErrMultVectors
  (src/crava.cpp:1337-1386) built on the host in C++.
"""
from __future__ import annotations

import ctypes as ct
import os

import numpy as np
import torch

from ._native import check, lib

DATA, PARAMETER, COVARIANCE, VELOCITY, OPERATOR = 1, 2, 3, 4, 5
PREC_FP32, PREC_MIXED, PREC_FP64 = 0, 1, 2


def dims(nxp: int):
    cnxp = nxp // 2 + 1
    return cnxp, 2 * cnxp


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ct.c_void_p(s.cuda_stream)


def _vp(t: torch.Tensor):
    return ct.c_void_p(t.data_ptr())


def _pp(ts):
    arr = (ct.c_void_p * len(ts))(*[t.data_ptr() for t in ts])
    return ct.cast(arr, ct.POINTER(ct.c_void_p)), arr


def check_call(name, *args):
    """Call a C-ABI entry point by name; tensors and streams become pointers."""
    conv = []
    for a in args:
        if isinstance(a, torch.Tensor):
            conv.append(ct.c_void_p(a.data_ptr()))
        elif isinstance(a, torch.cuda.Stream):
            conv.append(ct.c_void_p(a.cuda_stream))
        else:
            conv.append(a)
    check(getattr(lib(), name)(*conv), name)


def new_cube(nxp, nyp, nzp, dtype=torch.float32, device="cuda"):
    """Zeroed padded cube (nzp, nyp, rnxp) in the FFTGrid in-place layout."""
    _, rnxp = dims(nxp)
    return torch.zeros((nzp, nyp, rnxp), dtype=dtype, device=device)


def as_spectrum(cube: torch.Tensor) -> torch.Tensor:
    """Complex view (nzp, nyp, cnxp) of a transformed cube."""
    nzp, nyp, rnxp = cube.shape
    return torch.view_as_complex(cube.view(nzp, nyp, rnxp // 2, 2))


def _check_cube(t: torch.Tensor, nxp: int):
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("cube must be a contiguous CUDA tensor")
    _, rnxp = dims(nxp)
    if t.dim() != 3 or t.shape[2] != rnxp:
        raise ValueError(f"cube shape {tuple(t.shape)} does not match nxp={nxp} (rnxp={rnxp})")


def fft_in_place(cube: torch.Tensor, nxp: int, cubetype: int, stream=None):
    _check_cube(cube, nxp)
    nzp, nyp, _ = cube.shape
    if cube.dtype == torch.float32:
        check(lib().cg_fft3d_r2c(_vp(cube), nxp, nyp, nzp, cubetype, _stream(stream)), "cg_fft3d_r2c")
    elif cube.dtype == torch.float64:
        check(lib().cg_fft3d_r2c_f64(_vp(cube), nxp, nyp, nzp, cubetype, _stream(stream)), "cg_fft3d_r2c_f64")
    else:
        raise TypeError(cube.dtype)
    return cube


def inv_fft_in_place(cube: torch.Tensor, nxp: int, cubetype: int, stream=None):
    _check_cube(cube, nxp)
    nzp, nyp, _ = cube.shape
    if cube.dtype == torch.float32:
        check(lib().cg_fft3d_c2r(_vp(cube), nxp, nyp, nzp, cubetype, _stream(stream)), "cg_fft3d_c2r")
    elif cube.dtype == torch.float64:
        check(lib().cg_fft3d_c2r_f64(_vp(cube), nxp, nyp, nzp, cubetype, _stream(stream)), "cg_fft3d_c2r_f64")
    else:
        raise TypeError(cube.dtype)
    return cube


def fft_in_place_batch(cubes, nxp: int, cubetype: int, inverse=False, stream=None):
    for c in cubes:
        _check_cube(c, nxp)
        if c.dtype != torch.float32:
            raise TypeError("batched transforms take float32 cubes")
    nzp, nyp, _ = cubes[0].shape
    pp, keep = _pp(cubes)
    fn = lib().cg_fft3d_c2r_batch if inverse else lib().cg_fft3d_r2c_batch
    check(fn(pp, len(cubes), nxp, nyp, nzp, cubetype, _stream(stream)), "cg_fft3d batch")
    del keep
    return cubes


def operator_tables(wavelets, A, nz, nzp, dt_ms, low_cut, high_cut, min_rel_thick=1.0):
    """Per-k forward operator and error multipliers (host, C++)."""
    w = np.ascontiguousarray(wavelets, dtype=np.float32)
    n = w.shape[0]
    A32 = np.ascontiguousarray(A, dtype=np.float32)
    K = np.zeros((nzp, n, 3), dtype=np.complex64)
    e1 = np.zeros((nzp, n), dtype=np.complex64)
    e2 = np.zeros((nzp, n), dtype=np.complex64)
    e3 = np.zeros((nzp, n), dtype=np.complex64)
    band = np.zeros(nzp, dtype=np.uint8)
    L = lib()
    check(L.cg_operator_tables(n, nz, nzp, w.ctypes.data, A32.ctypes.data, dt_ms, min_rel_thick, low_cut, high_cut,
                               K.ctypes.data, e1.ctypes.data, e2.ctypes.data, e3.ctypes.data, band.ctypes.data),
          "cg_operator_tables")
    return {"K": K, "em1": e1, "em2": e2, "em3": e3, "band": band}


def operator_tables_nct(wavelets, A, nz, nzp, dt_ms, low_cut, high_cut, min_rel_thick):
    """fillErrMultVectors tables, non-constant-thickness branch (cg_operator_tables_ex)."""
    w = np.ascontiguousarray(wavelets, dtype=np.float32)
    n = w.shape[0]
    A32 = np.ascontiguousarray(A, dtype=np.float32)
    K = np.zeros((nzp, n, 3), dtype=np.complex64)
    e1 = np.zeros((nzp, n), dtype=np.complex64)
    e2 = np.zeros((nzp, n), dtype=np.complex64)
    e3 = np.zeros((nzp, n), dtype=np.complex64)
    band = np.zeros(nzp, dtype=np.uint8)
    check(lib().cg_operator_tables_ex(n, nz, nzp, w.ctypes.data, A32.ctypes.data, dt_ms, min_rel_thick, low_cut,
                                      high_cut, 0, K.ctypes.data, e1.ctypes.data, e2.ctypes.data, e3.ctypes.data,
                                      band.ctypes.data), "cg_operator_tables_ex")
    return {"K": K, "em1": e1, "em2": e2, "em3": e3, "band": band}


def scale_wavelet_tables(wavelets, A, prior_var0, circ_corr_t, err_theta_cov, nz, dz_ms, lz_ms, low_cut, high_cut,
                         wnc):
    """Per-angle tables of Crava::computeAdjustmentFactor (host, C++): (ntheta, table_size) float32."""
    w = np.ascontiguousarray(wavelets, dtype=np.float32)
    n, nzp = w.shape
    A32 = np.ascontiguousarray(A, dtype=np.float32)
    pv = np.ascontiguousarray(prior_var0, dtype=np.float64)
    cc = np.ascontiguousarray(circ_corr_t, dtype=np.float32)
    etc = np.ascontiguousarray(err_theta_cov, dtype=np.float64)
    ts = lib().cg_scale_wavelet_table_size(nzp)
    out = np.zeros((n, ts), dtype=np.float32)
    check(lib().cg_scale_wavelet_tables(n, nz, nzp, w.ctypes.data, A32.ctypes.data, pv.ctypes.data, cc.ctypes.data,
                                        etc.ctypes.data, dz_ms, lz_ms, low_cut, high_cut, wnc, out.ctypes.data),
          "cg_scale_wavelet_tables")
    return out


def divide_by_scale_wavelet(cubes, nx, ny, nz, nxp, tables: torch.Tensor, rel_thick: torch.Tensor, dz_ms, lz_ms,
                            low_cut, high_cut, energy_threshold=0.0, shift=None, gain=None, stream=None):
    """Crava::divideDataByScaleWavelet (+ interpolateSeismic unless energy_threshold < 0) on real padded
    DATA cubes in place (cg_divide_by_scale_wavelet); returns the per-cube count of traces at or below
    the energy limit."""
    nzp, nyp, _ = cubes[0].shape
    pc, keep = _pp(cubes)
    nbad = (ct.c_int * len(cubes))()
    check(lib().cg_divide_by_scale_wavelet(pc, len(cubes), nx, ny, nz, nxp, nyp, nzp, _vp(tables), _vp(rel_thick),
                                           _vp(shift) if shift is not None else None,
                                           _vp(gain) if gain is not None else None, float(dz_ms), float(lz_ms),
                                           float(low_cut), float(high_cut), float(energy_threshold), nbad,
                                           _stream(stream)), "cg_divide_by_scale_wavelet")
    return list(nbad)


def multiply_by_scale_wavelet(cubes, nx, ny, nxp, tables: torch.Tensor, rel_thick: torch.Tensor, dz_ms, shift=None,
                              gain=None, stream=None):
    """The per-trace product of Crava::multiplyDataByScaleWaveletAndWriteToFile on real padded cubes in place."""
    nzp, nyp, _ = cubes[0].shape
    pc, keep = _pp(cubes)
    check(lib().cg_multiply_by_scale_wavelet(pc, len(cubes), nx, ny, nxp, nyp, nzp, _vp(tables), _vp(rel_thick),
                                             _vp(shift) if shift is not None else None,
                                             _vp(gain) if gain is not None else None, float(dz_ms),
                                             _stream(stream)), "cg_multiply_by_scale_wavelet")


def interpolate_seismic(cube: torch.Tensor, nx, ny, nz, nxp, energy_threshold=0.0, stream=None):
    """FFTGrid::interpolateSeismic on one real padded DATA cube in place; returns the count of bad traces."""
    nzp, nyp, _ = cube.shape
    nbad = ct.c_int()
    check(lib().cg_interpolate_seismic(_vp(cube), nx, ny, nz, nxp, nyp, nzp, float(energy_threshold), ct.byref(nbad),
                                       _stream(stream)), "cg_interpolate_seismic")
    return nbad.value


def _sort3x3(ev, V):
    """NRLib::Sort3x3 (libs/nrlib/flens/nrlib_flens.cpp:211-245): eigenvalues in decreasing order, the
    first of equal values first, eigenvectors permuted alike."""
    idx = []
    for _ in range(3):
        best, bi = -100000.0, -1
        for i in range(3):
            if i not in idx and ev[i] > best:
                best, bi = ev[i], i
        idx.append(bi)
    return ev[idx], V[:, idx]


def _eig(M):
    """NRLib::ComputeEigenVectors: the general LAPACK eigen solver (geev) on a symmetric matrix, real parts."""
    w, V = np.linalg.eig(np.asarray(M, dtype=np.float64))
    return np.real(w), np.real(V)


def local_noise_g(err_theta_cov, prior_var0, post_var0):
    """Crava::computeG (src/crava.cpp:2261-2343) on the host with LAPACK's geev through numpy, as the
    reference's NRLib::ComputeEigenVectors does: G (ntheta, 3) for cg_correct_alpha_beta_rho.  The
    correction depends on the signs of the eigenvectors of Sm^-1/2 (Sm - Spost) Sm^-1/2, which are the
    eigen routine's choice."""
    E = np.asarray(err_theta_cov, dtype=np.float64)
    n = E.shape[0]
    Sm = np.asarray(prior_var0, dtype=np.float64)
    Sdelta = Sm - np.asarray(post_var0, dtype=np.float64)
    ev, V = _eig(Sdelta)
    Sdelta = V @ np.diag(np.where(ev > 0.0, ev, 0.0)) @ V.T
    ev, V = _eig(Sm)
    Sinv = V @ np.diag(np.where(ev > 0.0000001, 1.0 / np.sqrt(np.abs(ev)), 0.0)) @ V.T
    A = Sinv @ Sdelta @ Sinv
    ev, V = _sort3x3(*_eig(A))
    Lg = np.zeros((n, 3))
    for i in range(min(n, 3)):
        Lg[i, i] = np.sqrt(ev[i] / (1.0 - ev[i]))
    eve, Ve = _eig(E)
    Esq = Ve @ np.diag(np.where(eve > 0.0, np.sqrt(np.abs(eve)), 0.0)) @ Ve.T
    return Esq @ Lg @ V.T @ Sinv


def correct_alpha_beta_rho(post, mean, nx, ny, nz, nxp, G, err_theta_cov, prior_var0, post_var0,
                           noise_scale: torch.Tensor, sigmamd: torch.Tensor | None = None, stream=None):
    """Crava::correctAlphaBetaRho on 3 real padded posterior-mean cubes in place (cg_correct_alpha_beta_rho).
    noise_scale: (ntheta, ny, nx) float64 device tensor; sigmamd: optional (ny, nx, 9) float64 device tensor."""
    nzp, nyp, _ = post[0].shape
    pp, k1 = _pp(post)
    pm, k2 = _pp(mean)
    G = np.ascontiguousarray(G, dtype=np.float64)
    h = [np.ascontiguousarray(x, dtype=np.float64) for x in (err_theta_cov, prior_var0, post_var0)]
    check(lib().cg_correct_alpha_beta_rho(pp, pm, nx, ny, nz, nxp, nyp, nzp, G.shape[0], G.ctypes.data,
                                          h[0].ctypes.data, h[1].ctypes.data, h[2].ctypes.data, _vp(noise_scale),
                                          _vp(sigmamd) if sigmamd is not None else None, _stream(stream)),
          "cg_correct_alpha_beta_rho")


def apply_trace_matrices(fields, mats: torch.Tensor, nx, ny, nz, nxp, mean=None, stream=None):
    """The local-noise step of Crava::simulate: simbox cells times the trace's 3x3 matrix, then + mean."""
    nzp, nyp, _ = fields[0].shape
    pf, k1 = _pp(fields)
    pm, k2 = _pp(mean) if mean is not None else (None, None)
    check(lib().cg_apply_trace_matrices(pf, pm, _vp(mats), nx, ny, nz, nxp, nyp, nzp, _stream(stream)),
          "cg_apply_trace_matrices")


class _Model(ct.Structure):
    _fields_ = [("ntheta", ct.c_int), ("wnc", ct.c_float), ("is4d", ct.c_int), ("K", ct.c_void_p),
                ("em1", ct.c_void_p), ("em2", ct.c_void_p), ("em3", ct.c_void_p), ("band", ct.c_void_p),
                ("err_theta_cov", ct.c_void_p), ("sigma0", ct.c_void_p), ("cond_threshold", ct.c_double)]


class Workspace:
    """Device state of one inversion model (cg_workspace)."""

    def __init__(self, nxp, nyp, nzp, ntheta):
        self.nxp, self.nyp, self.nzp, self.ntheta = nxp, nyp, nzp, ntheta
        h = ct.c_void_p()
        check(lib().cg_workspace_create(ct.byref(h), nxp, nyp, nzp, ntheta), "cg_workspace_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().cg_workspace_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_model(self, tables, err_theta_cov, sigma0, wnc, is4d=False, cond_threshold=0.0, stream=None,
                  asynchronous=False):
        """Upload the model (host arrays) and build the per-k tables.  asynchronous=True queues the
        upload and the table kernel on ``stream`` (cg_workspace_set_model_async) instead of waiting."""
        keep = [np.ascontiguousarray(tables[k], dtype=np.complex64) for k in ("K", "em1", "em2", "em3")]
        band = np.ascontiguousarray(tables["band"], dtype=np.uint8)
        etc = np.ascontiguousarray(err_theta_cov, dtype=np.float64)
        s0 = np.ascontiguousarray(sigma0, dtype=np.float64).reshape(9)
        m = _Model(self.ntheta, float(wnc), int(is4d), *[a.ctypes.data for a in keep], band.ctypes.data,
                   etc.ctypes.data, s0.ctypes.data, float(cond_threshold))
        if asynchronous:
            check(lib().cg_workspace_set_model_async(self.h, ct.byref(m), _stream(stream)),
                  "cg_workspace_set_model_async")
        else:
            check(lib().cg_workspace_set_model(self.h, ct.byref(m)), "cg_workspace_set_model")

    def condition_histogram(self, nbuckets=24, stream=None):
        """Decade histograms of the in-band bins' condition estimates (cg_condition_histogram): the FP64
        Cholesky of the data covariance and the FP32 3 x 3 information-form matrix.  Needs prior_spectra."""
        hc = (ct.c_ulonglong * nbuckets)()
        hi = (ct.c_ulonglong * nbuckets)()
        check(lib().cg_condition_histogram(self.h, hc, hi, nbuckets, _stream(stream)), "cg_condition_histogram")
        return list(hc), list(hi)

    def reset_stats(self, stream=None):
        check(lib().cg_workspace_reset_stats(self.h, _stream(stream)), "cg_workspace_reset_stats")

    def stats(self):
        a, b, c = ct.c_int(), ct.c_int(), ct.c_int()
        check(lib().cg_workspace_stats(self.h, ct.byref(a), ct.byref(b), ct.byref(c)), "cg_workspace_stats")
        return {"flagged": a.value, "failed": b.value, "overflow": c.value}

    def invert_plain(self, data, mean, cov, errcorr, stream=None):
        pd, k1 = _pp(data)
        pm, k2 = _pp(mean)
        pc, k3 = _pp(cov)
        check(lib().cg_invert_bins_plain(self.h, pd, pm, pc, _vp(errcorr), _stream(stream)), "cg_invert_bins_plain")

    def prior_spectra(self, corr_xy, circ_corr_t, precision=PREC_MIXED, stream=None, grad=(0.0, 0.0)):
        """Prior of the fused forms (cg_prior_spectra; cg_prior_spectra_grad for nonzero correlation
        gradients grad = (corrGradI, corrGradJ))."""
        gi, gj = float(grad[0]), float(grad[1])
        if gi == 0.0 and gj == 0.0:
            check(lib().cg_prior_spectra(self.h, _vp(corr_xy), _vp(circ_corr_t), precision, _stream(stream)),
                  "cg_prior_spectra")
        else:
            check(lib().cg_prior_spectra_grad(self.h, _vp(corr_xy), _vp(circ_corr_t), gi, gj, precision,
                                              _stream(stream)), "cg_prior_spectra_grad")

    def invert_cubes(self, data, mean, cov, precision=PREC_MIXED, stream=None):
        """Whole fused inversion from real-domain cubes (cg_invert_cubes_fused)."""
        pd, k1 = _pp(data)
        pm, k2 = _pp(mean)
        pc, k3 = _pp(cov)
        check(lib().cg_invert_cubes_fused(self.h, pd, pm, pc, precision, _stream(stream)), "cg_invert_cubes_fused")

    def invert_fused(self, data, mean, cov, precision=PREC_MIXED, stream=None):
        pd, k1 = _pp(data)
        pm, k2 = _pp(mean)
        pc, k3 = _pp(cov)
        if data[0].dtype == torch.float64:
            check(lib().cg_invert_bins_fused_f64(self.h, pd, pm, pc, _stream(stream)), "cg_invert_bins_fused_f64")
        else:
            check(lib().cg_invert_bins_fused(self.h, pd, pm, pc, precision, _stream(stream)), "cg_invert_bins_fused")


def posterior_cholesky(post_cov, nxp, stream=None):
    """Per-bin Cholesky factor of the posterior covariance spectra (9 float planes)."""
    nzp, nyp, _ = post_cov[0].shape
    cnxp, _ = dims(nxp)
    chol = torch.empty((9, nzp, nyp, cnxp), dtype=torch.float32, device=post_cov[0].device)
    nfail = torch.zeros(1, dtype=torch.int32, device=post_cov[0].device)
    pc, k = _pp(post_cov)
    check(lib().cg_posterior_cholesky(pc, _vp(chol), nxp, nyp, nzp, _vp(nfail), _stream(stream)),
          "cg_posterior_cholesky")
    return chol, nfail


def simulate_fields(chol, fields, nxp, seed=0, real0=0, noise=None, post_mean=None, stream=None):
    """Fill fields (3 per realisation) with posterior realisations (see cg_simulate_fields)."""
    nzp, nyp, _ = fields[0].shape
    pf, k1 = _pp(fields)
    pn, k2 = _pp(noise) if noise is not None else (None, None)
    pm, k3 = _pp(post_mean) if post_mean is not None else (None, None)
    check(lib().cg_simulate_fields(_vp(chol), pn, pf, len(fields) // 3, real0, seed, nxp, nyp, nzp, pm,
                                   _stream(stream)), "cg_simulate_fields")


def fill_in_data(buf: torch.Tensor, nxp: int, nz: int, cubetype: int, traces: torch.Tensor, state: torch.Tensor,
                 z0_data: torch.Tensor, z0_grid: torch.Tensor, dz_grid: torch.Tensor, dz_data: float,
                 smooth_length: float, stream=None):
    """FFTGrid::fillInData's per-trace core (cg_fill_in_data); returns the extrapolation counts."""
    nzp, nyp, _ = buf.shape
    ext = (ct.c_int * 2)()
    check(lib().cg_fill_in_data(_vp(buf), nxp, nyp, nzp, nz, cubetype, _vp(traces), traces.shape[1], _vp(state),
                                _vp(z0_data), _vp(z0_grid), _vp(dz_grid), float(dz_data), float(smooth_length),
                                ext, _stream(stream)), "cg_fill_in_data")
    return [ext[0], ext[1]]


# ---------------------------------------------------------------------------
# file formats (host memory)
# ---------------------------------------------------------------------------
class StormHeader(ct.Structure):
    _fields_ = [("zone_number", ct.c_int), ("model_file", ct.c_char * 256), ("missing_code", ct.c_float),
                ("variable", ct.c_char * 256), ("x_min", ct.c_double), ("lx", ct.c_double), ("y_min", ct.c_double),
                ("ly", ct.c_double), ("z_top", ct.c_double), ("z_bot", ct.c_double), ("erosion_top", ct.c_double),
                ("erosion_bot", ct.c_double), ("lz", ct.c_double), ("angle_deg", ct.c_double),
                ("z_top_file", ct.c_char * 256), ("z_bot_file", ct.c_char * 256),
                ("erosion_top_file", ct.c_char * 256), ("erosion_bot_file", ct.c_char * 256)]


# the four surfaces of a STORM grid: header field of the file name, suffix the reference gives the file
STORM_SURFACES = (("z_top_file", "_top"), ("z_bot_file", "_bot"), ("erosion_top_file", "_erosion_top"),
                  ("erosion_bot_file", "_erosion_bot"))


class StormSurface:
    """A regular surface (NRLib RegularSurface): z (nj, ni) float64, nodes over [x_min, x_min + lx] x
    [y_min, y_min + ly]; -999 marks a missing node."""

    def __init__(self, z, x_min, y_min, lx, ly):
        self.z = np.ascontiguousarray(z, dtype=np.float64)
        self.x_min, self.y_min, self.lx, self.ly = float(x_min), float(y_min), float(lx), float(ly)


def write_storm_surface(path, surf: StormSurface):
    """STORM binary surface file (cg_storm_surface_write)."""
    nj, ni = surf.z.shape
    check(lib().cg_storm_surface_write(str(path).encode(), surf.z.ctypes.data, ni, nj, surf.x_min, surf.y_min,
                                       surf.lx, surf.ly), "cg_storm_surface_write")


def read_storm_surface(path) -> StormSurface:
    """STORM binary surface file (cg_storm_surface_read_header / cg_storm_surface_read)."""
    ni, nj = ct.c_int(), ct.c_int()
    g = [ct.c_double() for _ in range(4)]
    check(lib().cg_storm_surface_read_header(str(path).encode(), ct.byref(ni), ct.byref(nj),
                                             *[ct.byref(x) for x in g]), "cg_storm_surface_read_header")
    z = np.empty((nj.value, ni.value), dtype=np.float64)
    check(lib().cg_storm_surface_read(str(path).encode(), z.ctypes.data, z.size), "cg_storm_surface_read")
    return StormSurface(z, *[x.value for x in g])


def write_crava_file(path, cube: np.ndarray, geom, nx: int, ny: int):
    """FFTGrid::writeCravaFile: cube (nzp, nyp, rnxp) float32, geom 11 doubles (x0 y0 dx dy IL0 XL0 ILStepX
    ILStepY XLStepX XLStepY angle)."""
    c = np.ascontiguousarray(cube, dtype=np.float32)
    g = np.ascontiguousarray(geom, dtype=np.float64)
    n = np.array([nx, ny], dtype=np.int32)
    nzp, nyp, rnxp = c.shape
    check(lib().cg_crava_file_write(str(path).encode(), c.ctypes.data, rnxp, nyp, nzp, g.ctypes.data, n.ctypes.data),
          "cg_crava_file_write")


def read_crava_file(path, nxp: int, nyp: int, nzp: int):
    """FFTGrid::readCravaFile: (cube (nzp, nyp, rnxp), geom (11,), (nx, ny))."""
    _, rnxp = dims(nxp)
    c = np.empty((nzp, nyp, rnxp), dtype=np.float32)
    g = np.empty(11, dtype=np.float64)
    n = np.empty(2, dtype=np.int32)
    check(lib().cg_crava_file_read(str(path).encode(), c.ctypes.data, rnxp, nyp, nzp, g.ctypes.data, n.ctypes.data),
          "cg_crava_file_read")
    return c, g, (int(n[0]), int(n[1]))


def write_storm(path, values: np.ndarray, header: StormHeader, surfaces=None):
    """STORM binary grid; values (nk, nj, ni) float32 (i fastest).  surfaces: optional dict of StormSurface by
    header field ("z_top_file", "z_bot_file", "erosion_top_file", "erosion_bot_file"); each is written beside
    the grid as <path>_top, <path>_bot, ... and named in the header without its directory, as
    StormContGrid::WriteToFile does by default (remove_path)."""
    v = np.ascontiguousarray(values, dtype=np.float32)
    nk, nj, ni = v.shape
    for field, suffix in STORM_SURFACES:
        if surfaces and field in surfaces:
            write_storm_surface(str(path) + suffix, surfaces[field])
            setattr(header, field, os.path.basename(str(path) + suffix).encode())
    check(lib().cg_storm_write(str(path).encode(), v.ctypes.data, ni, nj, nk, ct.byref(header)), "cg_storm_write")


def read_storm(path):
    """STORM binary grid: (values (nk, nj, ni), StormHeader).  Surfaces given as files keep their names in the
    header's *_file fields (read_storm_surfaces loads them)."""
    h = StormHeader()
    ni, nj, nk = ct.c_int(), ct.c_int(), ct.c_int()
    check(lib().cg_storm_read_header(str(path).encode(), ct.byref(h), ct.byref(ni), ct.byref(nj), ct.byref(nk)),
          "cg_storm_read_header")
    v = np.empty((nk.value, nj.value, ni.value), dtype=np.float32)
    check(lib().cg_storm_read(str(path).encode(), v.ctypes.data, v.size), "cg_storm_read")
    return v, h


def read_storm_surfaces(path, header: StormHeader):
    """The surface files a STORM grid's header names, resolved against the grid file's directory as
    StormContGrid::ReadFromFile does (commonPath): dict of StormSurface by header field."""
    out = {}
    for field, _ in STORM_SURFACES:
        name = getattr(header, field).decode()
        if name:
            out[field] = read_storm_surface(os.path.join(os.path.dirname(str(path)), name))
    return out


def exp_transform(t: torch.Tensor, stream=None):
    """FFTGrid::expTransf in place (cg_exp_transform)."""
    check(lib().cg_exp_transform(_vp(t), t.numel(), _stream(stream)), "cg_exp_transform")


def log_transform(t: torch.Tensor, stream=None):
    """FFTGrid::logTransf in place (cg_log_transform)."""
    check(lib().cg_log_transform(_vp(t), t.numel(), _stream(stream)), "cg_log_transform")


def inv_fft_exp_batch(cubes, nxp: int, cubetype: int, stream=None):
    """Inverse transforms with expTransf fused into the last pass (cg_fft3d_c2r_exp_batch)."""
    nzp, nyp, _ = cubes[0].shape
    p, k = _pp(cubes)
    check(lib().cg_fft3d_c2r_exp_batch(p, len(cubes), nxp, nyp, nzp, cubetype, _stream(stream)),
          "cg_fft3d_c2r_exp_batch")


def cov_origin(cov_real, nxp: int, nz: int, stream=None):
    """(postVar0 3x3 float64, postCov00 (3, nz) float32) from real-domain covariance grids (00 11 22 01 02 12)."""
    nzp, nyp, _ = cov_real[0].shape
    v0 = np.zeros(9, dtype=np.float64)
    c00 = np.zeros((3, nz), dtype=np.float32)
    p, k = _pp(cov_real)
    check(lib().cg_cov_origin(p, nxp, nyp, nzp, nz, v0.ctypes.data, c00.ctypes.data, _stream(stream)),
          "cg_cov_origin")
    return v0.reshape(3, 3), c00


def state4d_merge(mu_s, mu_d, ss, sd, dd, mu_cur, cov_cur, nxp, stream=None):
    """State4D::merge/mergeCov into mu_cur[3], cov_cur[6] (order 00 01 02 11 12 22)."""
    nzp, nyp, _ = mu_s[0].shape
    keep = [_pp(x) for x in (mu_s, mu_d, ss, sd, dd, mu_cur, cov_cur)]
    check(lib().cg_state4d_merge(*[k[0] for k in keep], nxp, nyp, nzp, _stream(stream)), "cg_state4d_merge")


def state4d_evolve(mu_s, mu_d, ss, sd, dd, nxp, E, c, C, lam=None, stream=None):
    """State4D::evolve on the state spectra in place (cg_state4d_evolve): E, C (6, 6), c (6,) float64;
    lam the transformed increment correlation cube (fill_genexp_corr + COVARIANCE transform) or None."""
    nzp, nyp, _ = mu_s[0].shape
    Ed, cd, Cd = (np.ascontiguousarray(x, dtype=np.float64) for x in (E, c, C))
    ps = [_pp(g) for g in (mu_s, mu_d, ss, sd, dd)]
    check(lib().cg_state4d_evolve(*[p for p, _ in ps], _vp(lam) if lam is not None else None, Ed.ctypes.data,
                                  cd.ctypes.data, Cd.ctypes.data, nxp, nyp, nzp, _stream(stream)),
          "cg_state4d_evolve")


def fill_genexp_corr(buf: torch.Tensor, nxp, range_x, range_y, range_z, grad_i=0.0, grad_j=0.0, stream=None):
    """FFTGrid::fillInGenExpCorr into a real padded cube (cg_fill_genexp_corr)."""
    nzp, nyp, _ = buf.shape
    check(lib().cg_fill_genexp_corr(_vp(buf), nxp, nyp, nzp, float(range_x), float(range_y), float(range_z),
                                    float(grad_i), float(grad_j), _stream(stream)), "cg_fill_genexp_corr")


def state4d_split(mu_s, mu_d, ss, sd, dd, mu_post, cov_post, nxp, stream=None):
    """State4D::split in place; returns a device counter of bins that kept the prior."""
    nzp, nyp, _ = mu_s[0].shape
    nfail = torch.zeros(1, dtype=torch.int32, device=mu_s[0].device)
    keep = [_pp(x) for x in (mu_s, mu_d, ss, sd, dd, mu_post, cov_post)]
    check(lib().cg_state4d_split(*[k[0] for k in keep], nxp, nyp, nzp, _vp(nfail), _stream(stream)),
          "cg_state4d_split")
    return nfail


def vintage4d(ws, mu_s, mu_d, ss, sd, dd, data, errcorr, post_mean, nxp, precision=None, stream=None):
    """One 4D vintage in one pass (cg_vintage4d): state updated in place, data -> residuals, post_mean <-
    the current state's posterior mean.  Returns a device counter of bins whose split kept the prior."""
    prec = PREC_MIXED if precision is None else precision
    nsplit = torch.zeros(1, dtype=torch.int32, device=mu_s[0].device)
    keep = [_pp(x) for x in (mu_s, mu_d, ss, sd, dd, data, post_mean)]
    check(lib().cg_vintage4d(ws.h, *[k[0] for k in keep[:6]], _vp(errcorr), keep[6][0], prec, _vp(nsplit),
                             _stream(stream)), "cg_vintage4d")
    return nsplit


def corr_grad(sc):
    """(corrGradI, corrGradJ) of a scenario as float32 values; (0, 0) when it has none."""
    g = getattr(sc, "corr_grad", (0.0, 0.0))
    return float(np.float32(g[0])), float(np.float32(g[1]))


class _InvModel(ct.Structure):
    _fields_ = [("ntheta", ct.c_int), ("wavelets", ct.c_void_p), ("A", ct.c_void_p), ("err_theta_cov", ct.c_void_p),
                ("sigma0", ct.c_void_p), ("corr_xy", ct.c_void_p), ("circ_corr_t", ct.c_void_p),
                ("wnc", ct.c_float), ("low_cut", ct.c_float), ("high_cut", ct.c_float), ("dt_ms", ct.c_float),
                ("min_rel_thick", ct.c_float), ("cond_threshold", ct.c_double), ("corr_grad_i", ct.c_float),
                ("corr_grad_j", ct.c_float)]


class HostInversion:
    """The C++ host layer's inversion context (cg_inversion_*): host buffers in and out."""

    FORMS = {"plain": 0, "fp32": 1, "mixed": 2}

    def __init__(self, sc, cond_threshold=0.0):
        self.sc = sc
        self._arrs = [np.ascontiguousarray(sc.wavelets, dtype=np.float32), np.ascontiguousarray(sc.A, np.float32),
                      np.ascontiguousarray(sc.err_theta_cov, np.float64),
                      np.ascontiguousarray(sc.sigma0, np.float64).reshape(9),
                      np.ascontiguousarray(sc.corr_xy, np.float32), np.ascontiguousarray(sc.circ_corr_t, np.float32)]
        m = _InvModel(sc.ntheta, *[a.ctypes.data for a in self._arrs], sc.wnc, sc.low_cut, sc.high_cut, sc.dt_ms,
                      sc.min_rel_thick, cond_threshold, *corr_grad(sc))
        h = ct.c_void_p()
        check(lib().cg_inversion_create(ct.byref(h), sc.nx, sc.ny, sc.nz, sc.nxp, sc.nyp, sc.nzp, ct.byref(m)),
              "cg_inversion_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().cg_inversion_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, data, mean, cov_out, form="mixed", prior_cov_real=None, err_corr_real=None):
        """data/mean/cov_out: lists of float32 host arrays (numpy or pinned torch) of rsize floats each."""
        def ptrs(xs):
            arr = (ct.c_void_p * len(xs))(*[(x.data_ptr() if isinstance(x, torch.Tensor) else x.ctypes.data)
                                            for x in xs])
            return ct.cast(arr, ct.POINTER(ct.c_void_p)), arr
        pd, k1 = ptrs(data)
        pm, k2 = ptrs(mean)
        pc, k3 = ptrs(cov_out)
        pp, k4 = ptrs(prior_cov_real) if prior_cov_real is not None else (None, None)
        pe = ct.c_void_p(err_corr_real.ctypes.data) if err_corr_real is not None else None
        check(lib().cg_inversion_run_host(self.h, pd, pm, pc, pp, pe, self.FORMS[form]), "cg_inversion_run_host")

    def submit(self, data, mean, resid_out, mean_out, cov_out, form="mixed", prior_cov_real=None,
               err_corr_real=None):
        """Queue one inversion (cg_inversion_submit_host); the buffers stay in use until wait()."""
        def ptrs(xs):
            arr = (ct.c_void_p * len(xs))(*[(x.data_ptr() if isinstance(x, torch.Tensor) else x.ctypes.data)
                                            for x in xs])
            return ct.cast(arr, ct.POINTER(ct.c_void_p)), arr
        keep = [ptrs(x) for x in (data, mean, resid_out, mean_out, cov_out)]
        pp, k4 = ptrs(prior_cov_real) if prior_cov_real is not None else (None, None)
        pe = ct.c_void_p(err_corr_real.ctypes.data) if err_corr_real is not None else None
        self._inflight = (keep, k4)
        check(lib().cg_inversion_submit_host(self.h, *[k[0] for k in keep], pp, pe, self.FORMS[form]),
              "cg_inversion_submit_host")

    def wait(self):
        check(lib().cg_inversion_wait(self.h), "cg_inversion_wait")
        self._inflight = None

    def stats(self):
        a, b, c = ct.c_int(), ct.c_int(), ct.c_int()
        check(lib().cg_inversion_stats(self.h, ct.byref(a), ct.byref(b), ct.byref(c)), "cg_inversion_stats")
        return {"flagged": a.value, "failed": b.value, "overflow": c.value}


class _BatchCube(ct.Structure):
    _fields_ = [("nx", ct.c_int), ("ny", ct.c_int), ("nz", ct.c_int), ("nxp", ct.c_int), ("nyp", ct.c_int),
                ("nzp", ct.c_int), ("model", _InvModel)]


class Batch:
    """Many independent inversions of uneven cubes as one unit of GPU work (cg_batch_*)."""

    def __init__(self, scenarios, nstreams=3, cond_threshold=0.0):
        self.scs = list(scenarios)
        self._keep = []
        cubes = (_BatchCube * len(self.scs))()
        for i, sc in enumerate(self.scs):
            arrs = [np.ascontiguousarray(sc.wavelets, dtype=np.float32), np.ascontiguousarray(sc.A, np.float32),
                    np.ascontiguousarray(sc.err_theta_cov, np.float64),
                    np.ascontiguousarray(sc.sigma0, np.float64).reshape(9),
                    np.ascontiguousarray(sc.corr_xy, np.float32), np.ascontiguousarray(sc.circ_corr_t, np.float32)]
            self._keep.append(arrs)
            m = _InvModel(sc.ntheta, *[a.ctypes.data for a in arrs], sc.wnc, sc.low_cut, sc.high_cut, sc.dt_ms,
                          sc.min_rel_thick, cond_threshold, *corr_grad(sc))
            cubes[i] = _BatchCube(sc.nx, sc.ny, sc.nz, sc.nxp, sc.nyp, sc.nzp, m)
        h = ct.c_void_p()
        check(lib().cg_batch_create(ct.byref(h), ct.cast(cubes, ct.c_void_p), len(self.scs), nstreams),
              "cg_batch_create")
        self.h = h
        for i, sc in enumerate(self.scs):
            pd, k1 = _pp_np([np.ascontiguousarray(d, np.float32) for d in sc.data])
            pm, k2 = _pp_np([np.ascontiguousarray(m, np.float32) for m in sc.mean])
            check(lib().cg_batch_load(self.h, i, pd, pm), "cg_batch_load")

    @property
    def bins(self):
        return lib().cg_batch_bins(self.h)

    def reset(self, stream=None):
        check(lib().cg_batch_reset(self.h, _stream(stream)), "cg_batch_reset")

    def run(self, form="mixed", use_graph=True, stream=None):
        f = {"fp32": 1, "mixed": 2}[form]
        check(lib().cg_batch_run(self.h, f, 1 if use_graph else 0, _stream(stream)), "cg_batch_run")

    def read(self, i):
        sc = self.scs[i]
        mean = [np.empty_like(sc.mean[0]) for _ in range(3)]
        res = [np.empty_like(sc.data[0]) for _ in range(sc.ntheta)]
        cov = [np.empty_like(sc.data[0]) for _ in range(6)]
        pm, k1 = _pp_np(mean)
        pr, k2 = _pp_np(res)
        pc, k3 = _pp_np(cov)
        check(lib().cg_batch_read(self.h, i, pm, pr, pc), "cg_batch_read")
        return (np.stack([m[:, :, :sc.nxp] for m in mean]), np.stack([r.view(np.complex64) for r in res]),
                np.stack([c.view(np.complex64) for c in cov]))

    def set_simulation(self, i, nreal, seed=0):
        """Draw nreal posterior realisations of cube i after its inversion in every later run
        (cg_batch_set_simulation); nreal = 0 removes them."""
        check(lib().cg_batch_set_simulation(self.h, i, nreal, ct.c_ulonglong(seed)), "cg_batch_set_simulation")

    def read_fields(self, i, r):
        """Realisation r of cube i: 3 real padded cubes (alpha, beta, rho) as numpy float32."""
        sc = self.scs[i]
        out = [np.empty_like(sc.mean[0]) for _ in range(3)]
        pf, k = _pp_np(out)
        check(lib().cg_batch_read_fields(self.h, i, r, pf), "cg_batch_read_fields")
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().cg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _pp_np(arrs):
    arr = (ct.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    return ct.cast(arr, ct.POINTER(ct.c_void_p)), (arr, arrs)
