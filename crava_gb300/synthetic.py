"""Seeded synthetic AVO inversion inputs (host-side input tooling, numpy FP64).

The reference publishes no benchmark data and ships no test suite, so every
workload here is synthetic: a prior model, a seismic forward model and data
built the way CRAVA's own setup code builds them.  Nothing in this module is
on the timed path.

Pieces and the reference code each one follows (paths relative to the CRAVA
source tree):

* padded sizes -- FFTGrid::findClosestFactorableNumber (src/fftgrid.cpp:2857-2885)
  applied to ceil(n*(1+pad)) (ModelGeneral::setPaddingSize, src/modelgeneral.cpp:617-622);
* PP reflection coefficients -- linearised Aki-Richards,
  ModelAVODynamic::setupDefaultReflectionMatrix (src/modelavodynamic.cpp:877-929);
* Ricker wavelet, 239 taps at 1 ms sampled onto dt in FFT order --
  Wavelet ctor and Wavelet::resample (src/wavelet.cpp:130-186, :416-463,
  Wavelet::Ricker :1354-1358);
* lateral correlation surface on the padded grid --
  ModelGeneral::findCorrXYGrid (src/modelgeneral.cpp:4194-4230) with a
  GenExpVario (src/vario.cpp:30-39, :88-93);
* temporal correlation, cyclic and made positive definite --
  computeCircCorrT / makeCircCorrTPosDef (src/seismicparametersholder.cpp:430-501),
  lowIntCut = floor(lowCut*nzp*0.001*dt) (src/modelgeneral.cpp:4081);
* error covariance between stacks -- Crava::computeDataVariance and
  setupErrorCorrelation (src/crava.cpp:408-487) with the default angular
  correlation GenExpVario(1, 10 deg) (src/modelsettings.h:449).

The "truth" is one prior realisation and data = forward model + white noise
at the requested signal-to-noise ratio (total variance / noise variance,
matching how CRAVA turns S/N into an error variance, src/crava.cpp:462-465).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

_FFT_WORKERS = os.cpu_count() or 1

try:  # multi-threaded transforms for the input generator when scipy is present
    import scipy.fft as _sfft

    def _fftn(a):
        return _sfft.fftn(a, norm="ortho", workers=_FFT_WORKERS)

    def _ifftn(a):
        return _sfft.ifftn(a, norm="ortho", workers=_FFT_WORKERS)
except ImportError:  # pragma: no cover
    def _fftn(a):
        return np.fft.fftn(a, norm="ortho")

    def _ifftn(a):
        return np.fft.ifftn(a, norm="ortho")

LN_VP, LN_VS, LN_RHO = math.log(3000.0), math.log(1500.0), math.log(2.3)


def find_closest_factorable(leastint: int) -> int:
    """Smallest 2^a 3^b 5^c 7^d >= leastint (FFTGrid::findClosestFactorableNumber)."""
    best = None
    n = int(leastint)
    p2 = 1
    while p2 < 2 * n:
        p3 = p2
        while p3 < 2 * n:
            p5 = p3
            while p5 < 2 * n:
                p7 = p5
                while p7 < 2 * n:
                    if p7 >= n and (best is None or p7 < best):
                        best = p7
                    p7 *= 7
                p5 *= 5
            p3 *= 3
        p2 *= 2
    return best


def padded_size(n: int, pad: float) -> int:
    return find_closest_factorable(int(math.ceil(n * (1.0 + pad))))


def aki_richards_pp(theta_deg, vsvp: float) -> np.ndarray:
    """n_theta x 3 PP coefficients (float32 like the reference's float** A)."""
    A = np.zeros((len(theta_deg), 3), dtype=np.float32)
    v2 = vsvp * vsvp
    for i, t in enumerate(theta_deg):
        a = math.radians(t)
        s2 = math.sin(a) ** 2
        tan2 = math.tan(a) ** 2
        A[i, 0] = (1.0 + tan2) / 2.0
        A[i, 1] = -4 * v2 * s2
        A[i, 2] = (1.0 - 4.0 * v2 * s2) / 2.0
    return A


def ricker(t_ms, f_peak):
    c = math.pi * math.pi * f_peak * f_peak * np.asarray(t_ms, dtype=np.float64) ** 2 * 1e-6
    return (1 - 2 * c) * np.exp(-c)


def ricker_fft_order(nzp: int, dt_ms: float, f_peak: float, half_length_ms: int = 119,
                     notches_hz=(), notch_width_hz: float = 1.5) -> np.ndarray:
    """Ricker sampled on dt in FFT order; optional spectral notches (zero-phase)."""
    k = np.arange(nzp)
    t = np.where(k < nzp // 2 + 1, dt_ms * k, dt_ms * (k - nzp)).astype(np.float64)
    w = np.where(np.abs(t) <= half_length_ms, ricker(t, f_peak), 0.0)
    if notches_hz:
        W = np.fft.rfft(w)
        f = np.fft.rfftfreq(nzp, d=dt_ms * 1e-3)
        g = np.ones_like(f)
        for f0 in notches_hz:
            g *= 1.0 - np.exp(-0.5 * ((f - f0) / notch_width_hz) ** 2)
        w = np.fft.irfft(W * g, n=nzp)
    return w


def genexp_corr_xy(nxp, nyp, dx, dy, range_m, power=1.0) -> np.ndarray:
    """(nyp, nxp) lateral correlation surface, index i + nxp*j."""
    i = np.arange(nxp)
    j = np.arange(nyp)
    ri = np.where(i < nxp // 2 + 1, i, i - nxp) * dx
    rj = np.where(j < nyp // 2 + 1, j, j - nyp) * dy
    d = np.sqrt(ri[None, :] ** 2 + rj[:, None] ** 2) / range_m
    return np.exp(-3.0 * d ** power).astype(np.float32)


def corr2d_positive_definite(cxy: np.ndarray) -> np.ndarray:
    """ModelGeneral::makeCorr2DPositiveDefinite (src/modelgeneral.cpp:5132-5170): the lateral correlation with
    its 2D spectrum replaced by the spectrum's modulus, rescaled to keep the value at lag 0."""
    c = np.asarray(cxy, dtype=np.float64)
    spec = np.abs(np.fft.rfft2(c))
    r = np.fft.irfft2(spec, s=c.shape)
    return (r * (c[0, 0] / r[0, 0])).astype(np.float32)


def genexp_corr_t(n, dt_ms, range_ms, power):
    lag = np.arange(n + 1) * dt_ms
    return np.exp(-3.0 * (lag / range_ms) ** power).astype(np.float32)


def circ_corr_t(prior_corr_t, min_int_fq, nzp) -> np.ndarray:
    """computeCircCorrT + makeCircCorrTPosDef in FP64."""
    cnzp = nzp // 2 + 1
    n = len(prior_corr_t)
    k = np.arange(nzp)
    refk = np.where(k < cnzp, k, nzp - k)
    c = np.where(refk < n, np.asarray(prior_corr_t, dtype=np.float64)[np.minimum(refk, n - 1)], 0.0)
    s = np.fft.rfft(c)
    mag = np.abs(s)
    mag[: min(min_int_fq + 1, cnzp)] = 0.0
    out = np.fft.irfft(mag, n=nzp) * nzp
    if not out[0] > 1e-5:
        raise ValueError("circular temporal correlation undefined; increase the number of layers")
    return (out / out[0]).astype(np.float32)


def sigma0_from(stds, corr) -> np.ndarray:
    s = np.asarray(stds, dtype=np.float64)
    r01, r02, r12 = corr
    R = np.array([[1, r01, r02], [r01, 1, r12], [r02, r12, 1]], dtype=np.float64)
    S = R * s[:, None] * s[None, :]
    # eigenvalue floor at 0.1 % of the largest (setCorrelationParameters,
    # src/seismicparametersholder.cpp:121-139)
    ev, V = np.linalg.eigh(S)
    mx = ev.max()
    for q in range(3):
        if ev[q] < mx * 0.001:
            S += np.outer(V[:, q], V[:, q]) * (mx * 0.0011 - ev[q])
    # the reference keeps priorVar0 in double but fills the cubes with float(Sigma0)
    return S


def angular_corr(theta_deg, range_deg=10.0, power=1.0):
    th = np.radians(np.asarray(theta_deg, dtype=np.float64))
    d = np.abs(th[:, None] - th[None, :]) / math.radians(range_deg)
    return np.exp(-3.0 * d ** power)


@dataclass
class Scenario:
    """Everything one inversion needs, in the reference's layouts."""

    nx: int
    ny: int
    nz: int
    nxp: int
    nyp: int
    nzp: int
    dt_ms: float
    theta_deg: list
    A: np.ndarray                 # (n, 3) float32
    wavelets: np.ndarray          # (n, nzp) float32, FFT order
    corr_xy: np.ndarray           # (nyp, nxp) float32
    circ_corr_t: np.ndarray       # (nzp,) float32
    sigma0: np.ndarray            # (3, 3) float64
    err_theta_cov: np.ndarray     # (n, n) float64
    data: list                    # n x (nzp, nyp, rnxp) float32, real domain
    mean: list                    # 3 x (nzp, nyp, rnxp) float32, real domain
    wnc: float = 0.1
    low_cut: float = 5.0
    high_cut: float = 55.0
    min_rel_thick: float = 1.0
    sn: list = field(default_factory=list)
    truth: list | None = None     # 3 x (nzp, nyp, nxp) float64 (log domain)
    # non-constant simbox thickness (None: constant thickness)
    rel_thick: np.ndarray | None = None       # (nyp, nxp) float32, Simbox::getRelThick per padded trace
    wavelet_shift: np.ndarray | None = None   # (n, ny, nx) float32 ms, local wavelet time shift
    wavelet_gain: np.ndarray | None = None    # (n, ny, nx) float32, local wavelet gain
    energy_threshold: float = 0.0             # FFTGrid::interpolateSeismic
    corr_t: np.ndarray | None = None          # the temporal correlation lags circ_corr_t was made from
    min_int_fq: int = 0                       # the lowest inverted frequency index of computeCircCorrT
    corr_grad: tuple = (0.0, 0.0)             # (corrGradI, corrGradJ), ModelGeneral::getCorrGradIJ

    @property
    def ntheta(self):
        return len(self.theta_deg)

    @property
    def cnxp(self):
        return self.nxp // 2 + 1

    @property
    def rnxp(self):
        return 2 * self.cnxp

    @property
    def nbins(self):
        return self.cnxp * self.nyp * self.nzp


def variable_thickness(sc: Scenario, amp=0.3, surfaces=True, dead_traces=0, seed=7) -> Scenario:
    """A copy of ``sc`` on a simbox whose relative thickness varies laterally (1 +- amp, smooth), with
    optional local wavelet shift (+-4 ms) and gain (0.85..1.2) surfaces and ``dead_traces`` all-zero
    traces in every angle cube (interpolateSeismic input)."""
    from dataclasses import replace
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:sc.nyp, 0:sc.nxp]
    rt = (1.0 + amp * np.sin(2 * np.pi * xx / max(sc.nx, 2) + 0.4) * np.cos(2 * np.pi * yy / max(sc.ny, 2))
          ).astype(np.float32)
    shift = gain = None
    if surfaces:
        shift = rng.uniform(-4.0, 4.0, (sc.ntheta, sc.ny, sc.nx)).astype(np.float32)
        gain = rng.uniform(0.85, 1.2, (sc.ntheta, sc.ny, sc.nx))
        # as Wavelet::setGainGrid leaves a gain grid (src/wavelet.cpp:704-737): divided by its geometric mean,
        # which then multiplies the wavelet; at mean 1 the wavelet is unchanged
        gain = (gain / np.exp(np.log(gain).mean(axis=(1, 2), keepdims=True))).astype(np.float32)
    data = [d.copy() for d in sc.data]
    if dead_traces:
        idx = rng.choice(sc.nx * sc.ny, dead_traces, replace=False)
        for d in data:
            for t in idx:
                d[:, t // sc.nx, t % sc.nx] = 0.0
    return replace(sc, data=data, rel_thick=rt, wavelet_shift=shift, wavelet_gain=gain,
                   min_rel_thick=float(rt[:sc.ny, :sc.nx].min()))


def _pad_x(cube, nxp):
    rnxp = 2 * (nxp // 2 + 1)
    out = np.zeros(cube.shape[:-1] + (rnxp,), dtype=np.float32)
    out[..., :nxp] = cube
    return out


def _forward_data(dm, A, wav, nxp, snr, rng):
    """Forward model per stack in the norm-preserving spectral domain, d^ = kD(k) conj(W(k)) A m^
    (src/crava.cpp:1349-1351), white noise on top at the stack's S/N; dm = truth minus prior mean."""
    n = len(wav)
    nzp = dm[0].shape[0]
    kk = np.arange(nzp)
    kD = -1.0 + np.exp(2j * np.pi * kk / nzp)  # FFT of {-1 at 0, +1 at nzp-1}
    M = [_fftn(x) for x in dm]
    data = []
    for l in range(n):
        W = np.fft.fft(wav[l].astype(np.float64))
        op = (kD * np.conj(W))[:, None, None]
        s = np.real(_ifftn(op * sum(float(A[l, q]) * M[q] for q in range(3))))
        var_s = float(np.var(s))
        noise_sd = math.sqrt(var_s / max(snr[l] - 1.0, 1e-3))
        d = s + rng.standard_normal(s.shape) * noise_sd
        data.append(_pad_x(d, nxp))
    return data


def _err_theta_cov(data, nx, ny, nz, snr, theta_deg):
    """Error covariance between stacks (Crava::computeDataVariance + setupErrorCorrelation)."""
    n = len(data)
    dvar = []
    for l in range(n):
        inner = data[l][:nz, :ny, :nx].astype(np.float32)
        nzmask = inner != 0.0
        dvar.append(float(np.sum(inner.astype(np.float64)[nzmask] ** 2) / max(1, int(nzmask.sum()))))
    ev = np.array([dvar[l] / snr[l] for l in range(n)], dtype=np.float32)
    ac = angular_corr(theta_deg)
    etc = np.zeros((n, n), dtype=np.float64)
    for i in range(n):
        for j in range(n):
            etc[i, j] = float(np.float32(math.sqrt(ev[i]) * math.sqrt(ev[j]) * np.float32(ac[i, j])))
    return etc


def make_scenario(nx, ny, nz, theta_deg, f_peak, *, nxp=None, nyp=None, nzp=None, pad=0.25, dt_ms=4.0,
                  dx=25.0, dy=25.0, sn=4.0, stds=(0.10, 0.07, 0.05), corr=(0.7, 0.3, 0.3),
                  lateral_range=1000.0, temporal_range_ms=20.0, temporal_power=1.5, low_cut=5.0,
                  high_cut=55.0, wnc=0.1, notches_hz=(), std_scale=1.0, seed=20261203,
                  keep_truth=False, pd_corr_xy=False, corr_grad=(0.0, 0.0)) -> Scenario:
    """Build one seeded scenario.  Sizes are log-domain (ln Vp, ln Vs, ln rho)."""
    rng = np.random.default_rng(seed)
    nxp = nxp or padded_size(nx, pad)
    nyp = nyp or padded_size(ny, pad)
    nzp = nzp or padded_size(nz, pad)
    n = len(theta_deg)
    A = aki_richards_pp(theta_deg, 1500.0 / 3000.0)
    wav = np.stack([ricker_fft_order(nzp, dt_ms, f_peak, notches_hz=notches_hz) for _ in range(n)])
    wav = wav.astype(np.float32)
    cxy = genexp_corr_xy(nxp, nyp, dx, dy, lateral_range)
    if pd_corr_xy:
        cxy = corr2d_positive_definite(cxy)
    n_corr_t = max(nz, 2)
    corr_t = genexp_corr_t(n_corr_t, dt_ms, temporal_range_ms, temporal_power)
    min_int_fq = int(math.floor(low_cut * (nzp * 0.001 * dt_ms)))
    cct = circ_corr_t(corr_t, min_int_fq, nzp)
    sig0 = sigma0_from(np.asarray(stds) * std_scale, corr)

    # prior correlation spectrum (COVARIANCE transform: unnormalised)
    c3 = np.abs(np.real(np.fft.fft2(cxy.astype(np.float64))))[None, :, :] * \
        np.abs(np.real(np.fft.fft(cct.astype(np.float64))))[:, None, None]
    # one prior realisation: m = mu + L0 * IFFT_u(sqrt(c) FFT_u(w))
    L0 = np.linalg.cholesky(sig0)
    z = []
    for _ in range(3):
        w = rng.standard_normal((nzp, nyp, nxp))
        f = _fftn(w) * np.sqrt(c3)
        z.append(np.real(_ifftn(f)))
    mu = np.array([LN_VP, LN_VS, LN_RHO])
    truth = [mu[p] + sum(L0[p, q] * z[q] for q in range(3)) for p in range(3)]

    snr = sn if np.ndim(sn) else [sn] * n
    data = _forward_data([truth[p] - mu[p] for p in range(3)], A, wav, nxp, snr, rng)
    etc = _err_theta_cov(data, nx, ny, nz, snr, theta_deg)

    mean = [_pad_x(np.full((nzp, nyp, nxp), mu[p], dtype=np.float32), nxp) for p in range(3)]
    return Scenario(nx=nx, ny=ny, nz=nz, nxp=nxp, nyp=nyp, nzp=nzp, dt_ms=dt_ms, theta_deg=list(theta_deg),
                    A=A, wavelets=wav, corr_xy=cxy, circ_corr_t=cct, sigma0=sig0, err_theta_cov=etc,
                    data=data, mean=mean, wnc=wnc, low_cut=low_cut, high_cut=high_cut, sn=list(snr),
                    truth=[t for t in truth] if keep_truth else None, corr_t=corr_t, min_int_fq=min_int_fq,
                    corr_grad=(float(np.float32(corr_grad[0])), float(np.float32(corr_grad[1]))))


# ----------------------------------------------------------------------------
# The workloads the benchmark quotes (seeded, reference-shaped)
# ----------------------------------------------------------------------------

def config0(seed=20261203, **kw) -> Scenario:
    """64x64x128 cells padded to 80x80x160, 3 stacks 10/20/30 deg, 30 Hz Ricker, S/N 4."""
    return make_scenario(64, 64, 128, [10.0, 20.0, 30.0], 30.0, nxp=80, nyp=80, nzp=160, sn=4.0,
                         seed=seed, **kw)


def config1(seed=20261204, **kw) -> Scenario:
    """256^3 padded cube, 5 stacks 0-40 deg, 25 Hz Ricker notched at 2 and 80 Hz, S/N 3,
    band widened to 1-100 Hz so the notch bins are inverted."""
    return make_scenario(205, 205, 205, [0.0, 10.0, 20.0, 30.0, 40.0], 25.0, nxp=256, nyp=256, nzp=256,
                         sn=3.0, notches_hz=(2.0, 80.0), low_cut=1.0, high_cut=100.0, seed=seed, **kw)


def scaled_config1(nxp, nyp, nzp, seed=20261204, **kw) -> Scenario:
    """config1's physics on a smaller padded cube (for parity tests)."""
    return make_scenario(max(2, int(nxp / 1.25)), max(2, int(nyp / 1.25)), max(2, int(nzp / 1.25)),
                         [0.0, 10.0, 20.0, 30.0, 40.0], 25.0, nxp=nxp, nyp=nyp, nzp=nzp, sn=3.0,
                         notches_hz=(2.0, 80.0), low_cut=1.0, high_cut=100.0, seed=seed, **kw)


def config3(seed=20261206, **kw) -> Scenario:
    """Posterior simulation workload: 200^3 padded cube, 3 stacks 10/20/30 deg, config-0 prior and
    wavelet (30 Hz Ricker, S/N 4); the realisations are drawn after the inversion."""
    return make_scenario(160, 160, 160, [10.0, 20.0, 30.0], 30.0, nxp=200, nyp=200, nzp=200, sn=4.0,
                         seed=seed, **kw)


def config2(ncubes=64, seed=20261205, workers=None, **kw):
    """64 independent cubes of uneven size: nx, ny ~ U{32..192}, nz ~ U{64..160},
    each padded (25 %) to the next 2/3/5/7-smooth size; 2-8 stacks at 0-40 deg,
    Ricker peak U(15, 45) Hz, S/N U(2, 6), prior stds scaled by U(0.5, 1.5).  ``workers`` > 1 builds
    the cubes in that many spawned processes (default: one per core)."""
    rng = np.random.default_rng(seed)
    jobs = []
    for c in range(ncubes):
        nx, ny = int(rng.integers(32, 193)), int(rng.integers(32, 193))
        nz = int(rng.integers(64, 161))
        nt = int(rng.integers(2, 9))
        theta = list(np.linspace(0.0, 40.0, nt)) if nt > 1 else [20.0]
        jobs.append(((nx, ny, nz, theta, float(rng.uniform(15, 45))),
                     dict(kw, sn=float(rng.uniform(2, 6)), std_scale=float(rng.uniform(0.5, 1.5)),
                          seed=seed + 1 + c)))
    if workers is None:
        workers = min(ncubes, os.cpu_count() or 1)
    if workers <= 1:
        return [make_scenario(*a, **k) for a, k in jobs]
    # every cube has its own seed, so a pool of single-threaded generators gives the same cubes; spawned
    # workers share no state (CUDA included) with the caller
    import concurrent.futures as cf
    import multiprocessing as mp
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn"),
                                initializer=_single_threaded) as ex:
        return list(ex.map(_make_scenario_job, jobs))


def _single_threaded():
    global _FFT_WORKERS
    _FFT_WORKERS = 1


def _make_scenario_job(job):
    args, kw = job
    return make_scenario(*args, **kw)


# ----------------------------------------------------------------------------
# 4D time-lapse workloads (State4D: static + dynamic parameters, 6x6 prior)
# ----------------------------------------------------------------------------

@dataclass
class TimeLapseScenario:
    """A 6-parameter state (static ln Vp/Vs/rho and their dynamic changes) with a separable prior
    (6x6 parameter covariance times one spatial correlation), observed by several vintages.  With no
    evolution between vintages (E = I, c = 0, C = 0) every vintage sees the current state
    m_s + m_d through the 3-parameter operator, with its own noise."""

    nx: int
    ny: int
    nz: int
    nxp: int
    nyp: int
    nzp: int
    dt_ms: float
    theta_deg: list
    A: np.ndarray                 # (n, 3) float32
    wavelets: np.ndarray          # (n, nzp) float32, FFT order
    corr_xy: np.ndarray           # (nyp, nxp) float32
    circ_corr_t: np.ndarray       # (nzp,) float32
    sigma_full: np.ndarray        # (6, 6) float64: static 0..2, dynamic 3..5
    mu_static: np.ndarray         # (3,) float64, log domain
    vintages: list                # per vintage: {"data": n x (nzp, nyp, rnxp) float32, "err_theta_cov": (n, n)}
    wnc: float = 0.1
    low_cut: float = 5.0
    high_cut: float = 55.0
    min_rel_thick: float = 1.0
    # per step between vintages v and v+1: (E (6, 6), c (6,), C (6, 6)) of the time evolution
    # (TimeEvolution::getEvolutionMatrix / getMeanCorrectionTerm / getCovarianceCorrectionTerm); None: none
    evolution: list | None = None

    @property
    def ntheta(self):
        return len(self.theta_deg)

    @property
    def cnxp(self):
        return self.nxp // 2 + 1

    @property
    def nbins(self):
        return self.cnxp * self.nyp * self.nzp

    def sigma_current(self):
        """3x3 prior covariance of the current state m_s + m_d."""
        F = self.sigma_full
        return F[:3, :3] + F[3:, 3:] + F[:3, 3:] + F[3:, :3]


def make_timelapse(nx, ny, nz, theta_deg, f_peak, *, nxp=None, nyp=None, nzp=None, nvintages=2, pad=0.25,
                   dt_ms=4.0, dx=25.0, dy=25.0, sn=4.0, stds=(0.10, 0.07, 0.05), corr=(0.7, 0.3, 0.3),
                   dyn_std_range=(0.02, 0.04), static_dynamic_corr=0.3, lateral_range=1000.0,
                   temporal_range_ms=20.0, temporal_power=1.5, low_cut=5.0, high_cut=55.0, wnc=0.1,
                   seed=20261207) -> TimeLapseScenario:
    rng = np.random.default_rng(seed)
    nxp = nxp or padded_size(nx, pad)
    nyp = nyp or padded_size(ny, pad)
    nzp = nzp or padded_size(nz, pad)
    n = len(theta_deg)
    A = aki_richards_pp(theta_deg, 1500.0 / 3000.0)
    wav = np.stack([ricker_fft_order(nzp, dt_ms, f_peak) for _ in range(n)]).astype(np.float32)
    cxy = genexp_corr_xy(nxp, nyp, dx, dy, lateral_range)
    corr_t = genexp_corr_t(max(nz, 2), dt_ms, temporal_range_ms, temporal_power)
    cct = circ_corr_t(corr_t, int(math.floor(low_cut * (nzp * 0.001 * dt_ms))), nzp)
    # 6x6 parameter covariance D^1/2 (M kron R) D^1/2, M = [[1, c], [c, 1]]: positive definite
    r01, r02, r12 = corr
    R = np.array([[1, r01, r02], [r01, 1, r12], [r02, r12, 1]], dtype=np.float64)
    dyn = rng.uniform(dyn_std_range[0], dyn_std_range[1], 3)
    sd = np.concatenate([np.asarray(stds, dtype=np.float64), dyn])
    Mc = np.array([[1.0, static_dynamic_corr], [static_dynamic_corr, 1.0]])
    F = np.kron(Mc, R) * sd[:, None] * sd[None, :]
    # one realisation of the current state: (m_s - mu_s) + m_d = L6 z folded by [I I]
    c3 = np.abs(np.real(np.fft.fft2(cxy.astype(np.float64))))[None, :, :] * \
        np.abs(np.real(np.fft.fft(cct.astype(np.float64))))[:, None, None]
    L6 = np.linalg.cholesky(F)
    z = []
    for _ in range(6):
        w = rng.standard_normal((nzp, nyp, nxp))
        z.append(np.real(_ifftn(_fftn(w) * np.sqrt(c3))))
    x6 = [sum(L6[p, q] * z[q] for q in range(6)) for p in range(6)]
    dm = [x6[p] + x6[p + 3] for p in range(3)]
    snr = [sn] * n
    vint = []
    for _ in range(nvintages):
        data = _forward_data(dm, A, wav, nxp, snr, rng)
        vint.append({"data": data, "err_theta_cov": _err_theta_cov(data, nx, ny, nz, snr, theta_deg)})
    return TimeLapseScenario(nx=nx, ny=ny, nz=nz, nxp=nxp, nyp=nyp, nzp=nzp, dt_ms=dt_ms, theta_deg=list(theta_deg),
                             A=A, wavelets=wav, corr_xy=cxy, circ_corr_t=cct, sigma_full=F,
                             mu_static=np.array([LN_VP, LN_VS, LN_RHO]), vintages=vint, wnc=wnc, low_cut=low_cut,
                             high_cut=high_cut)


def config4(seed=20261207, **kw) -> TimeLapseScenario:
    """4D time-lapse workload: 256x256x192 padded cube, two vintages x 4 stacks (0-40 deg, 25 Hz Ricker,
    S/N 4 each, independent noise), static prior as config 0, dynamic log-std U(0.02, 0.04),
    static-dynamic correlation 0.3."""
    return make_timelapse(205, 205, 154, [0.0, 40.0 / 3, 80.0 / 3, 40.0], 25.0, nxp=256, nyp=256, nzp=192,
                          seed=seed, **kw)
