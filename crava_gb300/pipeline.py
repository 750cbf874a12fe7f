"""One complete inversion on the GPU, in the reference's step order.

Crava's inversion (src/crava.cpp:177-184 and :975-1285) is, for a model with
n angle stacks:

    forward transform the n data cubes (DATA) and the 3 prior-mean cubes
    (PARAMETER); forward transform the 6 prior covariance cubes and the error
    correlation cube (COVARIANCE) -- FFTCovGrids / errCorr->fftInPlace; run the
    bin loop; inverse transform the 3 posterior-mean cubes.

``Inversion`` keeps pristine copies of the real-domain inputs on the device
and restores the working cubes before every run (the transforms are in
place).  ``run(form)`` executes one inversion:

* ``"plain"``  -- the reference dataflow on the GPU, all FP32: 5+3+7 forward
  transforms, the reference-order bin kernel, 3 inverse transforms;
* ``"fp32"`` / ``"mixed"`` -- the fused form: the separable prior spectra are
  rebuilt (two tiny transforms), then cg_invert_cubes_fused: x and z passes of
  the 5+3 forward transforms, one kernel doing the y pass, the bin loop (mixed:
  FP64 for guarded bins) and the inverse y pass of the means, then the z and x
  passes of the 3 inverse transforms;
* ``"fp32_3pass"`` / ``"mixed_3pass"`` -- the same arithmetic with three-pass
  transforms around the stand-alone fused bin kernel (and the FP64 fix-up
  pass);
* ``"fp64"`` -- the fused form entirely in FP64 (accuracy reference).

On a simbox of non-constant thickness (``sc.rel_thick`` set) every run starts
with the per-trace scale-wavelet division of the data and the dead-trace
interpolation (Crava::divideDataByScaleWavelet, src/crava.cpp:174-175; FP32
in every form), the operator tables take the non-constant-thickness branch
of fillErrMultVectors, and ``outputs`` multiplies the residuals back by the
scale wavelet (multiplyDataByScaleWaveletAndWriteToFile, src/crava.cpp:231-232).
"""
from __future__ import annotations

import numpy as np
import torch

from . import api
from .synthetic import Scenario

COV_PAIRS = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]


class Inversion:
    def __init__(self, sc: Scenario, device="cuda", cond_threshold=0.0, forms=("plain", "fp32", "mixed", "fp64")):
        self.sc = sc
        self.forms = set(forms)
        self.dev = torch.device(device)
        nxp, nyp, nzp, n = sc.nxp, sc.nyp, sc.nzp, sc.ntheta
        self.thick = sc.rel_thick is not None
        if self.thick:
            self.tables = api.operator_tables_nct(sc.wavelets, sc.A, sc.nz, nzp, sc.dt_ms, sc.low_cut, sc.high_cut,
                                                  sc.min_rel_thick)
            swt = api.scale_wavelet_tables(sc.wavelets, sc.A, sc.sigma0, sc.circ_corr_t, sc.err_theta_cov, sc.nz,
                                           sc.dt_ms, sc.nz * sc.dt_ms, sc.low_cut, sc.high_cut, sc.wnc)
            dev32 = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(self.dev)  # noqa: E731
            self.sw_tables = dev32(swt)
            self.rel_thick = dev32(sc.rel_thick)
            self.wshift = dev32(sc.wavelet_shift)
            self.wgain = dev32(sc.wavelet_gain)
            self.n_bad = None
        else:
            self.tables = api.operator_tables(sc.wavelets, sc.A, sc.nz, nzp, sc.dt_ms, sc.low_cut, sc.high_cut,
                                              sc.min_rel_thick)
        self.cond_threshold = cond_threshold
        self.ws = api.Workspace(nxp, nyp, nzp, n)
        self.ws.set_model(self.tables, sc.err_theta_cov, sc.sigma0, sc.wnc, cond_threshold=cond_threshold)
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.data_in = torch.from_numpy(np.stack(sc.data)).to(**f32)
        self.mean_in = torch.from_numpy(np.stack(sc.mean)).to(**f32)
        self.corr_xy = torch.from_numpy(np.ascontiguousarray(sc.corr_xy, dtype=np.float32)).to(**f32)
        self.circ_t = torch.from_numpy(np.ascontiguousarray(sc.circ_corr_t, dtype=np.float32)).to(**f32)
        self.grad = api.corr_grad(sc)
        shape = tuple(self.data_in.shape[1:])
        self.data = [torch.empty(shape, **f32) for _ in range(n)]
        self.mean = [torch.empty(shape, **f32) for _ in range(3)]
        self.cov = [torch.empty(shape, **f32) for _ in range(6)]
        if "plain" in self.forms:
            self.cov_in = torch.empty((6,) + shape, **f32)
            self.err_in = torch.empty(shape, **f32)
            self.errcorr = torch.empty(shape, **f32)
            s = torch.cuda.current_stream()
            gi, gj = self.grad
            for t, (p, q) in enumerate(COV_PAIRS):
                api.check_call("cg_fill_param_corr", self.cov_in[t], nxp, nyp, nzp, self.corr_xy, self.circ_t, gi,
                               gj, float(np.float32(sc.sigma0[p, q])), s)
            api.check_call("cg_fill_err_corr", self.err_in, nxp, nyp, nzp, self.corr_xy, gi, gj, s)
        if "fp64" in self.forms:
            f64 = dict(dtype=torch.float64, device=self.dev)
            self.data64 = [torch.empty(shape, **f64) for _ in range(n)]
            self.mean64 = [torch.empty(shape, **f64) for _ in range(3)]
            self.cov64 = [torch.empty(shape, **f64) for _ in range(6)]
        torch.cuda.synchronize()

    # -- bookkeeping -------------------------------------------------------
    def restore(self, form):
        """Reset the working cubes to the real-domain inputs (not part of a run)."""
        if form == "fp64":
            for l, d in enumerate(self.data64):
                d.copy_(self.data_in[l])
            for p, m in enumerate(self.mean64):
                m.copy_(self.mean_in[p])
            if self.thick:   # the FP32 data scaling feeds the FP64 cubes
                for l, d in enumerate(self.data):
                    d.copy_(self.data_in[l])
            return
        for l, d in enumerate(self.data):
            d.copy_(self.data_in[l])
        for p, m in enumerate(self.mean):
            m.copy_(self.mean_in[p])
        if form == "plain":
            for t in range(6):
                self.cov[t].copy_(self.cov_in[t])
            self.errcorr.copy_(self.err_in)

    # -- one inversion -----------------------------------------------------
    def scale_data(self, stream=None):
        """Crava::divideDataByScaleWavelet + interpolateSeismic on the FP32 working data cubes."""
        sc = self.sc
        self.n_bad = api.divide_by_scale_wavelet(self.data, sc.nx, sc.ny, sc.nz, sc.nxp, self.sw_tables,
                                                 self.rel_thick, sc.dt_ms, sc.nz * sc.dt_ms, sc.low_cut,
                                                 sc.high_cut, sc.energy_threshold, shift=self.wshift,
                                                 gain=self.wgain, stream=stream)

    def run(self, form, stream=None):
        sc = self.sc
        nxp = sc.nxp
        if self.thick:
            self.scale_data(stream)
            if form == "fp64":
                for l, d in enumerate(self.data64):
                    d.copy_(self.data[l])
        if form == "plain":
            api.fft_in_place_batch(self.data, nxp, api.DATA, stream=stream)
            api.fft_in_place_batch(self.mean, nxp, api.PARAMETER, stream=stream)
            api.fft_in_place_batch(self.cov + [self.errcorr], nxp, api.COVARIANCE, stream=stream)
            self.ws.invert_plain(self.data, self.mean, self.cov, self.errcorr, stream=stream)
            api.fft_in_place_batch(self.mean, nxp, api.PARAMETER, inverse=True, stream=stream)
        elif form in ("fp32", "mixed"):
            prec = api.PREC_MIXED if form == "mixed" else api.PREC_FP32
            main = stream if stream is not None else torch.cuda.current_stream()
            if self.ws_fused_y():
                self.ws.prior_spectra(self.corr_xy, self.circ_t, api.PREC_FP32, stream=main, grad=self.grad)
                self.ws.invert_cubes(self.data, self.mean, self.cov, prec, stream=main)
            else:
                # the prior spectra depend on the model only: a side branch beside the forward transforms
                side = self._prior_stream()
                side.wait_stream(main)
                self.ws.prior_spectra(self.corr_xy, self.circ_t, api.PREC_FP32, stream=side, grad=self.grad)
                api.fft_in_place_batch(self.data + self.mean, nxp, api.DATA, stream=main)
                main.wait_stream(side)
                self.ws.invert_fused(self.data, self.mean, self.cov, prec, stream=main)
                api.fft_in_place_batch(self.mean, nxp, api.PARAMETER, inverse=True, stream=main)
        elif form in ("fp32_3pass", "mixed_3pass"):
            prec = api.PREC_MIXED if form == "mixed_3pass" else api.PREC_FP32
            self.ws.prior_spectra(self.corr_xy, self.circ_t, api.PREC_FP32, stream=stream, grad=self.grad)
            api.fft_in_place_batch(self.data, nxp, api.DATA, stream=stream)
            api.fft_in_place_batch(self.mean, nxp, api.PARAMETER, stream=stream)
            self.ws.invert_fused(self.data, self.mean, self.cov, prec, stream=stream)
            api.fft_in_place_batch(self.mean, nxp, api.PARAMETER, inverse=True, stream=stream)
        elif form == "fp64":
            self.ws.prior_spectra(self.corr_xy, self.circ_t, api.PREC_FP64, stream=stream, grad=self.grad)
            for d in self.data64:
                api.fft_in_place(d, nxp, api.DATA, stream=stream)
            for m in self.mean64:
                api.fft_in_place(m, nxp, api.PARAMETER, stream=stream)
            self.ws.invert_fused(self.data64, self.mean64, self.cov64, api.PREC_FP64, stream=stream)
            for m in self.mean64:
                api.inv_fft_in_place(m, nxp, api.PARAMETER, stream=stream)
        else:
            raise ValueError(form)

    def capture(self, form):
        """The inversion of ``form`` on the working cubes captured once as a CUDA graph (after one warm run,
        which creates the transform tables and kernel attributes outside the capture); replay() runs the
        same launches on the same buffers with one host call, so a small cube's step is not bound by the
        host's launch rate.  Restore the inputs before each replay, as before each run."""
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.restore(form)
            self.run(form)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        with torch.cuda.graph(g):
            self.run(form)
        torch.cuda.synchronize()
        return g

    def ws_fused_y(self):
        """Whether cg_invert_cubes_fused takes a y-fused, y-split or z-chunked route for this cube (tuning
        table CG_TUNE_FUSED_Y for its y length, separable prior): those interleave the y transforms with the
        bins and run as one call."""
        sc = self.sc
        if any(self.grad):
            return False
        zc = api.lib().cg_tune_get(4, sc.nyp)  # CG_TUNE_FUSED_Y
        return zc == 2 or zc >= 4 or (zc == 1 and sc.nyp in (128, 200, 256))

    def _prior_stream(self):
        if getattr(self, "_pstream", None) is None:
            self._pstream = torch.cuda.Stream()
        return self._pstream

    def run_cold(self, form="mixed", stream=None):
        """One inversion of a model the workspace has not seen: the per-model work happens inside the call,
        as the reference does it inside computePostMeanResidAndFFTCov (the per-k operator and error factors,
        fillErrMultVectors / getNextErrorVariance, src/crava.cpp:1108-1120).  The forward transforms of the
        data and prior means are queued first; the host builds the operator tables (from the wavelets) while
        the GPU transforms, then queues their upload, the per-k table kernel (cg_workspace_set_model_async)
        and the prior spectra on a high-priority side stream, so that they run beside the transforms (their
        single-warp CTAs take the SM slots the transform CTAs free first); the bin kernel waits for both,
        then the inverse transforms."""
        sc = self.sc
        if self.thick:
            raise ValueError("run_cold covers the constant-thickness model")
        prec = {"mixed": api.PREC_MIXED, "fp32": api.PREC_FP32}[form]
        nxp = sc.nxp
        main = stream if stream is not None else torch.cuda.current_stream()
        if getattr(self, "_side", None) is None:
            self._side = torch.cuda.Stream(priority=-100)  # mapped to the device's highest priority
        side = self._side
        side.wait_stream(main)  # the workspace's earlier work is done before its tables change
        # DATA and PARAMETER cubes share the 1/sqrt(N) scaling: one batched launch per pass for all of them
        api.fft_in_place_batch(self.data + self.mean, nxp, api.DATA, stream=main)
        tables = api.operator_tables(sc.wavelets, sc.A, sc.nz, sc.nzp, sc.dt_ms, sc.low_cut, sc.high_cut,
                                     sc.min_rel_thick)
        self.ws.set_model(tables, sc.err_theta_cov, sc.sigma0, sc.wnc, cond_threshold=self.cond_threshold,
                          stream=side, asynchronous=True)
        self.ws.prior_spectra(self.corr_xy, self.circ_t, api.PREC_FP32, stream=side, grad=self.grad)
        main.wait_stream(side)
        self.ws.invert_fused(self.data, self.mean, self.cov, prec, stream=main)
        api.fft_in_place_batch(self.mean, nxp, api.PARAMETER, inverse=True, stream=main)

    # -- output grids (the steps after the bin loop) ------------------------
    def outputs(self, form, stream=None):
        """The reference's steps after the inversion, on the working cubes of ``form``:
        invFFTCovGrids (the 6 posterior covariance spectra to the real domain, in place), updatePriorVar +
        createPostCov00 (src/seismicparametersholder.cpp:771-807), the residual spectra to the real domain
        (src/crava.cpp:229-244, in place), and Vp / Vs / density = exp(posterior mean) as new cubes
        (ParameterOutput::writeParameters, src/parameteroutput.cpp:87-108).
        Returns (post_var0 (3,3), post_cov00 (3, nz), [Vp, Vs, rho] device cubes)."""
        sc = self.sc
        nxp = sc.nxp
        cov = self.cov64 if form == "fp64" else self.cov
        data = self.data64 if form == "fp64" else self.data
        if form == "fp64":
            raise ValueError("output grids are produced from the FP32 forms")
        api.fft_in_place_batch(cov, nxp, api.COVARIANCE, inverse=True, stream=stream)
        post_var0, post_cov00 = api.cov_origin(cov, nxp, sc.nz, stream=stream)
        api.fft_in_place_batch(data, nxp, api.DATA, inverse=True, stream=stream)
        if self.thick:
            api.multiply_by_scale_wavelet(data, sc.nx, sc.ny, nxp, self.sw_tables, self.rel_thick, sc.dt_ms,
                                          shift=self.wshift, gain=self.wgain, stream=stream)
        elastic = [m.clone() for m in self.mean]
        for e in elastic:
            api.exp_transform(e, stream=stream)
        return post_var0, post_cov00, elastic

    # -- local noise -------------------------------------------------------
    def correct_local_noise(self, form, noise_scale: torch.Tensor, post_var0, G=None, stream=None):
        """Crava::correctAlphaBetaRho (src/crava.cpp:266-282, 2471-2569) on the posterior means of ``form``
        (real domain, after ``run``): noise_scale (ntheta, ny, nx) float64 device tensor of local noise
        scales, post_var0 the 3x3 posterior variance at the origin (``outputs``).  G defaults to
        ``api.local_noise_g``.  Returns the per-trace matrices sigmamd (ny, nx, 9) for simulation."""
        sc = self.sc
        if form == "fp64":
            raise ValueError("the local-noise correction works on the FP32 forms")
        s0 = np.asarray(sc.sigma0, dtype=np.float64)
        if G is None:
            G = api.local_noise_g(sc.err_theta_cov, s0, post_var0)
        mean0 = [self.mean_in[p] for p in range(3)]
        sigmamd = torch.empty((sc.ny, sc.nx, 9), dtype=torch.float64, device=self.dev)
        api.correct_alpha_beta_rho(self.mean, mean0, sc.nx, sc.ny, sc.nz, sc.nxp, G, sc.err_theta_cov, s0, post_var0,
                                   noise_scale, sigmamd, stream=stream)
        return sigmamd

    # -- results -----------------------------------------------------------
    def results(self, form):
        """(posterior-mean real cubes, residual spectra, posterior-cov spectra) as numpy."""
        if form == "fp64":
            mean, data, cov = self.mean64, self.data64, self.cov64
        else:
            mean, data, cov = self.mean, self.data, self.cov
        nxp = self.sc.nxp
        pm = np.stack([m[:, :, :nxp].cpu().numpy() for m in mean])
        res = np.stack([api.as_spectrum(d).cpu().numpy() for d in data])
        pc = np.stack([api.as_spectrum(c).cpu().numpy() for c in cov])
        return pm, res, pc

    def algorithmic_bytes(self, form):
        """Minimum HBM traffic of one run: single-pass transforms and the bin kernel."""
        sc = self.sc
        n = sc.ntheta
        cells = sc.nxp * sc.nyp * sc.nzp
        bins = sc.nbins
        per_fft = 4 * cells + 8 * bins
        inband = int(self.tables["band"].sum()) * sc.cnxp * sc.nyp
        outband = bins - inband
        word = 8 if form == "fp64" else 4
        if form == "plain":
            nfft = n + 3 + 7 + 3
            binb = inband * 2 * word * ((n + 3 + 7) + (n + 3 + 6)) + outband * 2 * word * (6 + 6)
        else:
            nfft = n + 3 + 3
            binb = inband * 2 * word * ((n + 3) + (n + 3 + 6)) + outband * 2 * word * 6
        return nfft * per_fft * (word // 4) + binb


# State4D grid orders (src/state4d.cpp): static-static, static-dynamic and dynamic-dynamic blocks of the
# 6x6 covariance (parameters 0..2 static, 3..5 dynamic)
SS_PAIRS = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
SD_PAIRS = [(0, 3), (0, 4), (0, 5), (1, 3), (1, 4), (1, 5), (2, 3), (2, 4), (2, 5)]
DD_PAIRS = [(3, 3), (3, 4), (3, 5), (4, 4), (4, 5), (5, 5)]
# merge/split order of the current 3x3 covariance (00 01 02 11 12 22) -> bin-loop order (00 11 22 01 02 12)
MERGE_TO_BIN = [0, 3, 5, 1, 2, 4]


class TimeLapse:
    """4D time-lapse inversion in the reference's sequential form, per vintage:

        State4D::merge / mergeCov (src/state4d.cpp:140-299) -> current prior spectra;
        forward transform of the vintage's data cubes (DATA);
        the bin loop with the 4D branch of findParameterVariances
        (src/seismicparametersholder.cpp:366-373), plain form (the prior is no longer separable);
        State4D::split (src/state4d.cpp:301-580) -> updated static and dynamic state;
        inverse transform of a copy of the current posterior mean (the vintage's output).

    The state is held as spectra (27 cubes: 3 + 3 means, 6 + 9 + 6 covariance blocks), built from the
    separable prior exactly as the reference builds its 4D grids (fillInParamCorr x Sigma entry, then a
    COVARIANCE transform).  Between vintages v and v + 1 the state evolves when the scenario gives a time
    evolution (State4D::evolve, src/state4d.cpp:800-996, called by ModelGeneral::advanceTime before the next
    merge, src/modelgeneral.cpp:4852-4870): mu <- E mu + c, Sig <- E Sig E^T + C Re(lambda), lambda the
    transformed GenExp correlation evolve builds (ranges nx/3, ny/3, 20); with none, nothing evolves
    (E = I, c = 0, C = 0).  The reference's
    inverse-then-forward transform of the posterior means between the bin loop and split
    (src/crava.cpp:1262-1264, :352-354) is an identity up to rounding and is not repeated here.
    """

    def __init__(self, tl, device="cuda"):
        self.tl = tl
        dev = torch.device(device)
        f32 = dict(dtype=torch.float32, device=dev)
        nxp, nyp, nzp, n = tl.nxp, tl.nyp, tl.nzp, tl.ntheta
        cnxp, rnxp = api.dims(nxp)
        shape = (nzp, nyp, rnxp)
        self.shape = shape
        s = torch.cuda.current_stream()
        corr_xy = torch.from_numpy(np.ascontiguousarray(tl.corr_xy, dtype=np.float32)).to(**f32)
        circ_t = torch.from_numpy(np.ascontiguousarray(tl.circ_corr_t, dtype=np.float32)).to(**f32)
        F = tl.sigma_full

        def cov_spec(i, j):
            c = torch.empty(shape, **f32)
            api.check_call("cg_fill_param_corr", c, nxp, nyp, nzp, corr_xy, circ_t, 0.0, 0.0,
                           float(np.float32(F[i, j])), s)
            api.fft_in_place(c, nxp, api.COVARIANCE)
            return c

        self.ss0 = [cov_spec(i, j) for i, j in SS_PAIRS]
        self.sd0 = [cov_spec(i, j) for i, j in SD_PAIRS]
        self.dd0 = [cov_spec(i, j) for i, j in DD_PAIRS]
        self.mu_s0 = []
        for p in range(3):
            m = torch.zeros(shape, **f32)
            m[:, :, :nxp] = float(tl.mu_static[p])
            api.fft_in_place(m, nxp, api.PARAMETER)
            self.mu_s0.append(m)
        self.mu_d0 = [torch.zeros(shape, **f32) for _ in range(3)]
        # working state (restored from the pristine copies above before a run)
        self.mu_s = [torch.empty(shape, **f32) for _ in range(3)]
        self.mu_d = [torch.empty(shape, **f32) for _ in range(3)]
        self.ss = [torch.empty(shape, **f32) for _ in range(6)]
        self.sd = [torch.empty(shape, **f32) for _ in range(9)]
        self.dd = [torch.empty(shape, **f32) for _ in range(6)]
        self.mu_cur = [torch.empty(shape, **f32) for _ in range(3)]
        self.cov_cur = [torch.empty(shape, **f32) for _ in range(6)]
        self.data = [torch.empty(shape, **f32) for _ in range(n)]
        self.post_mean = [torch.empty(shape, **f32) for _ in range(3)]
        self.errcorr = torch.empty(shape, **f32)
        api.check_call("cg_fill_err_corr", self.errcorr, nxp, nyp, nzp, corr_xy, 0.0, 0.0, s)
        api.fft_in_place(self.errcorr, nxp, api.COVARIANCE)
        self.evolution = getattr(tl, "evolution", None)
        self.lam = None
        if self.evolution:
            # the increment's spatial correlation State4D::evolve transforms (its fixed ranges)
            self.lam = torch.empty(shape, **f32)
            api.fill_genexp_corr(self.lam, nxp, float(np.float32(tl.nx)) / 3.0, float(np.float32(tl.ny)) / 3.0,
                                 20.0)
            api.fft_in_place(self.lam, nxp, api.COVARIANCE)
        self.tables = api.operator_tables(tl.wavelets, tl.A, tl.nz, nzp, tl.dt_ms, tl.low_cut, tl.high_cut,
                                          tl.min_rel_thick)
        self.data_in, self.ws = [], []
        for v in tl.vintages:
            self.data_in.append(torch.from_numpy(np.stack(v["data"])).to(**f32))
            ws = api.Workspace(nxp, nyp, nzp, n)
            ws.set_model(self.tables, v["err_theta_cov"], tl.sigma_current(), tl.wnc, is4d=True)
            self.ws.append(ws)
        self.nfail_split = []
        torch.cuda.synchronize()

    def restore(self):
        """Reset the state to the prior (not part of a run)."""
        for dst, src in ((self.mu_s, self.mu_s0), (self.mu_d, self.mu_d0), (self.ss, self.ss0),
                         (self.sd, self.sd0), (self.dd, self.dd0)):
            for a, b in zip(dst, src):
                a.copy_(b)
        for ws in self.ws:
            ws.reset_stats()
        self.nfail_split = []

    def run_vintage(self, v, stream=None, form="plain"):
        """One vintage.  form "plain": the reference's three passes (merge, the 4D bin loop, split) as
        separate kernels; "fp32" / "mixed": one pass per bin (cg_vintage4d), bit for bit the plain form in
        FP32, or with the FP64 redo of guarded bins."""
        nxp = self.tl.nxp
        if form in ("fp32", "mixed"):
            for l, d in enumerate(self.data):
                d.copy_(self.data_in[v][l])
            api.fft_in_place_batch(self.data, nxp, api.DATA, stream=stream)
            prec = api.PREC_MIXED if form == "mixed" else api.PREC_FP32
            self.nfail_split.append(api.vintage4d(self.ws[v], self.mu_s, self.mu_d, self.ss, self.sd, self.dd,
                                                  self.data, self.errcorr, self.post_mean, nxp, precision=prec,
                                                  stream=stream))
            api.fft_in_place_batch(self.post_mean, nxp, api.PARAMETER, inverse=True, stream=stream)
            return
        if form != "plain":
            raise ValueError(form)
        api.state4d_merge(self.mu_s, self.mu_d, self.ss, self.sd, self.dd, self.mu_cur, self.cov_cur, nxp,
                          stream=stream)
        for l, d in enumerate(self.data):
            d.copy_(self.data_in[v][l])
        api.fft_in_place_batch(self.data, nxp, api.DATA, stream=stream)
        self.ws[v].invert_plain(self.data, self.mu_cur, [self.cov_cur[t] for t in MERGE_TO_BIN], self.errcorr,
                                stream=stream)
        self.nfail_split.append(api.state4d_split(self.mu_s, self.mu_d, self.ss, self.sd, self.dd, self.mu_cur,
                                                  self.cov_cur, nxp, stream=stream))
        for p in range(3):
            self.post_mean[p].copy_(self.mu_cur[p])
        api.fft_in_place_batch(self.post_mean, nxp, api.PARAMETER, inverse=True, stream=stream)

    def evolve(self, step, stream=None):
        """State4D::evolve with time step `step` of the scenario's evolution (between vintages step and
        step + 1)."""
        E, c, C = self.evolution[step]
        api.state4d_evolve(self.mu_s, self.mu_d, self.ss, self.sd, self.dd, self.tl.nxp, E, c, C, lam=self.lam,
                           stream=stream)

    def run(self, stream=None, form="plain"):
        for v in range(len(self.tl.vintages)):
            if v > 0 and self.evolution:
                self.evolve(v - 1, stream=stream)
            self.run_vintage(v, stream=stream, form=form)

    def state(self):
        """(mu_s, mu_d, ss, sd, dd) spectra as numpy complex arrays."""
        return [[api.as_spectrum(x).cpu().numpy() for x in grp]
                for grp in (self.mu_s, self.mu_d, self.ss, self.sd, self.dd)]

    def algorithmic_bytes(self):
        """Joint 6-state / (vintages x n)-data solve lower bound: per bin, read the data and the 6 prior
        means, write 6 means, the residuals and the 21 covariance entries (8 B each), plus one DATA
        transform (4 B/cell + 8 B/bin) per data cube."""
        tl = self.tl
        nd = len(tl.vintages) * tl.ntheta
        cells = tl.nxp * tl.nyp * tl.nzp
        return tl.nbins * 8 * ((nd + 6) + (6 + nd + 21)) + nd * (4 * cells + 8 * tl.nbins)
