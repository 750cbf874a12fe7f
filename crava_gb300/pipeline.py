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
  rebuilt (two tiny transforms), 5+3 forward transforms, the fused bin kernel
  (mixed: plus the FP64 fix-up pass), 3 inverse transforms;
* ``"fp64"`` -- the fused form entirely in FP64 (accuracy reference).
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
        self.tables = api.operator_tables(sc.wavelets, sc.A, sc.nz, nzp, sc.dt_ms, sc.low_cut, sc.high_cut,
                                          sc.min_rel_thick)
        self.ws = api.Workspace(nxp, nyp, nzp, n)
        self.ws.set_model(self.tables, sc.err_theta_cov, sc.sigma0, sc.wnc, cond_threshold=cond_threshold)
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.data_in = torch.from_numpy(np.stack(sc.data)).to(**f32)
        self.mean_in = torch.from_numpy(np.stack(sc.mean)).to(**f32)
        self.corr_xy = torch.from_numpy(np.ascontiguousarray(sc.corr_xy, dtype=np.float32)).to(**f32)
        self.circ_t = torch.from_numpy(np.ascontiguousarray(sc.circ_corr_t, dtype=np.float32)).to(**f32)
        shape = tuple(self.data_in.shape[1:])
        self.data = [torch.empty(shape, **f32) for _ in range(n)]
        self.mean = [torch.empty(shape, **f32) for _ in range(3)]
        self.cov = [torch.empty(shape, **f32) for _ in range(6)]
        if "plain" in self.forms:
            self.cov_in = torch.empty((6,) + shape, **f32)
            self.err_in = torch.empty(shape, **f32)
            self.errcorr = torch.empty(shape, **f32)
            s = torch.cuda.current_stream()
            for t, (p, q) in enumerate(COV_PAIRS):
                api.check_call("cg_fill_param_corr", self.cov_in[t], nxp, nyp, nzp, self.corr_xy, self.circ_t, 0.0,
                               0.0, float(np.float32(sc.sigma0[p, q])), s)
            api.check_call("cg_fill_err_corr", self.err_in, nxp, nyp, nzp, self.corr_xy, 0.0, 0.0, s)
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
    def run(self, form, stream=None):
        sc = self.sc
        nxp = sc.nxp
        if form == "plain":
            api.fft_in_place_batch(self.data, nxp, api.DATA, stream=stream)
            api.fft_in_place_batch(self.mean, nxp, api.PARAMETER, stream=stream)
            api.fft_in_place_batch(self.cov + [self.errcorr], nxp, api.COVARIANCE, stream=stream)
            self.ws.invert_plain(self.data, self.mean, self.cov, self.errcorr, stream=stream)
            api.fft_in_place_batch(self.mean, nxp, api.PARAMETER, inverse=True, stream=stream)
        elif form in ("fp32", "mixed"):
            prec = api.PREC_MIXED if form == "mixed" else api.PREC_FP32
            self.ws.prior_spectra(self.corr_xy, self.circ_t, api.PREC_FP32, stream=stream)
            api.fft_in_place_batch(self.data, nxp, api.DATA, stream=stream)
            api.fft_in_place_batch(self.mean, nxp, api.PARAMETER, stream=stream)
            self.ws.invert_fused(self.data, self.mean, self.cov, prec, stream=stream)
            api.fft_in_place_batch(self.mean, nxp, api.PARAMETER, inverse=True, stream=stream)
        elif form == "fp64":
            self.ws.prior_spectra(self.corr_xy, self.circ_t, api.PREC_FP64, stream=stream)
            for d in self.data64:
                api.fft_in_place(d, nxp, api.DATA, stream=stream)
            for m in self.mean64:
                api.fft_in_place(m, nxp, api.PARAMETER, stream=stream)
            self.ws.invert_fused(self.data64, self.mean64, self.cov64, api.PREC_FP64, stream=stream)
            for m in self.mean64:
                api.inv_fft_in_place(m, nxp, api.PARAMETER, stream=stream)
        else:
            raise ValueError(form)

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
