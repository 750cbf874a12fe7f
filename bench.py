"""Benchmark: 256^3 FFT-domain AVO inversion on one GB300 (per GPU replica).

Workload: a 256x256x256 padded cube, 5 angle stacks at 0/10/20/30/40 deg, a
25 Hz Ricker wavelet notched at 2 and 80 Hz, S/N 3, inversion band 1-100 Hz
(seeded synthetic data, generated on the host).  One step = one complete
inversion (forward transforms of the 5 data and 3 prior-mean cubes, the
prior/error spectra, the per-bin posterior, inverse transforms of the 3
posterior means), inputs resident in HBM.

Forms timed: "plain" (the reference dataflow on the GPU, all FP32), "fp32"
(fused, all FP32), "mixed" (fused, FP32 bulk + FP64-guarded bins; the
headline).  "fp64" runs once as the accuracy reference.  Each form's step is
captured once as a CUDA graph and replayed per timed step (the same launches
on the same buffers; inputs restored and L2 flushed between steps, outside
the events); the same steps issued launch by launch are reported beside them
(forms_ms_eager).

Metric: Mbins/s = (cnxp*nyp*nzp bins) / (ms per inversion).  With --gpus N
under torchrun each rank runs an independent replica (the path does not shard
a cube; cubes are independent), value = total bins / max time.

--impl reference times the reference algorithm on the host cores (the C
oracle port: its FFTs and its lib_matr-order bin loop, OpenMP over k like the
reference): one complete inversion per step, operator tables from the
oracle's own restatement.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "256^3 AVO inversion ms, Mbins/s: mixed vs plain FP32 GPU at <=1e-5 err vs FP64"
WORKLOAD = ("256^3 padded cube, 5 stacks 0-40 deg, 25 Hz Ricker notched at 2/80 Hz, S/N 3, "
            "band 1-100 Hz, seeded synthetic inputs")


def load_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    p = os.path.join(REPO, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """SM clock and clock-event reasons of the measured GPU, sampled during the timed region.

    Samples every 10 ms from a separate process (crava_gb300.clocks, NVML by GPU UUID); falls back to
    nvidia-smi every 200 ms when NVML cannot be opened.  Read-only: no GPU setting is touched."""

    SMI_FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                  "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                  "clocks_event_reasons.sw_power_cap")
    SMI_NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.kind = None
        self.lines = []
        self.t = None
        self.ready = threading.Event()

    def _uuid(self):
        try:
            import torch
            u = str(torch.cuda.get_device_properties(self.gpu).uuid)
            return u if u.startswith("GPU-") else "GPU-" + u
        except Exception:
            return None

    def start(self):
        uuid = self._uuid()
        cmds = []
        if uuid:
            cmds.append(("nvml", [sys.executable, "-m", "crava_gb300.clocks", "--uuid", uuid, "--interval-ms", "10"]))
        cmds.append(("smi", ["nvidia-smi", "-i", uuid or str(self.gpu), f"--query-gpu={self.SMI_FIELDS}",
                             "--format=csv,noheader,nounits", "-lms", "200"]))
        for kind, cmd in cmds:
            try:
                self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
                                             cwd=REPO)
            except Exception:
                self.proc = None
                continue
            self.kind = kind
            self.lines = []
            self.ready.clear()
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            if self.ready.wait(timeout=20):
                return
            self._kill()
        self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            line = line.strip()
            if line == "ready":
                self.ready.set()
                continue
            self.lines.append(line)
            self.ready.set()

    def _kill(self):
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)

    def stop(self):
        if self.proc is None:
            return None
        self._kill()
        sm, mx, reasons = [], [], set()
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            try:
                if self.kind == "nvml" and len(parts) == 4:
                    sm.append(float(parts[0]))
                    mx.append(float(parts[1]))
                    from crava_gb300.clocks import REASONS
                    bits = int(parts[3])
                    reasons.update(name for bit, name in REASONS.items() if bits & bit)
                elif self.kind == "smi" and len(parts) >= 7:
                    sm.append(float(parts[0]))
                    mx.append(float(parts[1]))
                    reasons.update(n for n, v in zip(self.SMI_NAMES, parts[3:7]) if v.lower().startswith("active"))
            except ValueError:
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "source": "NVML every 10 ms" if self.kind == "nvml" else "nvidia-smi every 200 ms"}


def dist_setup():
    from crava_gb300 import replicas
    return replicas.world()


def barrier(world):
    from crava_gb300 import replicas
    replicas.barrier(world)


def max_over_ranks(x, world):
    from crava_gb300 import replicas
    return replicas.max_over_ranks(x, world, device="cuda")


def rel(a, b):
    import numpy as np
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


# ---------------------------------------------------------------------------
# CPU reference (oracle port): one complete inversion on the host cores
# ---------------------------------------------------------------------------
COV_PAIRS = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]


def cpu_inversion(sc, tables, prec="f", threads=None):
    """The whole inversion of ``sc`` on the CPU oracle, in the reference's dataflow and order
    (Crava::computePostMeanResidAndFFTCov, src/crava.cpp:975-1285, with the data and prior-mean transforms
    of src/crava.cpp:177-184): n data + 3 prior-mean forward transforms, the 6 prior covariance cubes
    (fillInParamCorr) and the error correlation cube (fillInErrCorr) filled and forward transformed, the
    lib_matr-order bin loop over every bin (OpenMP over k), 3 inverse transforms of the posterior means.
    prec "f" is the reference's FP32 arithmetic, "d" the FP64 oracle.  ``tables`` are the per-k FP32
    operator tables.  Returns (seconds per phase, posterior-mean real cubes, residual spectra, covariance
    spectra, failed-Cholesky count)."""
    import numpy as np
    from oracle import oracle as O
    nt = threads or os.cpu_count() or 1
    tab = dict(tables)
    tab["nxp"] = sc.nxp
    if prec == "d":
        tab = {k: (v.astype(np.complex128) if hasattr(v, "dtype") and v.dtype == np.complex64 else v)
               for k, v in tab.items()}
    t = {}
    t0 = time.perf_counter()
    data = [O.fft3d_r2c(d, sc.nxp, O.DATA, prec, nt) for d in sc.data]
    mean = [O.fft3d_r2c(m, sc.nxp, O.PARAMETER, prec, nt) for m in sc.mean]
    t["data_mean_fft_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    covs = []
    for (p, q) in COV_PAIRS:
        c = O.fill_param_corr(sc.nxp, sc.nyp, sc.nzp, sc.corr_xy, sc.circ_corr_t, 0, 0,
                              float(np.float32(sc.sigma0[p, q])), prec=prec)
        covs.append(O.fft3d_r2c(c, sc.nxp, O.COVARIANCE, prec, nt))
    ec = O.fft3d_r2c(O.fill_err_corr(sc.nxp, sc.nyp, sc.nzp, sc.corr_xy, prec=prec), sc.nxp, O.COVARIANCE, prec,
                     nt)
    t["cov_fill_fft_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    s0 = np.asarray(sc.sigma0, dtype=np.float64).astype(np.float32).astype(np.float64)
    res, mu, cov, nf = O.invert_bins(data, mean, covs, ec, tab, sc.err_theta_cov, s0, sc.wnc, prec=prec,
                                     nthreads=nt)
    t["bins_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    post = np.stack([O.fft3d_c2r(m, sc.nxp, O.PARAMETER, prec, nt)[:, :, :sc.nxp] for m in mu])
    t["inverse_fft_s"] = time.perf_counter() - t0
    t["total_s"] = sum(t.values())
    return t, post, np.stack(res), np.stack(cov), nf


def simulated_fields_vs_fp64(sc, inv, threads):
    """One realisation of the posterior, GPU chain (mixed inversion, per-bin factor, inverse transforms, mean
    add) against the FP64 oracle chain (FP64 inversion of the same inputs with the same operator tables, FP64
    factor and transforms), both fed the same noise field: the reference's own fillInComplexNoise stream
    (seed 231171) injected into cg_simulate_fields.  Relative L2 error of the three fields, and of the
    fields' deviation from the posterior mean (the simulated part alone)."""
    import numpy as np
    import torch
    from crava_gb300 import api
    from oracle import oracle as O
    nxp = sc.nxp
    noise = O.fill_complex_noise(nxp, sc.nyp, sc.nzp, 231171, 3)
    _, post64, _, cov64, _ = cpu_inversion(sc, inv.tables, "d", threads)
    z64 = O.simulate_bins(list(cov64), list(noise), prec="d", nthreads=threads)
    dev64 = np.stack([O.fft3d_c2r(z, nxp, O.PARAMETER, "d", threads)[:, :, :nxp] for z in z64])
    f64 = dev64 + post64
    chol, _ = api.posterior_cholesky(inv.cov, nxp)
    _, rnxp = api.dims(nxp)
    fields = [torch.empty((sc.nzp, sc.nyp, rnxp), device="cuda") for _ in range(3)]
    nz = [torch.from_numpy(np.ascontiguousarray(x).view(np.float32)).cuda() for x in noise]
    api.simulate_fields(chol, fields, nxp, noise=nz, post_mean=inv.mean)
    torch.cuda.synchronize()
    got = np.stack([f.cpu().numpy()[:, :, :nxp] for f in fields])
    pm = np.stack([m.cpu().numpy()[:, :, :nxp] for m in inv.mean])
    return {"fields_rel_err": float(f"{rel(got, f64):.3e}"),
            "simulated_part_rel_err": float(f"{rel(got - pm, dev64):.3e}"),
            "noise": "reference fillInComplexNoise stream (oracle restatement pinned to RandomGen), seed 231171"}


def oracle_tables(sc):
    """The per-k operator tables from the oracle's own restatement (no product code on the CPU arm)."""
    from oracle import oracle as O
    return O.k_tables(sc.nxp, sc.wavelets, sc.A, sc.nz, sc.nzp, sc.dt_ms, sc.low_cut, sc.high_cut,
                      sc.min_rel_thick, prec="f")


CPU_SAMPLE = ("one complete inversion of the workload: {n} data + 3 prior-mean + 7 prior/error forward 256^3 "
              "transforms, the bin loop over all bins, 3 inverse transforms (no extrapolation)")


def run_reference(args, world, rank):
    if rank != 0:
        return
    from crava_gb300 import synthetic as S
    sc = S.config1()
    tables = oracle_tables(sc)
    bins = sc.nbins
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_inversion(sc, tables, "f", threads)
    times = []
    info = None
    for _ in range(args.steps):
        info = cpu_inversion(sc, tables, "f", threads)[0]
        times.append(info["total_s"])
    ms = 1e3 * statistics.mean(times)
    value = bins / (ms * 1e-3) / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mbins/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "nxp": sc.nxp, "nyp": sc.nyp, "nzp": sc.nzp, "ntheta": sc.ntheta,
                   "bins": bins, "form": "reference dataflow on the host (C oracle port, OpenMP)"},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mbins/s", "cores": threads, "kind": "port",
                         "sample": CPU_SAMPLE.format(n=sc.ntheta),
                         "last_step_phases_s": {k: round(v, 4) for k, v in info.items()}},
        "e2e": {"value": round(value, 4), "unit": "Mbins/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
COND_BUCKETS = 16


def conditioning_case(args, stream, flush, rank, sn, wnc):
    """8 stacks 0-40 deg (near-collinear Aki-Richards rows), 25 Hz Ricker without notches, band 1-100 Hz,
    256x256x128 padded, at signal-to-noise ratio ``sn`` and white-noise component ``wnc``.  Times the fused
    FP32 and mixed forms and reports the FP64 fix-up's share, the condition histograms and both forms'
    errors vs the FP64 form."""
    import numpy as np
    import torch
    from crava_gb300 import _native
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    sc = S.make_scenario(205, 205, 102, list(np.linspace(0.0, 40.0, 8)), 25.0, nxp=256, nyp=256, nzp=128,
                         sn=sn, wnc=wnc, low_cut=1.0, high_cut=100.0, seed=20261209 + rank)
    inv = Inversion(sc, forms=("fp32", "mixed", "fp64"))
    ms = {}
    for form in ("fp32", "mixed"):
        for _ in range(max(args.warmup, 1)):
            inv.restore(form)
            inv.run(form)
        ev = []
        for _ in range(args.steps):
            inv.restore(form)
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            inv.run(form)
            e1.record(stream)
            ev.append((e0, e1))
        torch.cuda.synchronize()
        ms[form] = statistics.mean(a.elapsed_time(b) for a, b in ev)
    inv.restore("fp64")
    inv.run("fp64")
    torch.cuda.synchronize()
    pm64, res64, cov64 = inv.results("fp64")
    prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
    out = {"workload": f"256x256x128 padded, 8 stacks 0-40 deg, 25 Hz Ricker, S/N {sn:g}, wnc {wnc:g}, band 1-100 Hz",
           "bins": sc.nbins, "ms": {k: round(v, 4) for k, v in ms.items()}}
    for form in ("fp32", "mixed"):
        inv.restore(form)
        inv.ws.reset_stats()
        inv.run(form)
        torch.cuda.synchronize()
        pm, res, cov = inv.results(form)
        st = inv.ws.stats()
        out[form] = {"mean_rel_err": float(f"{rel(pm, pm64):.3e}"),
                     "update_rel_err": float(f"{rel(pm - prior, pm64 - prior):.3e}"),
                     "resid_rel_err": float(f"{rel(res, res64):.3e}"), "cov_rel_err": float(f"{rel(cov, cov64):.3e}"),
                     "fp64_bins": st["flagged"] if form == "mixed" else 0, "chol_fail": st["failed"]}
        if form == "mixed":
            hc, hi = inv.ws.condition_histogram(COND_BUCKETS)
            out["condition_histogram"] = {"chol_form_fp64": hc, "info_form_fp32": hi}
    inv.restore("mixed")
    torch.cuda.synchronize()
    _native.trace_enable(True)
    inv.run("mixed")
    tr = _native.trace_collect()
    _native.trace_enable(False)
    total = sum(v[1] for v in tr.values())
    fix = sum(v[1] for k, v in tr.items() if "fixup" in k)
    out["fixup_ms"] = round(fix, 4)
    out["fixup_share_of_kernel_time"] = round(fix / total, 4) if total > 0 else None
    del inv
    return out


def cpu_simulation_sample(sc, cov_spec, post_mean, nreal, threads):
    """Seconds per realisation of the oracle's posterior simulation (src/crava.cpp:1551-1734): seeded noise
    (fillInComplexNoise), the per-bin factor applied in the reference's lib_matr order, three inverse
    transforms and the posterior-mean add, over ``nreal`` realisations."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    for r in range(nreal):
        seeds = O.fill_complex_noise(sc.nxp, sc.nyp, sc.nzp, 1000 + r, ncubes=3)
        sim = O.simulate_bins(cov_spec, seeds, "f", threads)
        for p in range(3):
            f = O.fft3d_c2r(sim[p], sc.nxp, O.PARAMETER, "f", threads)
            f[:, :, :sc.nxp] += post_mean[p]
    return (time.perf_counter() - t0) / nreal


def cpu_timelapse_vintage(tl, state, errc, threads):
    """Seconds for one vintage of the oracle's 4D chain (State4D::merge, the data transforms, the 4D
    branch of the bin loop, State4D::split, the posterior-mean inverse transforms), reference order, FP32."""
    from oracle import oracle as O
    from crava_gb300.pipeline import MERGE_TO_BIN
    mu_s, mu_d, ss, sd, dd = state
    tab = O.k_tables(tl.nxp, tl.wavelets, tl.A, tl.nz, tl.nzp, tl.dt_ms, tl.low_cut, tl.high_cut,
                     tl.min_rel_thick, prec="f")
    tab = dict(tab, nxp=tl.nxp)
    v = tl.vintages[0]
    t0 = time.perf_counter()
    mu_cur, cov_cur = O.state4d_merge(mu_s, mu_d, ss, sd, dd, "f", threads)
    data = [O.fft3d_r2c(d, tl.nxp, O.DATA, "f", threads) for d in v["data"]]
    _, mu_post, cov_bin, _ = O.invert_bins(data, mu_cur, [cov_cur[t] for t in MERGE_TO_BIN], errc, tab,
                                           v["err_theta_cov"], tl.sigma_current(), tl.wnc, is4d=True, prec="f",
                                           nthreads=threads)
    cov_post = [None] * 6
    for k, t in enumerate(MERGE_TO_BIN):
        cov_post[t] = cov_bin[k]
    O.state4d_split(mu_s, mu_d, ss, sd, dd, mu_post, cov_post, "f", threads)
    for m in mu_post:
        O.fft3d_c2r(m, tl.nxp, O.PARAMETER, "f", threads)
    return time.perf_counter() - t0


def other_workloads(args, stream, flush, rank, peak, cpu_ok, sc1=None):
    """The other workloads the metric's configuration list names, each timed with CUDA events after
    warm-up, with the dominant kernel's roofline fraction and (rank 0, one GPU) the CPU oracle port timed
    on the host cores beside it:
      * the small CPU-sized inversion (80x80x160, 3 stacks), L2 flushed between steps;
      * 64 uneven cubes in one graph-replayed batch;
      * posterior simulation, 200^3, 128 realisations;
      * 4D time-lapse, 256x256x192, two vintages x 4 stacks (three-pass plain form and one-pass fused form);
      * the headline model with nonzero correlation gradients (non-separable prior: plain form against the
        fused form reading the per-bin prior table)."""
    import numpy as np
    import torch
    from crava_gb300 import api, microbench as MB
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    threads = os.cpu_count() or 1
    steps = max(1, min(args.steps, 5))
    out = {}

    # small inversion (the reference's own CPU-sized case)
    sc0 = S.config0(seed=20261203 + rank)
    inv0 = Inversion(sc0, forms=("plain", "mixed"))
    small = {"workload": "80x80x160 padded (64x64x128 cells), 3 stacks 10-30 deg, 30 Hz Ricker, S/N 4",
             "bins": sc0.nbins, "ms": {}, "ms_stat": "median"}
    for form in ("plain", "mixed"):
        for _ in range(max(args.warmup, 1)):
            inv0.restore(form)
            inv0.run(form)

        def before(form=form):
            inv0.restore(form)
            flush.fill_(1.0)
        small["ms"][form] = round(statistics.median(MB._events_ms(lambda: inv0.run(form), steps, before)), 4)
    small["ms_graph"] = {}
    for form in ("plain", "mixed"):
        g = inv0.capture(form)

        def before(form=form):
            inv0.restore(form)
            flush.fill_(1.0)
        small["ms_graph"][form] = round(statistics.median(MB._events_ms(lambda: g.replay(), steps, before)), 4)
        del g
    small["speedup_mixed_vs_plain_graph"] = round(small["ms_graph"]["plain"] / small["ms_graph"]["mixed"], 3)
    small["Mbins_per_s_mixed"] = round(sc0.nbins / (small["ms"]["mixed"] * 1e-3) / 1e6, 1)
    small["Mbins_per_s_mixed_graph"] = round(sc0.nbins / (small["ms_graph"]["mixed"] * 1e-3) / 1e6, 1)
    inv0.restore("mixed")
    tr = MB._traced(lambda: inv0.run("mixed"))
    small["roofline"] = MB.roofline_of(tr, peak)
    if cpu_ok:
        t = cpu_inversion(sc0, oracle_tables(sc0), "f", threads)[0]
        small["cpu_baseline"] = {"value": round(sc0.nbins / t["total_s"] / 1e6, 3), "unit": "Mbins/s",
                                 "cores": threads, "kind": "port", "sample": "one complete inversion"}
        t1 = cpu_inversion(sc0, oracle_tables(sc0), "f", 1)[0]
        small["cpu_baseline_1core"] = {"value": round(sc0.nbins / t1["total_s"] / 1e6, 3), "unit": "Mbins/s",
                                       "cores": 1, "kind": "port", "sample": "one complete inversion"}
    del inv0
    out["small_80x80x160_3stacks"] = small

    # the headline model with correlation gradients
    if sc1 is not None:
        import dataclasses
        gsc = dataclasses.replace(sc1, corr_grad=(0.37, -0.21))
        invg = Inversion(gsc, forms=("plain", "mixed"))
        grad = {"workload": "the 256^3 5-stack model with correlation gradients (corrGradI, corrGradJ) = "
                            "(0.37, -0.21): a prior that is not separable",
                "bins": gsc.nbins, "ms": {}, "ms_stat": "median"}
        outs = {}
        for form in ("plain", "mixed"):
            for _ in range(max(args.warmup, 1)):
                invg.restore(form)
                invg.run(form)

            def before(form=form):
                invg.restore(form)
                flush.fill_(1.0)
            grad["ms"][form] = round(statistics.median(MB._events_ms(lambda: invg.run(form), steps, before)), 4)
            invg.restore(form)
            invg.run(form)
            torch.cuda.synchronize()
            outs[form] = invg.results(form)
        grad["Mbins_per_s_mixed"] = round(gsc.nbins / (grad["ms"]["mixed"] * 1e-3) / 1e6, 1)
        grad["speedup_mixed_vs_plain"] = round(grad["ms"]["plain"] / grad["ms"]["mixed"], 3)
        prior = np.stack([m[:, :, :gsc.nxp] for m in gsc.mean]).astype(np.float64)
        pm_p, _, cov_p = outs["plain"]
        pm_m, _, cov_m = outs["mixed"]
        grad["mixed_vs_plain"] = {"update_rel_diff": float(f"{rel(pm_m - prior, pm_p - prior):.3e}"),
                                  "cov_rel_diff": float(f"{rel(cov_m, cov_p):.3e}")}
        invg.restore("mixed")
        grad["roofline"] = MB.roofline_of(MB._traced(lambda: invg.run("mixed")), peak)
        del invg, outs
        out["gradients_256_5stacks"] = grad

    # batch of uneven cubes
    t0 = time.perf_counter()
    scs = S.config2(64)
    t_gen = time.perf_counter() - t0
    batch = MB.measure_batch(scs, "mixed", reps=steps, warmup=args.warmup, peak=peak, flush=flush)
    batch["workload"] = ("64 cubes, nx, ny ~ U{32..192}, nz ~ U{64..160}, padded 25 % to 2/3/5/7-smooth sizes, "
                         "2-8 stacks, Ricker 15-45 Hz, S/N 2-6, prior stds x U(0.5, 1.5)")
    batch["generation_s"] = round(t_gen, 1)
    if cpu_ok:
        done, secs, ncubes = 0, 0.0, 0
        for sc in scs:
            secs += cpu_inversion(sc, oracle_tables(sc), "f", threads)[0]["total_s"]
            done += sc.nbins
            ncubes += 1
            if secs > 8.0:
                break
        batch["cpu_baseline"] = {"value": round(done / secs / 1e6, 3), "unit": "Mbins/s", "cores": threads,
                                 "kind": "port", "sample": f"complete inversions of the first {ncubes} cubes"}
    # the same batch with per-cube realisation counts (0-4), drawn after each cube's inversion in the graph
    import numpy as np
    nreal = np.random.default_rng(20261210).integers(0, 5, len(scs))
    bsim = MB.measure_batch(scs, "mixed", reps=steps, warmup=args.warmup, peak=peak, flush=flush, nreal=nreal)
    bsim["workload"] = "the batch above, each cube also drawing U{0..4} posterior realisations inside the graph"
    batch["with_realisations"] = {k: bsim[k] for k in ("ms", "ms_stat", "realisations", "launches")}
    batch["with_realisations"]["realisations_per_s"] = round(bsim["realisations"] / (bsim["ms"] * 1e-3), 1)
    del scs
    out["batch_64_uneven_cubes"] = batch

    # posterior simulation
    sim, sc3 = MB.measure_simulate(nreal=128, reps=steps, warmup=1, peak=peak)
    if cpu_ok:
        inv3 = Inversion(sc3, forms=("mixed",))
        inv3.restore("mixed")
        inv3.run("mixed")
        torch.cuda.synchronize()
        pm, _, cov = inv3.results("mixed")
        spr = cpu_simulation_sample(sc3, list(cov), list(pm), 2, threads)
        sim["cpu_baseline"] = {"value": round(1.0 / spr, 3), "unit": "realisations/s", "cores": threads,
                               "kind": "port", "sample": "2 realisations (noise, factor, 3 inverse transforms, mean add)"}
        try:
            sim["fields_vs_cpu_fp64"] = simulated_fields_vs_fp64(sc3, inv3, threads)
        except Exception as e:  # an accuracy side figure must not cost the bench line
            sim["fields_vs_cpu_fp64"] = {"error": repr(e)[:300]}
        del inv3
    out["simulation_200cube_128_realisations"] = sim

    # 4D time-lapse
    tl = S.config4()
    from crava_gb300.pipeline import TimeLapse
    run = TimeLapse(tl)
    four = {"workload": "256x256x192 padded, 6-parameter state, 2 vintages x 4 stacks, S/N 4"}
    for form in ("plain", "mixed"):
        four[form], run = MB.measure_timelapse(tl, form, reps=steps, warmup=1, peak=peak, run=run)
    four["speedup_mixed_vs_plain"] = round(four["plain"]["ms"] / four["mixed"]["ms"], 3)
    # the step between vintages when the state evolves (State4D::evolve): not part of the workload above
    four["evolve_step"] = MB.measure_evolve(run, reps=max(steps, 3), peak=peak)
    if cpu_ok:
        run.restore()
        torch.cuda.synchronize()
        state = run.state()
        errc = api.as_spectrum(run.errcorr).cpu().numpy()
        tv = cpu_timelapse_vintage(tl, state, errc, threads)
        four["cpu_baseline"] = {"value": round(tl.nbins / (tv * len(tl.vintages)) / 1e6, 3), "unit": "Mbins/s",
                                "cores": threads, "kind": "port",
                                "sample": "one vintage of the 4D chain (merge, 4 data transforms, 4D bin loop, "
                                          "split, 3 inverse transforms), scaled to two vintages"}
    del run
    out["timelapse_4d_256x256x192"] = four
    return out


def run_ours(args, world, rank, local):
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import crava_gb300
    from crava_gb300 import _native, api
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion

    crava_gb300.lib()
    t0 = time.perf_counter()
    sc = S.config1(seed=20261204 + rank)
    t_gen = time.perf_counter() - t0
    inv = Inversion(sc, forms=("plain", "fp32", "mixed", "fp64"))
    bins = sc.nbins
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def timed(form, k):
        evs = []
        for _ in range(k):
            inv.restore(form)          # real-domain inputs back in place (not timed)
            flush.fill_(1.0)           # evict L2 between steps
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            inv.run(form)
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    results = {}
    forms = ["plain", "fp32", "mixed"]
    clocks = ClockSampler(local)
    for form in forms:
        timed(form, args.warmup)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    for form in forms:
        barrier(world)
        torch.cuda.synchronize()
        ms = timed(form, args.steps)
        barrier(world)
        torch.cuda.synchronize()
        results[form] = statistics.mean(ms)

    # the same steps captured once as CUDA graphs and replayed (one host call per step)
    def timed_graph(g, form, k):
        evs = []
        for _ in range(k):
            inv.restore(form)
            flush.fill_(1.0)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            g.replay()
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    results_graph = {}
    for form in forms:
        g = inv.capture(form)
        timed_graph(g, form, args.warmup)
        barrier(world)
        torch.cuda.synchronize()
        results_graph[form] = statistics.mean(timed_graph(g, form, args.steps))
        del g

    # one-shot inversion of a model seen for the first time (per-model set-up inside the step)
    def timed_cold(k):
        evs = []
        for _ in range(k):
            inv.restore("mixed")
            flush.fill_(1.0)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            inv.run_cold("mixed")
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    timed_cold(args.warmup)
    barrier(world)
    torch.cuda.synchronize()
    ms_cold = statistics.mean(timed_cold(args.steps))
    barrier(world)
    inv.restore("mixed")
    torch.cuda.synchronize()
    _native.trace_enable(True)
    inv.run_cold("mixed")
    tr_cold = _native.trace_collect()
    _native.trace_enable(False)

    # accuracy against the FP64 run on the same inputs
    inv.restore("fp64")
    inv.run("fp64")
    torch.cuda.synchronize()
    pm64, res64, cov64 = inv.results("fp64")
    prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
    acc = {}
    for form in forms:
        inv.restore(form)
        inv.ws.reset_stats()
        inv.run(form)
        torch.cuda.synchronize()
        pm, res, cov = inv.results(form)
        st = inv.ws.stats()
        acc[form] = {"mean_rel_err": rel(pm, pm64), "update_rel_err": rel(pm - prior, pm64 - prior),
                     "resid_rel_err": rel(res, res64), "cov_rel_err": rel(cov, cov64),
                     "fp64_bins": st["flagged"] if form == "mixed" else 0, "chol_fail": st["failed"]}
        if form == "mixed":
            mixed_out = (pm, res, cov)
            hist_chol, hist_info = inv.ws.condition_histogram(COND_BUCKETS)
        del pm, res, cov
    inv.restore("mixed")
    inv.run_cold("mixed")
    torch.cuda.synchronize()
    pmc, resc, covc = inv.results("mixed")
    acc["mixed_cold"] = {"mean_rel_err": rel(pmc, pm64), "update_rel_err": rel(pmc - prior, pm64 - prior),
                         "resid_rel_err": rel(resc, res64), "cov_rel_err": rel(covc, cov64),
                         "identical_to_mixed": bool((pmc == mixed_out[0]).all() and (resc == mixed_out[1]).all()
                                                    and (covc == mixed_out[2]).all())}
    del pmc, resc, covc, pm64, res64, cov64

    # per-kernel launch times and algorithmic bytes, one traced mixed step
    inv.restore("mixed")
    torch.cuda.synchronize()
    _native.trace_enable(True)
    inv.run("mixed")
    tr = _native.trace_collect()
    _native.trace_enable(False)
    launches_per_step = sum(v[0] for v in tr.values())
    dom = max(tr.items(), key=lambda kv: kv[1][1])
    dname, (dl, dms, dbytes) = dom
    peak, peak_kind = load_peaks()
    achieved = (dbytes / dl) / (dms / dl * 1e-3) / 1e9 if dms > 0 else 0.0
    tinfo = load_traffic().get(dname)
    # DRAM bytes per launch: the ncu read+write / algorithmic ratio of a smaller capture times this launch's
    # algorithmic bytes (single-pass kernels: traffic scales with the cube size)
    traffic = None
    if isinstance(tinfo, dict) and tinfo.get("ratio"):
        traffic = round(float(tinfo["ratio"]) * dbytes / dl)

    # end to end through the C-ABI host entry points (the calls the reference's
    # Crava::computePostMeanResidAndFFTCov shim makes): pinned host cubes in, residual, covariance and
    # posterior-mean cubes out, every host<->device copy of every step inside the timed region.
    #  * e2e: a sequence of K inversions through cg_inversion_submit_host / cg_inversion_wait on two
    #    contexts used in turn, so one step's output copies overlap the next step's input copies and
    #    compute (inputs read-only, outputs to separate buffers);
    #  * e2e_sync: one synchronous cg_inversion_run_host call per step (in place, as the reference loop).
    pristine = [torch.from_numpy(np.ascontiguousarray(x)).pin_memory() for x in list(sc.data) + list(sc.mean)]
    h2d = sum(x.numel() for x in pristine) * 4
    d2h = (len(pristine) + 6) * pristine[0].numel() * 4
    ctxs = [api.HostInversion(sc) for _ in range(2)]
    outs = [[torch.empty_like(pristine[0]).pin_memory() for _ in range(len(pristine) + 6)] for _ in range(2)]

    def submit(i):
        c, o = ctxs[i % 2], outs[i % 2]
        c.submit(pristine[:sc.ntheta], pristine[sc.ntheta:], o[:sc.ntheta], o[sc.ntheta:sc.ntheta + 3],
                 o[sc.ntheta + 3:], "mixed")

    def pipelined(k):
        t0 = time.perf_counter()
        for i in range(k):
            if i >= 2:
                ctxs[i % 2].wait()
            submit(i)
        for c in ctxs:
            c.wait()
        return (time.perf_counter() - t0) * 1e3 / k

    # warm-up: a whole sequence (the first copies into and out of freshly pinned buffers run slower: 8.9 against
    # 5.65 ms per step measured for a first K-step sequence after three warm-up steps)
    pipelined(max(args.warmup, args.steps, 2))
    barrier(world)
    # three sequences of K pipelined steps, the median of their per-step times: a sequence that meets a host
    # hiccup (the copies depend on the host thread issuing them in time) does not decide the figure
    e2e_seq = [pipelined(args.steps) for _ in range(3)]
    e2e_ms = statistics.median(e2e_seq)

    work = [torch.empty_like(x).pin_memory() for x in pristine]
    h_cov = outs[0][len(pristine):]

    def sync_step():
        for w, p0 in zip(work, pristine):
            w.copy_(p0)              # the call overwrites its inputs: restore them, outside the timed region
        t0 = time.perf_counter()
        ctxs[0].run(work[:sc.ntheta], work[sc.ntheta:], h_cov, "mixed")
        return (time.perf_counter() - t0) * 1e3

    for _ in range(args.warmup):
        sync_step()
    barrier(world)
    e2e_sync_ms = sum(sync_step() for _ in range(args.steps)) / args.steps
    for c in ctxs:
        c.close()
    # the three-stack form of the target: a 256^3 cube with THREE stacks (0/20/40 deg), mixed vs plain,
    # timed the same way (restore + L2 flush outside the events), error vs the FP64 GPU form
    sc3 = S.make_scenario(205, 205, 205, [0.0, 20.0, 40.0], 25.0, nxp=256, nyp=256, nzp=256, sn=3.0,
                          notches_hz=(2.0, 80.0), low_cut=1.0, high_cut=100.0, seed=20261208 + rank)
    inv3 = Inversion(sc3, forms=("plain", "mixed", "fp64"))
    three = {}
    for form in ("plain", "mixed"):
        for _ in range(max(args.warmup, 1)):
            inv3.restore(form)
            inv3.run(form)
        ev = []
        for _ in range(args.steps):
            inv3.restore(form)
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            inv3.run(form)
            e1.record(stream)
            ev.append((e0, e1))
        torch.cuda.synchronize()
        three[form] = statistics.mean(a.elapsed_time(b) for a, b in ev)
    inv3.restore("fp64")
    inv3.run("fp64")
    inv3.restore("mixed")
    inv3.run("mixed")
    torch.cuda.synchronize()
    pm3, _, _ = inv3.results("mixed")
    pm3_64, _, _ = inv3.results("fp64")
    from crava_gb300 import microbench as MB
    inv3.restore("mixed")
    tr3 = MB._traced(lambda: inv3.run("mixed"))
    three_stack = {"ms": {k: round(v, 4) for k, v in three.items()},
                   "speedup_mixed_vs_plain": round(three["plain"] / three["mixed"], 3),
                   "mean_rel_err_vs_fp64": float(f"{rel(pm3, pm3_64):.3e}"),
                   "Mbins_per_s_mixed": round(sc3.nbins / (three["mixed"] * 1e-3) / 1e6, 1),
                   "roofline": MB.roofline_of(tr3, peak),
                   "kernels": MB.kernel_table(tr3)}
    del inv3, pm3, pm3_64
    clk = clocks.stop()  # sampled from the first timed form step to the last end-to-end step

    # the step as the library runs it repeatedly: captured once as a CUDA graph, replayed per step (the same
    # launches on the same buffers, one host call); the eager figures (one host call per launch) beside it
    ms_mixed = max_over_ranks(results_graph["mixed"], world)
    ms_plain = max_over_ranks(results_graph["plain"], world)
    ms_fp32 = max_over_ranks(results_graph["fp32"], world)
    ms_mixed_eager = max_over_ranks(results["mixed"], world)
    ms_plain_eager = max_over_ranks(results["plain"], world)
    ms_fp32_eager = max_over_ranks(results["fp32"], world)
    e2e_ms = max_over_ranks(e2e_ms, world)
    e2e_sync_ms = max_over_ranks(e2e_sync_ms, world)
    from crava_gb300 import replicas
    total_bins = bins * world
    value = replicas.whole_job_rate(bins, ms_mixed, world)

    # conditioning: the reference accepts 1 < S/N <= 10 (src/modelavodynamic.cpp:1255-1260); at its maximum
    # no bin crosses the guard, so a second case goes far beyond that range to exercise the FP64 fix-up
    cond_case = {"sn_10_reference_max": conditioning_case(args, stream, flush, rank, 10.0, 0.1),
                 "sn_1e5_outside_reference_range": conditioning_case(args, stream, flush, rank, 1.0e5, 1.0e-4)}

    others = None
    if not args.no_other_workloads:
        others = other_workloads(args, stream, flush, rank, peak,
                                 rank == 0 and world == 1 and not args.no_cpu_baseline, sc1=sc)

    cpu = None
    vs_cpu64 = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        # the posterior of the mixed GPU form against the CPU FP64 oracle on the same inputs and tables
        t64, post64, r64, c64, nf64 = cpu_inversion(sc, inv.tables, "d", threads)
        pm, res, cov = mixed_out
        vs_cpu64 = {"mean_rel_err": float(f"{rel(pm, post64):.3e}"),
                    "update_rel_err": float(f"{rel(pm - prior, post64 - prior):.3e}"),
                    "resid_rel_err": float(f"{rel(res, r64):.3e}"), "cov_rel_err": float(f"{rel(cov, c64):.3e}"),
                    "oracle_chol_fail": int(nf64), "oracle_s": round(t64["total_s"], 2),
                    "oracle": "C oracle in FP64, reference dataflow, the GPU's operator tables"}
        del post64, r64, c64, pm, res, cov
        tcpu = cpu_inversion(sc, oracle_tables(sc), "f", threads)[0]
        cpu = {"value": round(bins / tcpu["total_s"] / 1e6, 4), "unit": "Mbins/s", "cores": threads, "kind": "port",
               "sample": CPU_SAMPLE.format(n=sc.ntheta), "phases_s": {k: round(v, 4) for k, v in tcpu.items()}}
    del mixed_out

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mbins/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_mixed, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FP64-guarded bins)", "data": "synthetic",
            "config": {"workload": WORKLOAD, "nxp": sc.nxp, "nyp": sc.nyp, "nzp": sc.nzp, "ntheta": sc.ntheta,
                       "bins": bins, "inband_bins": int(inv.tables["band"].sum()) * sc.cnxp * sc.nyp,
                       "form": "mixed (fused, FP64-guarded)", "parallelism": f"replicas x{world}",
                       "l2": "256 MB flush + ~1.3 GB input restore between timed steps; working set 1.4 GB > L2"},
            "forms_ms": {"plain": round(ms_plain, 4), "fp32": round(ms_fp32, 4), "mixed": round(ms_mixed, 4),
                         "how": "CUDA-graph replay of the captured step"},
            "forms_ms_eager": {"plain": round(ms_plain_eager, 4), "fp32": round(ms_fp32_eager, 4),
                               "mixed": round(ms_mixed_eager, 4), "how": "one host call per launch"},
            "speedup_mixed_vs_plain": round(ms_plain / ms_mixed, 3),
            "cold_one_shot": {"ms": round(ms_cold, 4), "Mbins_per_s": round(bins / (ms_cold * 1e-3) / 1e6, 1),
                              "vs_repeated_model": round(ms_cold / ms_mixed_eager, 4),
                              "vs_what": "the eager repeated-model step (both issue one host call per launch)",
                              "kernels": {k: {"launches": v[0], "ms": round(v[1], 4)}
                                          for k, v in sorted(tr_cold.items(), key=lambda kv: -kv[1][1])},
                              "what": "mixed form with the model's per-k set-up inside the step: host operator "
                                      "tables built while the forward transforms run, one upload, the per-k "
                                      "table kernel (cg_workspace_set_model_async) and the prior spectra on a "
                                      "high-priority side stream beside the transforms"},
            "accuracy_vs_cpu_fp64": vs_cpu64,
            "condition_histogram": {"buckets": "decades of the squared Cholesky pivot ratio, last = failed",
                                    "threshold": 1.0e3, "chol_form_fp64": hist_chol, "info_form_fp32": hist_info},
            "conditioning_stress": cond_case,
            "three_stack_256": three_stack,
            "accuracy_vs_fp64": {f: {k: (float(f"{v:.3e}") if isinstance(v, float) else v) for k, v in d.items()}
                                 for f, d in acc.items()},
            "roofline": {"bound": "hbm", "kernel": dname, "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                         "traffic": traffic, "launches_per_step": dl,
                         "algorithmic_bytes_per_launch": dbytes / dl,
                         "pipeline_algorithmic_GBps": round(inv.algorithmic_bytes("mixed") / (ms_mixed * 1e-3) / 1e9, 1)},
            "kernels_per_step": {k: {"launches": v[0], "ms": round(v[1], 4), "GBps": round(v[2] / max(v[1], 1e-9) / 1e6, 1)}
                                 for k, v in sorted(tr.items(), key=lambda kv: -kv[1][1])},
            "e2e": {"value": round(total_bins / (e2e_ms * 1e-3) / 1e6, 3), "unit": "Mbins/s",
                    "ms_per_step": round(e2e_ms, 3), "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "api": "cg_inversion_submit_host/cg_inversion_wait, 2 contexts in turn",
                    "ms_per_step_sequences": [round(x, 3) for x in e2e_seq], "ms_stat": "median of 3 sequences",
                    "sync_call": {"value": round(total_bins / (e2e_sync_ms * 1e-3) / 1e6, 3),
                                  "ms_per_step": round(e2e_sync_ms, 3), "api": "cg_inversion_run_host"}},
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clk,
            "cpu_baseline": cpu,
            "other_workloads": others,
            "setup_s": {"synthetic_generation": round(t_gen, 1)},
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="skip the small, batch, simulation and 4D workloads")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
