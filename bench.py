"""Benchmark: 256^3 FFT-domain AVO inversion on one GB300 (per GPU replica).

Workload: a 256x256x256 padded cube, 5 angle stacks at 0/10/20/30/40 deg, a
25 Hz Ricker wavelet notched at 2 and 80 Hz, S/N 3, inversion band 1-100 Hz
(seeded synthetic data, generated on the host).  One step = one complete
inversion (forward transforms of the 5 data and 3 prior-mean cubes, the
prior/error spectra, the per-bin posterior, inverse transforms of the 3
posterior means), inputs resident in HBM.

Forms timed: "plain" (the reference dataflow on the GPU, all FP32), "fp32"
(fused, all FP32), "mixed" (fused, FP32 bulk + FP64-guarded bins; the
headline).  "fp64" runs once as the accuracy reference.

Metric: Mbins/s = (cnxp*nyp*nzp bins) / (ms per inversion).  With --gpus N
under torchrun each rank runs an independent replica (the path does not shard
a cube; cubes are independent), value = total bins / max time.

--impl reference times the reference algorithm on the host cores (the C
oracle port: its FFTs and its lib_matr-order bin loop, OpenMP over k like the
reference) on a bounded sample scaled to a full inversion.
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
# CPU reference (oracle port) timing
# ---------------------------------------------------------------------------
def cpu_reference_sample(sc, tables, kplanes=8, threads=None):
    """Time the reference algorithm on the host on a bounded sample.

    Sample: one forward and one inverse 3D transform of a full cube, plus the
    bin loop over `kplanes` in-band k-planes.  Scaled to one inversion of the
    reference dataflow: (n + 3 + 6 + 1) forward transforms, 3 inverse
    transforms, all bins.
    """
    import numpy as np
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    nxp, nyp, nzp, n = sc.nxp, sc.nyp, sc.nzp, sc.ntheta
    t0 = time.perf_counter()
    spec = O.fft3d_r2c(sc.data[0], nxp, O.DATA, "f", threads)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.fft3d_c2r(spec, nxp, O.PARAMETER, "f", threads)
    t_inv = time.perf_counter() - t0
    # bin loop on a slab of in-band k-planes (inputs: random spectra of the right shape)
    ks = [k for k in range(nzp) if tables["band"][k]][:kplanes]
    rng = np.random.default_rng(1)
    cnxp = nxp // 2 + 1
    shp = (len(ks), nyp, cnxp)

    def rc():
        return (rng.standard_normal(shp) + 1j * rng.standard_normal(shp)).astype(np.complex64)
    data = [rc() for _ in range(n)]
    mean = [rc() for _ in range(3)]
    # prior spectra of the planes from the separable model (so every Cholesky does its full work)
    cxy = np.fft.rfft2(sc.corr_xy.astype(np.float64))            # (nyp, cnxp)
    ctk = np.fft.fft(sc.circ_corr_t.astype(np.float64))[ks]      # (len(ks),)
    c = (ctk[:, None, None] * cxy[None, :, :]).real.astype(np.float32)
    s0 = sc.sigma0.astype(np.float32)
    cov = [(c * s0[p, q]).astype(np.complex64) for (p, q) in [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]]
    ec = np.broadcast_to(cxy.real.astype(np.float32), shp).astype(np.complex64)
    sub = {"K": tables["K"][ks], "em1": tables["em1"][ks], "em2": tables["em2"][ks], "em3": tables["em3"][ks],
           "band": np.ones(len(ks), np.uint8), "nxp": nxp}
    t0 = time.perf_counter()
    O.invert_bins(data, mean, cov, ec, sub, sc.err_theta_cov, sc.sigma0, sc.wnc, prec="f", nthreads=threads)
    t_bins = time.perf_counter() - t0
    inband = int(np.asarray(tables["band"]).sum())
    t_full = (n + 3 + 6 + 1) * t_fwd + 3 * t_inv + t_bins * inband / max(1, len(ks))
    sample = (f"1 forward + 1 inverse 256^3 transform and the bin loop over {len(ks)} of {inband} in-band "
              f"k-planes, scaled to {n + 10} forward + 3 inverse transforms and all bins")
    return t_full, threads, sample, {"t_fwd_s": t_fwd, "t_inv_s": t_inv, "t_bins_sample_s": t_bins}


def run_reference(args, world, rank):
    if rank != 0:
        return
    import numpy as np
    from crava_gb300 import synthetic as S
    from crava_gb300 import api
    sc = S.config1()
    tables = api.operator_tables(sc.wavelets, sc.A, sc.nz, sc.nzp, sc.dt_ms, sc.low_cut, sc.high_cut)
    bins = sc.nbins
    for _ in range(args.warmup):
        cpu_reference_sample(sc, tables, kplanes=2)
    times = []
    info = None
    for _ in range(args.steps):
        t, cores, sample, info = cpu_reference_sample(sc, tables)
        times.append(t)
    ms = 1e3 * statistics.mean(times)
    value = bins / (ms * 1e-3) / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mbins/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "nxp": sc.nxp, "nyp": sc.nyp, "nzp": sc.nzp, "ntheta": sc.ntheta,
                   "bins": bins, "form": "reference dataflow on the host (C oracle port, OpenMP)"},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mbins/s", "cores": cores, "kind": "port",
                         "sample": sample, **{k: round(v, 4) for k, v in info.items()}},
        "e2e": {"value": round(value, 4), "unit": "Mbins/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
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
        del pm, res, cov

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

    pipelined(max(args.warmup, 2))
    barrier(world)
    e2e_ms = pipelined(args.steps)

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
    three_stack = {"ms": {k: round(v, 4) for k, v in three.items()},
                   "speedup_mixed_vs_plain": round(three["plain"] / three["mixed"], 3),
                   "mean_rel_err_vs_fp64": float(f"{rel(pm3, pm3_64):.3e}"),
                   "Mbins_per_s_mixed": round(sc3.nbins / (three["mixed"] * 1e-3) / 1e6, 1)}
    del inv3, pm3, pm3_64
    clk = clocks.stop()  # sampled from the first timed form step to the last end-to-end step

    ms_mixed = max_over_ranks(results["mixed"], world)
    ms_plain = max_over_ranks(results["plain"], world)
    ms_fp32 = max_over_ranks(results["fp32"], world)
    e2e_ms = max_over_ranks(e2e_ms, world)
    e2e_sync_ms = max_over_ranks(e2e_sync_ms, world)
    from crava_gb300 import replicas
    total_bins = bins * world
    value = replicas.whole_job_rate(bins, ms_mixed, world)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        t_full, cores, sample, info = cpu_reference_sample(sc, inv.tables)
        cpu = {"value": round(bins / t_full / 1e6, 4), "unit": "Mbins/s", "cores": cores, "kind": "port",
               "sample": sample}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mbins/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_mixed, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FP64-guarded bins)", "data": "synthetic",
            "config": {"workload": WORKLOAD, "nxp": sc.nxp, "nyp": sc.nyp, "nzp": sc.nzp, "ntheta": sc.ntheta,
                       "bins": bins, "inband_bins": int(inv.tables["band"].sum()) * sc.cnxp * sc.nyp,
                       "form": "mixed (fused, FP64-guarded)", "parallelism": f"replicas x{world}",
                       "l2": "256 MB flush + ~1.3 GB input restore between timed steps; working set 1.4 GB > L2"},
            "forms_ms": {"plain": round(ms_plain, 4), "fp32": round(ms_fp32, 4), "mixed": round(ms_mixed, 4)},
            "speedup_mixed_vs_plain": round(ms_plain / ms_mixed, 3),
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
                    "sync_call": {"value": round(total_bins / (e2e_sync_ms * 1e-3) / 1e6, 3),
                                  "ms_per_step": round(e2e_sync_ms, 3), "api": "cg_inversion_run_host"}},
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clk,
            "cpu_baseline": cpu,
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
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
