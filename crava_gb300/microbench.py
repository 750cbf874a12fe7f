"""Time (or profile) one stage of the inversion in isolation on the GPU.

    python -m crava_gb300.microbench fft   --nxp 256 --nyp 256 --nzp 64 --batch 5 --reps 3
    python -m crava_gb300.microbench invert --nxp 256 --nyp 256 --nzp 64 --form mixed --reps 3
    python -m crava_gb300.microbench copy  --mb 512 --reps 5
    python -m crava_gb300.microbench simulate --nreal 128 --reps 3
    python -m crava_gb300.microbench timelapse --reps 3
    python -m crava_gb300.microbench ingest --reps 3

Inputs are seeded random cubes (fft) or a scaled config-1 scenario (invert).
Prints one JSON line with per-kernel launch times and algorithmic bandwidth
from the library's launch tracer.  Small sizes keep ncu captures short.
"""
from __future__ import annotations

import argparse
import json
import statistics

import numpy as np
import torch

from . import _native, api


def fft_case(a):
    g = torch.Generator(device="cuda").manual_seed(1)
    _, rnxp = api.dims(a.nxp)
    cubes = [torch.randn((a.nzp, a.nyp, rnxp), device="cuda", generator=g) for _ in range(a.batch)]
    for _ in range(a.reps):
        api.fft_in_place_batch(cubes, a.nxp, api.DATA)
        api.fft_in_place_batch(cubes, a.nxp, api.DATA, inverse=True)


def invert_case(a):
    from . import synthetic as S
    from .pipeline import Inversion
    sc = S.scaled_config1(a.nxp, a.nyp, a.nzp, seed=5)
    inv = Inversion(sc, forms=(a.form,))
    for _ in range(a.reps):
        inv.restore(a.form)
        inv.run(a.form)


def batch_case(a):
    from . import synthetic as S
    if not hasattr(a, "_batch"):
        scs = S.config2(a.ncubes)
        a._batch = api.Batch(scs, nstreams=a.streams)
    a._batch.reset()
    a._batch.run(a.form, use_graph=True)


def copy_case(a):
    """Pinned host <-> device copy rates: one stream, split over streams, both directions at once."""
    n = a.mb * (1 << 20) // 4
    h_in = torch.empty(n, dtype=torch.float32).pin_memory()
    h_out = torch.empty(n, dtype=torch.float32).pin_memory()
    d_in = torch.empty(n, dtype=torch.float32, device="cuda")
    d_out = torch.empty(n, dtype=torch.float32, device="cuda")
    streams = [torch.cuda.Stream() for _ in range(4)]

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best = None
        for _ in range(a.reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for s in streams:
                s.wait_event(e0)
            fn()
            for s in streams:
                torch.cuda.current_stream().wait_stream(s)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        return best

    def split(k, src, dst):
        def fn():
            c = (n + k - 1) // k
            for i in range(k):
                with torch.cuda.stream(streams[i]):
                    dst[i * c:(i + 1) * c].copy_(src[i * c:(i + 1) * c], non_blocking=True)
        return fn

    gb = n * 4 / 1e9
    out = {}
    for k in (1, 2, 4):
        out[f"h2d_{k}streams_GBps"] = gb / (timed(split(k, h_in, d_in)) * 1e-3)
        out[f"d2h_{k}streams_GBps"] = gb / (timed(split(k, d_out, h_out)) * 1e-3)

    def both():
        with torch.cuda.stream(streams[0]):
            d_in.copy_(h_in, non_blocking=True)
        with torch.cuda.stream(streams[1]):
            h_out.copy_(d_out, non_blocking=True)
    out["h2d_plus_d2h_concurrent_GBps_total"] = 2 * gb / (timed(both) * 1e-3)

    # the same traffic moved by kernels that load/store host memory directly (cg_copy)
    L = _native.lib()

    def kcopy(dst, src):
        def fn():
            _native.check(L.cg_copy(dst.data_ptr(), src.data_ptr(), n * 4, torch.cuda.current_stream().cuda_stream),
                          "cg_copy")
        return fn
    out["kernel_h2d_GBps"] = gb / (timed(kcopy(d_in, h_in)) * 1e-3)
    out["kernel_d2h_GBps"] = gb / (timed(kcopy(h_out, d_out)) * 1e-3)
    out["kernel_d2d_GBps_read_plus_write"] = 2 * gb / (timed(kcopy(d_out, d_in)) * 1e-3)

    def kboth():
        with torch.cuda.stream(streams[0]):
            _native.check(L.cg_copy(d_in.data_ptr(), h_in.data_ptr(), n * 4, streams[0].cuda_stream), "cg_copy")
        with torch.cuda.stream(streams[1]):
            _native.check(L.cg_copy(h_out.data_ptr(), d_out.data_ptr(), n * 4, streams[1].cuda_stream), "cg_copy")
    out["kernel_h2d_plus_d2h_GBps_total"] = 2 * gb / (timed(kboth) * 1e-3)
    out["host_access_bits"] = int(L.cg_host_access())
    print(json.dumps({"case": {"what": "copy", "mb": a.mb, "reps": a.reps}, "rates": out}))


def kernel_table(tr):
    """Launch-tracer totals as {kernel: {launches, ms, GBps}}, longest first."""
    return {k: {"launches": v[0], "ms": round(v[1], 4), "GBps": round(v[2] / max(v[1], 1e-12) / 1e6, 1)}
            for k, v in sorted(tr.items(), key=lambda kv: -kv[1][1])}


def roofline_of(tr, peak):
    """The kernel with the largest share of a traced run against the HBM peak (GB/s): algorithmic bytes
    over the launches' CUDA-event time."""
    name, (nl, ms, by) = max(tr.items(), key=lambda kv: kv[1][1])
    ach = by / max(ms * 1e-3, 1e-12) / 1e9
    total = sum(v[1] for v in tr.values())
    return {"bound": "hbm", "kernel": name, "launches": nl, "ms": round(ms, 4), "share": round(ms / total, 3),
            "achieved": round(ach, 1), "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4)}


def _events_ms(fn, reps, before=None):
    """CUDA-event time of fn() on the current stream, ``before()`` (untimed) ahead of each repetition."""
    st = torch.cuda.current_stream()
    ev = []
    for _ in range(reps):
        if before is not None:
            before()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fn()
        e1.record(st)
        ev.append((e0, e1))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def _traced(fn):
    torch.cuda.synchronize()
    _native.trace_enable(True)
    fn()
    torch.cuda.synchronize()
    tr = _native.trace_collect()
    _native.trace_enable(False)
    return tr


def measure_batch(scs, form="mixed", reps=3, warmup=3, streams=3, peak=None, flush=None, nreal=None):
    """The uneven-cube batch (cg_batch_run, graph replay) timed with CUDA events; the batch's own inputs
    are restored (cg_batch_reset) before each repetition, outside the timed region.  Per-kernel shares
    from one eager (not graph-replayed) single-stream run under the launch tracer.  nreal: optional
    posterior realisations per cube (cg_batch_set_simulation), drawn inside the same graph."""
    def with_sims(b):
        if nreal is not None:
            for i, n in enumerate(nreal):
                if n > 0:
                    b.set_simulation(i, int(n), seed=1000 + i)
        return b
    b = with_sims(api.Batch(scs, nstreams=streams))
    bins = b.bins

    def before():
        b.reset()
        if flush is not None:
            flush.fill_(1.0)
    for _ in range(max(warmup, 1)):
        before()
        b.run(form, use_graph=True)
    ms = _events_ms(lambda: b.run(form, use_graph=True), reps, before)
    b.close()
    # per-kernel shares from one eager run on a single stream (kernels of concurrent streams would overlap
    # inside each other's event pairs)
    b = with_sims(api.Batch(scs, nstreams=1))
    b.reset()
    b.run(form, use_graph=False)
    b.reset()
    tr = _traced(lambda: b.run(form, use_graph=False))
    b.close()
    mean = statistics.median(ms)
    out = {"form": form, "cubes": len(scs), "bins": int(bins), "ms": round(mean, 4), "ms_stat": "median",
           "realisations": int(sum(nreal)) if nreal is not None else 0,
           "Mbins_per_s": round(bins / (mean * 1e-3) / 1e6, 1), "ms_per_rep": [round(x, 4) for x in ms],
           "eager_kernels": kernel_table(tr), "launches": int(sum(v[0] for v in tr.values()))}
    if peak:
        out["roofline"] = roofline_of(tr, peak)
    return out


def simulate_case(a):
    print(json.dumps(measure_simulate(nreal=a.nreal, reps=a.reps)[0]))


def measure_simulate(sc=None, nreal=128, reps=3, warmup=1, peak=None):
    """Posterior simulation on the 200^3 three-stack workload: one mixed inversion, then per call the
    per-bin posterior factor and nreal realisations (seeded noise, factor, inverse transform, mean add),
    timed with CUDA events (the fields, 3*nreal cubes, are far larger than L2)."""
    from . import synthetic as S
    from .pipeline import Inversion
    sc = sc or S.config3()
    inv = Inversion(sc, forms=("mixed",))
    inv.restore("mixed")
    inv.run("mixed")
    torch.cuda.synchronize()
    _, rnxp = api.dims(sc.nxp)
    fields = [torch.empty((sc.nzp, sc.nyp, rnxp), device="cuda") for _ in range(3 * nreal)]
    rep = [0]

    def step():
        rep[0] += 1
        c, _ = api.posterior_cholesky(inv.cov, sc.nxp)
        api.simulate_fields(c, fields, sc.nxp, seed=1000 + rep[0], post_mean=inv.mean)
    for _ in range(max(warmup, 1)):
        step()
    ms = _events_ms(step, reps)
    tr = _traced(step)
    _, nfail = api.posterior_cholesky(inv.cov, sc.nxp)
    best = statistics.median(ms)
    bins = sc.nbins
    # algorithmic bytes per realisation: 3 C2R (8 B/bin + 4 B/cell each) + mean read and field write
    # (2 x 3 x 4 B/cell); the factor (36 B/bin) is read once per call
    cells = sc.nxp * sc.nyp * sc.nzp
    alg = nreal * (3 * (8 * bins + 4 * cells) + 24 * cells) + 36 * bins
    out = {"workload": "200^3 padded cube, 3 stacks 10-30 deg, config-0 prior, 30 Hz Ricker, S/N 4",
           "nreal": nreal, "bins": bins, "chol_fail": int(nfail.item()), "ms": round(best, 4), "ms_stat": "median",
           "ms_per_call": [round(x, 4) for x in ms], "realisations_per_s": round(nreal / (best * 1e-3), 1),
           "Mbins_per_s": round(nreal * bins / (best * 1e-3) / 1e6, 1),
           "algorithmic_GBps": round(alg / (best * 1e-3) / 1e9, 1), "kernels": kernel_table(tr),
           "launches": int(sum(v[0] for v in tr.values()))}
    if peak:
        out["roofline"] = roofline_of(tr, peak)
    del fields, inv
    return out, sc


def timelapse_case(a):
    print(json.dumps(measure_timelapse(form=a.form, reps=a.reps)[0]))


def measure_timelapse(tl=None, form="mixed", reps=3, warmup=1, peak=None, run=None):
    """4D time-lapse on the 256x256x192 workload: two vintages x 4 stacks, per vintage the data
    transforms, merge -> 4D bin solve -> split (form "plain": three kernels as the reference's three
    passes; "fp32" / "mixed": one pass per bin, cg_vintage4d) and the posterior-mean inverse transforms;
    CUDA events, the state restored before each repetition outside the timed region."""
    from . import synthetic as S
    from .pipeline import TimeLapse
    tl = tl or S.config4()
    run = run or TimeLapse(tl)
    for _ in range(max(warmup, 1)):
        run.restore()
        run.run(form=form)
    ms = _events_ms(lambda: run.run(form=form), reps, run.restore)
    run.restore()
    tr = _traced(lambda: run.run(form=form))
    fails = [int(x.item()) for x in run.nfail_split]
    st = [w.stats() for w in run.ws]
    best = statistics.median(ms)
    bins = tl.nbins
    out = {"form": form, "bins": bins, "ms": round(best, 4), "ms_stat": "median", "ms_per_run": [round(x, 4) for x in ms],
           "Mbins_per_s": round(bins / (best * 1e-3) / 1e6, 1),
           "joint_algorithmic_GBps": round(run.algorithmic_bytes() / (best * 1e-3) / 1e9, 1),
           "split_fails": fails, "chol_fail": [x["failed"] for x in st], "fp64_bins": [x["flagged"] for x in st],
           "kernels": kernel_table(tr), "launches": int(sum(v[0] for v in tr.values()))}
    if peak:
        out["roofline"] = roofline_of(tr, peak)
    return out, run


def measure_evolve(run, reps=5, peak=None):
    """State4D::evolve (cg_state4d_evolve) on a TimeLapse run's state with an evolution that decays and couples
    the dynamic part and adds a covariance increment (transformed GenExp correlation), timed with CUDA
    events; algorithmic bytes per bin: read and write the 27 state spectra, read the increment's."""
    import numpy as np
    tl = run.tl
    nxp, nyp, nzp = tl.nxp, tl.nyp, tl.nzp
    E = np.block([[np.eye(3), np.zeros((3, 3))],
                  [0.1 * np.eye(3), 0.9 * np.eye(3) + 0.05 * (np.ones((3, 3)) - np.eye(3))]])
    c = np.array([0.0, 0.0, 0.0, 0.01, -0.02, 0.005])
    C = np.zeros((6, 6))
    C[3:, 3:] = 4e-4 * np.array([[1.0, 0.3, 0.2], [0.3, 1.0, 0.25], [0.2, 0.25, 1.0]])
    _, rnxp = api.dims(nxp)
    lam = torch.empty((nzp, nyp, rnxp), device="cuda")
    api.fill_genexp_corr(lam, nxp, tl.nx / 3.0, tl.ny / 3.0, 20.0)
    api.fft_in_place(lam, nxp, api.COVARIANCE)

    def step():
        api.state4d_evolve(run.mu_s, run.mu_d, run.ss, run.sd, run.dd, nxp, E, c, C, lam=lam)
    run.restore()
    step()
    ms = _events_ms(step, reps, run.restore)
    run.restore()
    tr = _traced(step)
    best = statistics.median(ms)
    byt = 8.0 * tl.nbins * (27 + 27 + 1)
    out = {"bins": tl.nbins, "ms": round(best, 4), "ms_stat": "median", "GBps": round(byt / (best * 1e-3) / 1e9, 1),
           "algorithmic_bytes": byt, "kernels": kernel_table(tr)}
    if peak:
        out["roofline"] = roofline_of(tr, peak)
    return out


def ingest_case(a):
    """Data ingest of one 256^3 DATA cube: 258 x 256 column traces of 205 samples (4 ms) resampled onto the
    grid (transforms of length 210 and 840), timed with CUDA events."""
    nxp = nyp = nzp = 256
    nz, n_data = 205, 205
    _, rnxp = api.dims(nxp)
    ncol = rnxp * nyp
    g = torch.Generator(device="cuda").manual_seed(3)
    traces = torch.randn((ncol, n_data), device="cuda", generator=g)
    state = torch.zeros(ncol, dtype=torch.uint8, device="cuda")
    z0d = torch.full((ncol,), 1000.0, device="cuda")
    z0g = z0d + 20.0
    dzg = torch.full((ncol,), 4.0, device="cuda")
    buf = torch.empty((nzp, nyp, rnxp), device="cuda")

    def run():
        api.fill_in_data(buf, nxp, nz, api.DATA, traces, state, z0d, z0g, dzg, 4.0, 40.0)
    run()
    torch.cuda.synchronize()
    ms = []
    for _ in range(a.reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        run()
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    _native.trace_enable(True)
    run()
    tr = _native.trace_collect()
    _native.trace_enable(False)
    best = min(ms)
    print(json.dumps({"case": {"what": "ingest", "workload": "256^3 DATA cube from 66048 traces of 205 samples"},
                      "ms_per_cube": ms, "Mtraces_per_s": ncol / (best * 1e-3) / 1e6,
                      "kernels": {k: {"launches": v[0], "ms": v[1], "GBps": v[2] / max(v[1], 1e-12) / 1e6}
                                  for k, v in tr.items()}}))


def thickness_case(a):
    """Non-constant simbox thickness on the 256^3 five-stack workload: the scale-wavelet division of the five
    DATA cubes with dead-trace interpolation (16 dead traces), the whole mixed inversion on that simbox,
    and the scale-wavelet product of five residual cubes; timed with CUDA events (inputs restored outside
    the timed region; cubes of 67.6 MB, five of them exceed L2)."""
    from . import synthetic as S
    from .pipeline import Inversion
    sc = S.variable_thickness(S.config1(seed=9), amp=0.3, surfaces=True, dead_traces=16, seed=2)
    inv = Inversion(sc, forms=("mixed",))

    def timed(fn, reps):
        ms = []
        for _ in range(reps):
            inv.restore("mixed")
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms

    def multiply():
        api.multiply_by_scale_wavelet(inv.data, sc.nx, sc.ny, sc.nxp, inv.sw_tables, inv.rel_thick, sc.dt_ms,
                                      shift=inv.wshift, gain=inv.wgain)
    for fn in (inv.scale_data, lambda: inv.run("mixed"), multiply):
        timed(fn, 2)
    res = {"divide": timed(inv.scale_data, a.reps), "inversion": timed(lambda: inv.run("mixed"), a.reps),
           "multiply": timed(multiply, a.reps)}
    inv.restore("mixed")
    torch.cuda.synchronize()
    _native.trace_enable(True)
    inv.scale_data()
    multiply()
    torch.cuda.synchronize()
    tr = _native.trace_collect()
    _native.trace_enable(False)
    cube_bytes = 4.0 * sc.rnxp * sc.nyp * sc.nzp
    n = sc.ntheta
    out = {"case": {"what": "thickness", "workload": "256^3 padded cubes, 5 stacks, relative thickness 1 +- 0.3, "
                                                     "local wavelet shift/gain surfaces, 16 dead traces"},
           "ms": res, "n_bad": inv.n_bad,
           # one read and one write of every cell: the per-trace operation's lower bound
           "divide_algorithmic_GBps": 2 * n * cube_bytes / (min(res["divide"]) * 1e-3) / 1e9,
           "multiply_algorithmic_GBps": 2 * n * cube_bytes / (min(res["multiply"]) * 1e-3) / 1e9,
           "inversion_Mbins_per_s": sc.nbins / (min(res["inversion"]) * 1e-3) / 1e6,
           "kernels": {k: {"launches": v[0], "ms": v[1], "GBps": v[2] / max(v[1], 1e-12) / 1e6}
                       for k, v in tr.items()}}
    print(json.dumps(out))


def localnoise_case(a):
    """Local-noise correction (correctAlphaBetaRho) after a 256^3 five-stack inversion: per-trace matrices for
    205 x 205 traces (FP64, one eigen-decomposition of a 5x5 and three of 3x3 matrices per trace) and the
    update of 205^3 cells of the three posterior-mean cubes; timed with CUDA events."""
    from . import synthetic as S
    sc = S.config1(seed=9)
    n = sc.ntheta
    Sm = sc.sigma0.astype(np.float64)
    Smd = 0.45 * Sm + 0.05 * np.diag(np.diag(Sm))
    G = api.local_noise_g(sc.err_theta_cov, Sm, Smd)
    yy, xx = np.mgrid[0:sc.ny, 0:sc.nx]
    scale = torch.from_numpy(np.stack([1.0 + 0.5 * (1 + np.sin(xx / 9.0 + l) * np.cos(yy / 7.0))
                                       for l in range(n)])).cuda()
    mean = [torch.from_numpy(np.ascontiguousarray(m)).cuda() for m in sc.mean]
    post0 = [m + 0.01 for m in mean]
    post = [m.clone() for m in post0]
    smd = torch.empty((sc.ny, sc.nx, 9), dtype=torch.float64, device="cuda")

    def run():
        api.correct_alpha_beta_rho(post, mean, sc.nx, sc.ny, sc.nz, sc.nxp, G, sc.err_theta_cov, Sm, Smd, scale, smd)
    ms = []
    for r in range(a.reps + 2):
        for p, q in zip(post, post0):
            p.copy_(q)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        run()
        e1.record()
        torch.cuda.synchronize()
        if r >= 2:
            ms.append(e0.elapsed_time(e1))
    _native.trace_enable(True)
    run()
    tr = _native.trace_collect()
    _native.trace_enable(False)
    cells = sc.nx * sc.ny * sc.nz
    print(json.dumps({"case": {"what": "localnoise", "workload": "205^3 simbox in 256^3 padded cubes, 5 stacks"},
                      "ms": ms, "traces": sc.nx * sc.ny,
                      "update_algorithmic_GBps": 36.0 * cells / (min(ms) * 1e-3) / 1e9,
                      "kernels": {k: {"launches": v[0], "ms": v[1], "GBps": v[2] / max(v[1], 1e-12) / 1e6}
                                  for k, v in tr.items()}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["fft", "invert", "batch", "copy", "simulate", "timelapse", "ingest",
                                     "thickness", "localnoise", "evolve"])
    ap.add_argument("--nreal", type=int, default=128)
    ap.add_argument("--mb", type=int, default=512)
    ap.add_argument("--ncubes", type=int, default=64)
    ap.add_argument("--streams", type=int, default=3)
    ap.add_argument("--nxp", type=int, default=256)
    ap.add_argument("--nyp", type=int, default=256)
    ap.add_argument("--nzp", type=int, default=64)
    ap.add_argument("--batch", type=int, default=5)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--form", default="mixed")
    a = ap.parse_args()
    _native.lib()
    if a.what == "copy":
        copy_case(a)
        return
    if a.what == "simulate":
        simulate_case(a)
        return
    if a.what == "timelapse":
        timelapse_case(a)
        return
    if a.what == "ingest":
        ingest_case(a)
        return
    if a.what == "thickness":
        thickness_case(a)
        return
    if a.what == "localnoise":
        localnoise_case(a)
        return
    if a.what == "evolve":
        # the 4D state of the 256x256x192 workload (one vintage's data is enough: evolve reads only the state)
        from . import synthetic as S
        from .pipeline import TimeLapse
        tl = S.make_timelapse(205, 205, 154, [0.0, 40.0 / 3, 80.0 / 3, 40.0], 25.0, nxp=256, nyp=256, nzp=192,
                              nvintages=1, seed=3)
        print(json.dumps(measure_evolve(TimeLapse(tl), reps=a.reps)))
        return
    if a.what == "batch":
        # graph replays: time the whole batch with CUDA events
        batch_case(a)  # warm-up and capture
        torch.cuda.synchronize()
        ms = []
        for _ in range(a.reps):
            a._batch.reset()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            a._batch.run(a.form, use_graph=True)
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        bins = a._batch.bins
        best = min(ms)
        # per-kernel view: one eager (not graph-replayed) run under the launch tracer
        a._batch.reset()
        torch.cuda.synchronize()
        _native.trace_enable(True)
        a._batch.run(a.form, use_graph=False)
        torch.cuda.synchronize()
        tr = _native.trace_collect()
        _native.trace_enable(False)
        print(json.dumps({"case": {k: v for k, v in vars(a).items() if not k.startswith("_")}, "bins": bins,
                          "ms_per_batch": ms, "Mbins_per_s": bins / (best * 1e-3) / 1e6,
                          "eager_kernels": {k: {"launches": v[0], "ms": v[1],
                                                "GBps": v[2] / max(v[1], 1e-12) / 1e6} for k, v in tr.items()}}))
        return
    run = {"fft": fft_case, "invert": invert_case, "batch": batch_case}[a.what]
    if a.what == "batch":
        run(a)  # warm-up and graph capture on the same batch
    else:
        run(argparse.Namespace(**{**vars(a), "reps": 1}))  # warm-up (plans, twiddles)
    torch.cuda.synchronize()
    _native.trace_enable(True)
    run(a)
    tr = _native.trace_collect()
    _native.trace_enable(False)
    out = {k: {"launches": v[0], "ms_per_launch": v[1] / v[0], "GBps": v[2] / max(v[1], 1e-12) / 1e6}
           for k, v in tr.items()}
    case = {k: v for k, v in vars(a).items() if not k.startswith("_")}
    print(json.dumps({"case": case, "kernels": out}))


if __name__ == "__main__":
    main()
