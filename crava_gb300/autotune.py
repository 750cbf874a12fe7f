"""Measure the launch variants of the hot kernels on this GPU and store the winners.

    python -m crava_gb300.autotune [--out crava_gb300/tuning.json] [--lengths ...] [--batch-lengths]

Candidates (see cg_tune_set in include/cravagpu.h):
  * column transform pass, per axis length: the kernel -- staged (0),
    persistent double-buffered (1), register-direct (2), four-step (3),
    persistent register-prefetch (4) or, at length 256, persistent four-step
    fed by tensor-memory-accelerator loads (5) -- where the length has the
    specialised kernels, with a resident-CTA target of 2 or 3 (or 4 for the
    register-direct and four-step kernels up to 256); and, for the four-step
    kernel, the tile shape: the factorisation N1 x N2 (smallest divisor of n
    not below sqrt(n), or swapped) and the tile width (16 or 32 columns);
  * x-row pass, per half length nxp/2: staged (0) or four-step (1) kernel;
  * fused bin kernel, per stack count: unconstrained build or a 128-, 96- or
    85-register build (4, 5 or 6 resident 128-thread CTAs), and the 256-bin runs
    one CTA solves per staged per-k table (1, 2, 4, 8, or adaptive).
Each candidate is timed with the library's launch tracer (CUDA events on the
launch stream) on cubes larger than L2; the fastest is kept.  The loader
(crava_gb300._native.lib) applies tuning.json when it is present.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import torch

from . import _native, api

KEY_COLS_MINB, KEY_COLS_PIPE, KEY_BIN_MINB, KEY_ROWS = 0, 1, 2, 3
KEY_COLS_SHAPE, KEY_BIN_RUNS = 7, 8

# the column lengths of the 64-cube batch workload that have no specialised staged / register-direct kernel
BATCH_LENGTHS = (40, 42, 45, 48, 54, 60, 75, 84, 90, 105, 108, 112, 125, 135, 140, 144, 147, 150, 162, 168, 175,
                 180, 189, 196, 210, 216, 224)


def _time_kernels(fn, prefix, reps=3):
    fn()  # warm-up: tables, attributes
    torch.cuda.synchronize()
    _native.trace_enable(True)
    for _ in range(reps):
        fn()
    tr = _native.trace_collect()
    _native.trace_enable(False)
    return sum(v[1] for k, v in tr.items() if k.startswith(prefix)) / reps


def _square(n):
    """True when the four-step factors of n are equal (n = d * d, d its smallest divisor not below sqrt(n))."""
    d = next(d for d in range(1, n + 1) if n % d == 0 and d * d >= n)
    return d * d == n


def tune_cols(lengths, L):
    out = {}
    for n in lengths:
        g = torch.Generator(device="cuda").manual_seed(n)
        nxp = 256
        cubes = [torch.randn((n, n, nxp + 2), device="cuda", generator=g) for _ in range(3)]

        def run():
            api.fft_in_place_batch(cubes, nxp, api.DATA)
            api.fft_in_place_batch(cubes, nxp, api.DATA, inverse=True)
        # does the length have the specialised kernels?  (the register-direct kernel shows in the trace)
        L.cg_tune_set(KEY_COLS_PIPE, n, 2)
        L.cg_tune_set(KEY_COLS_SHAPE, n, 0)
        run()
        torch.cuda.synchronize()
        _native.trace_enable(True)
        run()
        special = "k_fft_cols_rd" in _native.trace_collect()
        _native.trace_enable(False)
        shapes = (0, 2) if _square(n) else (0, 1, 2, 3)
        cands = []
        if special:
            for pipe in (0, 1, 2, 3, 4) + ((5,) if n == 256 else ()):
                for minb in ((2, 3, 4) if pipe in (2, 3) and n <= 256 else (3,) if pipe == 5 else (2, 3)):
                    for shape in (shapes if pipe == 3 else (0,)):
                        cands.append((pipe, minb, shape))
        else:
            cands = [(3, 3, shape) for shape in shapes]
        best = None
        for pipe, minb, shape in cands:
            L.cg_tune_set(KEY_COLS_PIPE, n, pipe)
            L.cg_tune_set(KEY_COLS_MINB, n, minb)
            L.cg_tune_set(KEY_COLS_SHAPE, n, shape)
            ms = _time_kernels(run, "k_fft_cols")
            if best is None or ms < best[0]:
                best = (ms, pipe, minb, shape)
        L.cg_tune_set(KEY_COLS_PIPE, n, best[1])
        L.cg_tune_set(KEY_COLS_MINB, n, best[2])
        L.cg_tune_set(KEY_COLS_SHAPE, n, best[3])
        out[str(n)] = {"pipe": best[1], "minb": best[2], "shape": best[3], "ms": round(best[0], 4),
                       "candidates": len(cands)}
        del cubes
        torch.cuda.empty_cache()
    return out


def tune_rows(halves, L):
    out = {}
    for m in halves:
        g = torch.Generator(device="cuda").manual_seed(m)
        nxp = 2 * m
        cubes = [torch.randn((128, 256, nxp + 2), device="cuda", generator=g) for _ in range(3)]

        def run():
            api.fft_in_place_batch(cubes, nxp, api.DATA)
            api.fft_in_place_batch(cubes, nxp, api.DATA, inverse=True)
        best = None
        for kern in (0, 1):
            L.cg_tune_set(KEY_ROWS, m, kern)
            ms = _time_kernels(run, ("k_r2c_rows", "k_c2r_rows"))
            if best is None or ms < best[0]:
                best = (ms, kern)
        L.cg_tune_set(KEY_ROWS, m, best[1])
        out[str(m)] = {"kernel": best[1], "ms": round(best[0], 4)}
        del cubes
        torch.cuda.empty_cache()
    return out


def tune_bin(ntheta_list, L):
    from . import synthetic as S
    from .pipeline import Inversion
    out = {}
    for nt in ntheta_list:
        sc = S.make_scenario(160, 160, 160, [40.0 * i / max(nt - 1, 1) for i in range(nt)], 25.0, nxp=200, nyp=200,
                             nzp=200, sn=3.0, seed=nt)
        inv = Inversion(sc, forms=("mixed",))

        def run():
            inv.restore("mixed")
            inv.run("mixed")
        best = None
        for minb in (1, 4, 5, 6):
            for runs in (0, 1, 2, 4, 8):
                L.cg_tune_set(KEY_BIN_MINB, nt, minb)
                L.cg_tune_set(KEY_BIN_RUNS, nt, runs)
                ms = _time_kernels(run, ("k_invert_fused", "k_invert_info"))
                if best is None or ms < best[0]:
                    best = (ms, minb, runs)
        L.cg_tune_set(KEY_BIN_MINB, nt, best[1])
        L.cg_tune_set(KEY_BIN_RUNS, nt, best[2])
        out[str(nt)] = {"minb": best[1], "runs": best[2], "ms": round(best[0], 4)}
        del inv
        torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json"))
    ap.add_argument("--lengths", default="128,160,192,200,240,256")
    ap.add_argument("--ntheta", default="3,5,8")
    ap.add_argument("--halves", default="64,100,128,200,256")
    ap.add_argument("--batch-lengths", action="store_true",
                    help="also tune the column lengths of the 64-cube batch workload")
    a = ap.parse_args()
    L = _native.lib()
    L.cg_tune_clear()
    t0 = time.time()
    lengths = [int(x) for x in a.lengths.split(",")]
    if a.batch_lengths:
        lengths += [n for n in BATCH_LENGTHS if n not in lengths]
    cols = tune_cols(lengths, L)
    rows = tune_rows([int(x) for x in a.halves.split(",")], L)
    binr = tune_bin([int(x) for x in a.ntheta.split(",")], L)
    res = {"device": torch.cuda.get_device_name(0), "cols": cols, "rows": rows, "bin": binr,
           "tuning_seconds": round(time.time() - t0, 1)}
    with open(a.out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
