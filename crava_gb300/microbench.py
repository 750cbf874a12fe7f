"""Time (or profile) one stage of the inversion in isolation on the GPU.

    python -m crava_gb300.microbench fft   --nxp 256 --nyp 256 --nzp 64 --batch 5 --reps 3
    python -m crava_gb300.microbench invert --nxp 256 --nyp 256 --nzp 64 --form mixed --reps 3

Inputs are seeded random cubes (fft) or a scaled config-1 scenario (invert).
Prints one JSON line with per-kernel launch times and algorithmic bandwidth
from the library's launch tracer.  Small sizes keep ncu captures short.
"""
from __future__ import annotations

import argparse
import json

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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["fft", "invert"])
    ap.add_argument("--nxp", type=int, default=256)
    ap.add_argument("--nyp", type=int, default=256)
    ap.add_argument("--nzp", type=int, default=64)
    ap.add_argument("--batch", type=int, default=5)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--form", default="mixed")
    a = ap.parse_args()
    _native.lib()
    run = fft_case if a.what == "fft" else invert_case
    run(argparse.Namespace(**{**vars(a), "reps": 1}))  # warm-up (plans, twiddles)
    torch.cuda.synchronize()
    _native.trace_enable(True)
    run(a)
    tr = _native.trace_collect()
    _native.trace_enable(False)
    out = {k: {"launches": v[0], "ms_per_launch": v[1] / v[0], "GBps": v[2] / max(v[1], 1e-12) / 1e6}
           for k, v in tr.items()}
    print(json.dumps({"case": vars(a), "kernels": out}))


if __name__ == "__main__":
    main()
