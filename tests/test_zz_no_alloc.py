"""The transforms that allocate nothing (cg_fft3d_r2c_noalloc / cg_fft3d_c2r_noalloc).

They exist for callers that cannot let a library call cudaMalloc -- an
application capturing a CUDA graph with allocation forbidden, or a host whose
device memory is owned by its own allocator.  They must give the same
spectra and cubes as cg_fft3d_r2c / cg_fft3d_c2r (whose twiddle tables are
allocated on first use), call after call, although every call rewrites the
one shared table array.  This file is collected last so that a failure here
cannot hide the result of any other test.
"""
import ctypes as ct

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FFT_TOL = 2e-6  # the FP32 transform tolerance used by the other transform tests


def _rel(a, b):
    return float(torch.linalg.vector_norm((a - b).double()) / torch.linalg.vector_norm(b.double()))


def _cube(nxp, nyp, nzp, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randn((nzp, nyp, 2 * (nxp // 2 + 1)), device="cuda", generator=g)
    x[..., nxp:] = 0
    return x


def test_noalloc_transforms_match_the_allocating_ones(cuda, native):
    from crava_gb300 import api
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    # two calls in a row with different sizes: the second must not see the first one's tables
    for (nxp, nyp, nzp, ctype, seed) in [(256, 256, 64, api.DATA, 1), (80, 160, 200, api.COVARIANCE, 2)]:
        x = _cube(nxp, nyp, nzp, seed)
        a = x.clone()
        b = x.clone()
        assert native.cg_fft3d_r2c(ct.c_void_p(a.data_ptr()), nxp, nyp, nzp, ctype, stream) == 0
        assert native.cg_fft3d_r2c_noalloc(ct.c_void_p(b.data_ptr()), nxp, nyp, nzp, ctype, stream) == 0, \
            native.cg_last_error()
        torch.cuda.synchronize()
        assert _rel(b, a) < FFT_TOL
        assert native.cg_fft3d_c2r(ct.c_void_p(a.data_ptr()), nxp, nyp, nzp, ctype, stream) == 0
        assert native.cg_fft3d_c2r_noalloc(ct.c_void_p(b.data_ptr()), nxp, nyp, nzp, ctype, stream) == 0, \
            native.cg_last_error()
        torch.cuda.synchronize()
        assert _rel(b[..., :nxp], a[..., :nxp]) < FFT_TOL
        assert _rel(b[..., :nxp], x[..., :nxp]) < FFT_TOL  # both cube types round-trip to the input


def test_noalloc_rejects_what_it_cannot_hold(cuda, native):
    from crava_gb300 import api
    x = torch.zeros((4, 4, 16), device="cuda")
    s = ct.c_void_p(0)
    # beyond the shared twiddle array
    assert native.cg_fft3d_r2c_noalloc(ct.c_void_p(x.data_ptr()), 8192, 8192, 8192, api.DATA, s) == -1
    assert b"exceeds" in native.cg_last_error()
    # a length without a specialised transform
    assert native.cg_fft3d_r2c_noalloc(ct.c_void_p(x.data_ptr()), 14, 4, 4, api.DATA, s) == -3
    assert b"no specialised transform" in native.cg_last_error()
    assert torch.count_nonzero(x) == 0


_CHILD = r"""
import ctypes as ct, json, sys
sys.path.insert(0, sys.argv[1])
import crava_gb300
L = crava_gb300.lib()
import torch
torch.cuda.init()
nxp, nyp, nzp = 256, 256, 64   # y axis of length 256: the TMA-fed pass when the tuning value is 5
x = torch.randn((nzp, nyp, nxp + 2), device="cuda")
x[..., nxp:] = 0
x0 = x.clone()
a = x.clone()
s = ct.c_void_p(0)
torch.cuda.synchronize()
calls0 = L.cg_alloc_calls()
rcs, free = [], []
for _ in range(3):
    rcs.append(L.cg_fft3d_r2c_noalloc(ct.c_void_p(x.data_ptr()), nxp, nyp, nzp, 1, s))
    rcs.append(L.cg_fft3d_c2r_noalloc(ct.c_void_p(x.data_ptr()), nxp, nyp, nzp, 1, s))
    torch.cuda.synchronize()
    free.append(torch.cuda.mem_get_info()[0])
calls1 = L.cg_alloc_calls()
# the allocating transform at the same size, for contrast: it allocates its twiddle tables and, on the
# TMA-fed pass, the fault word
rcs.append(L.cg_fft3d_r2c(ct.c_void_p(a.data_ptr()), nxp, nyp, nzp, 1, s))
torch.cuda.synchronize()
calls2 = L.cg_alloc_calls()
flag = ct.c_int(0)
rcs.append(L.cg_device_faults(ct.byref(flag)))
err = float(torch.linalg.vector_norm((x - x0)[..., :nxp].double()) / torch.linalg.vector_norm(x0.double()))
print(json.dumps({"rcs": rcs, "calls": [calls0, calls1, calls2], "free": free, "faults": flag.value,
                  "roundtrip_err": err}))
"""


def test_noalloc_allocates_nothing_with_the_tma_pass_selected(cuda, native):
    """A fresh process with the tuning table pointing length-256 column passes at the TMA-fed kernel,
    whose fault word is allocated on first use.  Three rounds of no-allocation transforms must make no
    memory allocation of the library's own (cg_alloc_calls counts every one it makes), while one call of
    the allocating transform at the same size does make some.  Device free memory is also compared
    across the later rounds: the first launches of kernels may still map memory of the driver's own
    (code and per-thread local memory are set up lazily), which no library call controls."""
    import json
    import os
    import subprocess
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, CRAVA_COLS_PIPE="5")
    out = subprocess.run([sys.executable, "-c", _CHILD, repo], env=env, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    r = json.loads(out.stdout.strip().splitlines()[-1])
    print(r)
    assert r["rcs"] == [0] * 8, r
    assert r["roundtrip_err"] < FFT_TOL, r
    assert r["faults"] == 0, r
    c0, c1, c2 = r["calls"]
    assert c1 == c0, f"the no-allocation transforms allocated: {r}"
    assert c2 > c1, f"the allocating transform was not seen allocating: {r}"
    assert r["free"][1] == r["free"][2], f"repeated no-allocation calls changed free device memory: {r}"
