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
