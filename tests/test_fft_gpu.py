"""GPU 3D transforms against the reference's FFTW 2.1.2 vectors and the oracle."""
import ctypes as ct

import numpy as np
import pytest
import torch

from conftest import from_cube, golden, rel

pytestmark = pytest.mark.gpu

FFT_TOL = 2e-6  # FP32, relative L2 over the cube


@pytest.mark.parametrize("case", ["fft_even.npz", "fft_odd.npz", "fft_mixed.npz"])
def test_fft_matches_reference_fftw(cuda, case):
    from crava_gb300 import api
    g = golden(case)
    nxp = int(g["nxp"])
    for ctype, key in ((api.DATA, "r2c_data"), (api.COVARIANCE, "r2c_cov")):
        x = torch.from_numpy(g["real_in"].copy()).cuda()
        api.fft_in_place(x, nxp, ctype)
        assert rel(from_cube(x), g[key]) < FFT_TOL, key
    for ctype, key in ((api.PARAMETER, "c2r_param"), (api.COVARIANCE, "c2r_cov")):
        x = torch.from_numpy(g["spec_in"].view(np.float32).copy()).cuda()
        api.inv_fft_in_place(x, nxp, ctype)
        assert rel(x.cpu().numpy()[..., :nxp], g[key][..., :nxp]) < FFT_TOL, key


SIZES = [(80, 80, 160), (16, 12, 20), (15, 9, 7), (21, 15, 35), (49, 27, 25), (128, 1, 1), (1, 64, 1),
         (2, 2, 2), (200, 100, 8), (98, 54, 45), (256, 16, 24), (7, 5, 3), (64, 343, 10),
         # specialised axes with one batch row and a column tail (2D / 1D prior-spectrum transforms)
         (80, 64, 1), (256, 256, 1), (100, 1, 128), (48, 1, 1)]


@pytest.mark.parametrize("dims", SIZES)
def test_fft_matches_oracle(cuda, oracle, dims):
    from crava_gb300 import api
    nxp, nyp, nzp = dims
    cnxp, rnxp = oracle.dims(nxp)
    rng = np.random.default_rng(nxp * 1000 + nyp * 10 + nzp)
    x = np.zeros((nzp, nyp, rnxp), np.float32)
    x[..., :nxp] = rng.standard_normal((nzp, nyp, nxp))
    ref = oracle.fft3d_r2c(x, nxp, oracle.DATA, "d")
    t = torch.from_numpy(x.copy()).cuda()
    api.fft_in_place(t, nxp, api.DATA)
    assert rel(from_cube(t), ref) < FFT_TOL
    spec = (rng.standard_normal((nzp, nyp, cnxp)) + 1j * rng.standard_normal((nzp, nyp, cnxp))).astype(np.complex64)
    ref = oracle.fft3d_c2r(spec, nxp, oracle.PARAMETER, "d")[..., :nxp]
    t = torch.from_numpy(spec.view(np.float32).copy()).cuda()
    api.inv_fft_in_place(t, nxp, api.PARAMETER)
    assert rel(t.cpu().numpy()[..., :nxp], ref) < FFT_TOL


@pytest.mark.parametrize("dims", [(80, 80, 160), (21, 15, 35), (64, 48, 40)])
def test_fft_fp64_matches_fp64_oracle(cuda, oracle, dims):
    from crava_gb300 import api
    nxp, nyp, nzp = dims
    cnxp, rnxp = oracle.dims(nxp)
    rng = np.random.default_rng(5)
    x = np.zeros((nzp, nyp, rnxp), np.float64)
    x[..., :nxp] = rng.standard_normal((nzp, nyp, nxp))
    ref = oracle.fft3d_r2c(x, nxp, oracle.COVARIANCE, "d")
    t = torch.from_numpy(x.copy()).cuda()
    api.fft_in_place(t, nxp, api.COVARIANCE)
    assert rel(from_cube(t), ref) < 1e-13
    api.inv_fft_in_place(t, nxp, api.COVARIANCE)
    assert rel(t.cpu().numpy()[..., :nxp], x[..., :nxp]) < 1e-13


def test_batch_equals_single(cuda):
    from crava_gb300 import api
    nxp, nyp, nzp = 40, 30, 24
    g = torch.Generator(device="cuda").manual_seed(3)
    cubes = [torch.randn((nzp, nyp, 42), device="cuda", generator=g) for _ in range(19)]
    singles = [c.clone() for c in cubes]
    api.fft_in_place_batch(cubes, nxp, api.DATA)
    for s in singles:
        api.fft_in_place(s, nxp, api.DATA)
    for a, b in zip(cubes, singles):
        assert torch.equal(a, b)
    api.fft_in_place_batch(cubes, nxp, api.DATA, inverse=True)


def test_round_trip_full_size(cuda):
    """256^3 DATA transform and back is the identity (1/sqrt(N) both ways)."""
    from crava_gb300 import api
    n = 256
    g = torch.Generator(device="cuda").manual_seed(11)
    x = torch.randn((n, n, n + 2), device="cuda", generator=g)
    x[..., n:] = 0
    y = x.clone()
    api.fft_in_place(y, n, api.DATA)
    # Parseval for the norm-preserving transform: sum |x|^2 = sum over the full spectrum
    s = api.as_spectrum(y)
    w = torch.full((n // 2 + 1,), 2.0, device="cuda", dtype=torch.float64)
    w[0] = 1
    w[-1] = 1
    e_spec = (s.abs().double() ** 2 * w).sum()
    e_x = (x[..., :n].double() ** 2).sum()
    assert abs(float(e_spec / e_x) - 1) < 1e-5
    api.inv_fft_in_place(y, n, api.DATA)
    err = float((y[..., :n] - x[..., :n]).norm() / x[..., :n].norm())
    assert err < 2e-6


def test_host_variant_matches_device(cuda, native):
    from crava_gb300 import api
    nxp, nyp, nzp = 30, 20, 18
    rng = np.random.default_rng(9)
    x = np.zeros((nzp, nyp, 32), np.float32)
    x[..., :nxp] = rng.standard_normal((nzp, nyp, nxp))
    h = x.copy()
    assert native.cg_fft3d_r2c_host(h.ctypes.data, nxp, nyp, nzp, api.DATA) == 0
    t = torch.from_numpy(x.copy()).cuda()
    api.fft_in_place(t, nxp, api.DATA)
    np.testing.assert_array_equal(h, t.cpu().numpy())
    assert native.cg_fft3d_c2r_host(h.ctypes.data, nxp, nyp, nzp, api.DATA) == 0
    assert rel(h[..., :nxp], x[..., :nxp]) < FFT_TOL


def test_bad_arguments_return_status(cuda, native):
    from crava_gb300 import api
    t = torch.zeros((8, 8, 12), device="cuda")
    s = ct.c_void_p(0)
    assert native.cg_fft3d_r2c(ct.c_void_p(t.data_ptr()), 0, 8, 8, api.DATA, s) == -1
    assert native.cg_fft3d_r2c(ct.c_void_p(t.data_ptr()), 10, 8, 8, 0, s) == -1
    assert native.cg_fft3d_r2c(None, 10, 8, 8, api.DATA, s) == -1
    # 11 and 13 are not factors the reference pads to; refused, not mis-transformed
    t2 = torch.zeros((8, 8, 12), device="cuda")
    assert native.cg_fft3d_r2c(ct.c_void_p(t2.data_ptr()), 11, 8, 8, api.DATA, s) == -3
    assert b"prime factor" in native.cg_last_error()
    torch.cuda.synchronize()


# every kernel variant of the tuning table -- column pass (CG_TUNE_COLS_PIPE: 0 staged, 1 persistent,
# 2 register-direct, 3 four-step) with both resident-CTA targets, x-row pass (CG_TUNE_ROWS_KERNEL: 0 staged,
# 1 four-step) -- on specialised lengths with full tiles, column tails and one-row batches
VARIANT_SIZES = [(80, 80, 160), (256, 256, 1), (100, 1, 128), (64, 200, 96), (128, 240, 64), (96, 64, 512),
                 (400, 120, 100), (480, 192, 80), (320, 384, 64), (200, 160, 200), (512, 100, 64), (120, 256, 240)]


_VARIANT_REFS = {}


def _variant_case(oracle, nxp, nyp, nzp):
    key = (nxp, nyp, nzp)
    if key not in _VARIANT_REFS:
        _, rnxp = oracle.dims(nxp)
        rng = np.random.default_rng(nxp + nyp + nzp)
        x = np.zeros((nzp, nyp, rnxp), np.float32)
        x[..., :nxp] = rng.standard_normal((nzp, nyp, nxp))
        _VARIANT_REFS[key] = (x, oracle.fft3d_r2c(x, nxp, oracle.DATA, "d"))
    return _VARIANT_REFS[key]


@pytest.mark.parametrize("pipe", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("minb", [2, 3, 4])
def test_column_pass_variants_match_oracle(cuda, oracle, native, pipe, minb):
    from crava_gb300 import api
    native.cg_tune_clear()
    try:
        assert native.cg_tune_set(1, 0, pipe) == 0 and native.cg_tune_set(0, 0, minb) == 0
        assert native.cg_tune_set(3, 0, minb % 2) == 0   # four-step rows with minb 3, staged rows otherwise
        for nxp, nyp, nzp in VARIANT_SIZES:
            x, ref = _variant_case(oracle, nxp, nyp, nzp)
            t = torch.from_numpy(x.copy()).cuda()
            api.fft_in_place(t, nxp, api.DATA)
            assert rel(from_cube(t), ref) < FFT_TOL, (nxp, nyp, nzp)
            api.inv_fft_in_place(t, nxp, api.DATA)
            assert rel(t.cpu().numpy()[..., :nxp], x[..., :nxp]) < FFT_TOL, (nxp, nyp, nzp)
    finally:
        from crava_gb300 import _native
        native.cg_tune_clear()
        _native._apply_tuning(native)


# the TMA-fed column pass (tuning value 5, length 256 along y or z): odd and even cnxp, odd rows
# shifted by one column in the z pass, tail column groups, cubes batched in one launch, and an odd
# nyp that falls back to the register-direct kernel for the z pass
TMA_SIZES = [(256, 256, 4), (30, 256, 256), (64, 40, 256), (120, 256, 6), (64, 45, 256), (256, 6, 256)]


@pytest.mark.parametrize("dims", TMA_SIZES)
def test_tma_column_pass_matches_oracle(cuda, oracle, native, dims):
    from crava_gb300 import _native, api
    nxp, nyp, nzp = dims
    native.cg_tune_clear()
    try:
        assert native.cg_tune_set(1, 256, 5) == 0
        x, ref = _variant_case(oracle, nxp, nyp, nzp)
        cubes = [torch.from_numpy(x.copy()).cuda() for _ in range(3)]
        _native.trace_enable(True)
        api.fft_in_place_batch(cubes, nxp, api.DATA)
        for t in cubes:
            assert rel(from_cube(t), ref) < FFT_TOL, dims
        api.fft_in_place_batch(cubes, nxp, api.DATA, inverse=True)
        tr = _native.trace_collect()
        _native.trace_enable(False)
        for t in cubes:
            assert rel(t.cpu().numpy()[..., :nxp], x[..., :nxp]) < FFT_TOL, dims
        uses = nyp == 256 or (nzp == 256 and nyp % 2 == 0)
        assert ("k_fft_cols_tma" in tr) == uses, tr.keys()
        assert _native.device_faults() == 0
    finally:
        _native.trace_enable(False)
        native.cg_tune_clear()
        _native._apply_tuning(native)


# four-step kernels of the further 7-smooth lengths (columns 16..504, even x rows up to nxp = 504)
EXT_SIZES = [(42, 54, 90), (126, 189, 144), (36, 500, 21), (180, 35, 405), (56, 243, 16), (504, 98, 75),
             (432, 448, 18), (84, 27, 441), (252, 150, 49), (300, 225, 28), (216, 63, 486), (448, 125, 32),
             (196, 336, 20), (288, 81, 360), (140, 392, 45), (112, 270, 105),
             # odd half lengths (nxp = 2M, M odd) and narrow cubes (every column a tail column)
             (54, 54, 90), (150, 25, 36), (270, 18, 49), (378, 20, 15), (90, 100, 64), (250, 64, 30), (30, 45, 63),
             # odd x lengths
             (15, 20, 16), (63, 40, 30), (75, 18, 28), (125, 32, 20), (189, 24, 16), (243, 16, 18), (45, 60, 21)]


@pytest.mark.parametrize("dims", EXT_SIZES)
def test_extended_lengths_match_oracle(cuda, oracle, dims):
    from crava_gb300 import api
    nxp, nyp, nzp = dims
    x, ref = _variant_case(oracle, nxp, nyp, nzp)
    t = torch.from_numpy(x.copy()).cuda()
    api.fft_in_place(t, nxp, api.DATA)
    assert rel(from_cube(t), ref) < FFT_TOL
    api.inv_fft_in_place(t, nxp, api.DATA)
    assert rel(t.cpu().numpy()[..., :nxp], x[..., :nxp]) < FFT_TOL


# x + y plane kernels (one z-plane per two-CTA cluster, intermediate spectrum in distributed shared memory):
# against the FP64 oracle, bit for bit against the separate four-step x-row and column passes they restate,
# several cubes in one launch, and the inverse's addend and exp epilogue
XY_SIZES = [(256, 256, 3), (256, 256, 40)]


@pytest.mark.parametrize("dims", XY_SIZES)
def test_xy_plane_kernels_match_oracle_and_separate_passes(cuda, oracle, native, dims):
    from crava_gb300 import _native, api
    nxp, nyp, nzp = dims
    x, ref = _variant_case(oracle, nxp, nyp, nzp)
    native.cg_tune_clear()
    try:
        # separate passes with the four-step column kernel (the arithmetic the plane kernels restate)
        assert native.cg_tune_set(6, 0, 0) == 0 and native.cg_tune_set(1, 0, 3) == 0
        sep = [torch.from_numpy(x.copy()).cuda() for _ in range(3)]
        api.fft_in_place_batch(sep, nxp, api.DATA)
        sep_spec = [s.clone() for s in sep]
        api.fft_in_place_batch(sep, nxp, api.DATA, inverse=True)
        assert native.cg_tune_set(6, 0, 1) == 0
        cubes = [torch.from_numpy(x.copy()).cuda() for _ in range(3)]
        _native.trace_enable(True)
        api.fft_in_place_batch(cubes, nxp, api.DATA)
        spec = [c.clone() for c in cubes]
        api.fft_in_place_batch(cubes, nxp, api.DATA, inverse=True)
        tr = _native.trace_collect()
        _native.trace_enable(False)
        assert "k_xy_r2c" in tr and "k_yx_c2r" in tr, tr.keys()
        for s, t, a, b in zip(spec, cubes, sep_spec, sep):
            assert rel(from_cube(s), ref) < FFT_TOL
            assert rel(t.cpu().numpy()[..., :nxp], x[..., :nxp]) < FFT_TOL
            assert torch.equal(s, a), "forward plane kernel differs from the separate passes"
            assert torch.equal(t, b), "inverse plane kernel differs from the separate passes"
        # inverse with an addend (the posterior-mean add of simulation) and with the exp epilogue: identical to
        # the separate passes
        cnxp, rnxp = oracle.dims(nxp)
        g = torch.Generator(device="cuda").manual_seed(7)
        chol = torch.randn((9, nzp, nyp, cnxp), device="cuda", generator=g)
        pm = [torch.randn((nzp, nyp, rnxp), device="cuda", generator=g) for _ in range(3)]
        spec = [torch.randn((nzp, nyp, rnxp), device="cuda", generator=g) * 0.01 for _ in range(2)]
        out = {}
        for xy in (0, 1):
            assert native.cg_tune_set(6, 0, xy) == 0
            fields = [torch.empty((nzp, nyp, rnxp), device="cuda") for _ in range(3)]
            api.simulate_fields(chol, fields, nxp, seed=5, post_mean=pm)
            ex = [s.clone() for s in spec]
            api.inv_fft_exp_batch(ex, nxp, api.PARAMETER)
            out[xy] = (fields, ex)
        for a, b in zip(out[0][0] + out[0][1], out[1][0] + out[1][1]):
            assert torch.equal(a, b), "inverse plane kernel with addend / epilogue differs from the separate passes"
    finally:
        _native.trace_enable(False)
        native.cg_tune_clear()
        _native._apply_tuning(native)


# the four-step column tile shapes the autotuner chooses among (CG_TUNE_COLS_SHAPE: swapped factors, other
# tile width), on tuned and further lengths, every axis
SHAPE_SIZES = [(200, 120, 90), (42, 150, 189), (64, 96, 45), (40, 216, 147)]


@pytest.mark.parametrize("shape", [1, 2, 3])
def test_column_tile_shapes_match_oracle(cuda, oracle, native, shape):
    from crava_gb300 import _native, api
    native.cg_tune_clear()
    try:
        assert native.cg_tune_set(1, 0, 3) == 0 and native.cg_tune_set(7, 0, shape) == 0
        for nxp, nyp, nzp in SHAPE_SIZES:
            x, ref = _variant_case(oracle, nxp, nyp, nzp)
            t = torch.from_numpy(x.copy()).cuda()
            api.fft_in_place(t, nxp, api.DATA)
            assert rel(from_cube(t), ref) < FFT_TOL, (shape, nxp, nyp, nzp)
            api.inv_fft_in_place(t, nxp, api.DATA)
            assert rel(t.cpu().numpy()[..., :nxp], x[..., :nxp]) < FFT_TOL, (shape, nxp, nyp, nzp)
    finally:
        native.cg_tune_clear()
        _native._apply_tuning(native)
