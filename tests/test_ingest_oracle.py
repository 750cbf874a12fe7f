"""The oracle's restatement of FFTGrid::fillInData's per-trace core, on cases with known answers."""
import numpy as np


def test_band_limited_trace_is_resampled_exactly(oracle):
    """A periodic band-limited trace: the 4x FFT upsampling + linear interpolation reproduces it at the cell
    times, scaled by nt/rnt as resampleTrace (src/fftgrid.cpp:506-561) scales by 1/rnt."""
    nxp, nyp, nzp, nz, nd = 4, 1, 64, 64, 64
    _, rnxp = oracle.dims(nxp)
    t = np.arange(nd)
    tr = np.tile(np.sin(2 * np.pi * 3 * t / nd).astype(np.float32), (rnxp * nyp, 1))
    st = np.zeros(rnxp * nyp, np.uint8)
    z0 = np.zeros(rnxp * nyp, np.float32)
    dzg = np.full(rnxp * nyp, 4.0, np.float32)
    out, ext = oracle.fill_in_data(nxp, nyp, nzp, nz, True, tr, st, z0, z0 + 1.0, dzg, 4.0, 0.0)
    expect = np.sin(2 * np.pi * 3 * (np.arange(nzp) + 0.25) / nd) * (64 / 66)
    assert np.abs(out[:32, 0, 0] - expect[:32]).max() < 1e-6
    assert ext == [0, 0]


def test_non_data_trend_and_extrapolation(oracle):
    """A pure linear ramp with leading and trailing zeros: extrapolation fills the ends, the trend is removed
    before and restored after resampling, so every simbox cell holds the ramp at the cell's time."""
    nxp, nyp, nzp, nz, nd = 4, 1, 40, 32, 50
    _, rnxp = oracle.dims(nxp)
    ramp = (2.0 + 0.1 * np.arange(nd)).astype(np.float32)
    tr = np.tile(ramp, (rnxp * nyp, 1))
    tr[:, :3] = 0
    tr[:, -2:] = 0
    st = np.zeros(rnxp * nyp, np.uint8)
    z0d = np.zeros(rnxp * nyp, np.float32)
    dzg = np.full(rnxp * nyp, 4.0, np.float32)
    out, ext = oracle.fill_in_data(nxp, nyp, nzp, nz, False, tr, st, z0d, z0d + 40.0, dzg, 4.0, 0.0)
    assert ext == [3, 2]
    # after extrapolation the trace is ramp[3] for k<3, ramp, ramp[-3] for the last 2 samples; the trend line
    # between the end samples is restored exactly; the residual (ramp minus that line) is resampled
    x = ramp.copy()
    x[:3] = ramp[3]
    x[-2:] = ramp[-3]
    line = x[0] + (x[-1] - x[0]) * np.arange(nd) / (nd - 1)
    k = np.arange(nz)
    tk = (40.0 + 4.0 * k) / 4.0                      # cell time in samples
    expect = np.interp(tk, np.arange(nd), x)        # the trace itself at the cell times (smooth region)
    mid = (tk > 8) & (tk < nd - 10)
    assert np.abs(out[:nz, 0, 0][mid] - expect[mid]).max() < 0.05 * np.abs(expect).max()
    assert np.all(np.isfinite(out))


def test_dead_columns_are_zero(oracle):
    nxp, nyp, nzp, nz, nd = 6, 2, 16, 12, 20
    _, rnxp = oracle.dims(nxp)
    tr = np.ones((rnxp * nyp, nd), np.float32)
    st = np.zeros(rnxp * nyp, np.uint8)
    st[[1, 5]] = 1
    z = np.zeros(rnxp * nyp, np.float32)
    out, _ = oracle.fill_in_data(nxp, nyp, nzp, nz, True, tr, st, z, z, z + 4.0, 4.0, 0.0)
    flat = out.reshape(nzp, -1)
    assert np.all(flat[:, [1, 5]] == 0) and np.any(flat[:, 0] != 0)
