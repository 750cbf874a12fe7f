"""Non-constant simbox thickness on the GPU against the oracle: the scale-wavelet division of the data
(Crava::divideDataByScaleWavelet), its inverse on output cubes (multiplyDataByScaleWaveletAndWriteToFile)
and the dead-trace interpolation (FFTGrid::interpolateSeismic)."""
import numpy as np
import pytest
import torch

from conftest import rel

pytestmark = pytest.mark.gpu

# (nx, ny, nz, nxp, nyp, nzp): even and odd padded lengths in x and z
DIMS = [(20, 16, 24, 24, 20, 30), (19, 15, 20, 25, 18, 27), (50, 40, 64, 64, 50, 80)]


def _case(dims, seed, surfaces):
    from crava_gb300 import synthetic as S
    nx, ny, nz, nxp, nyp, nzp = dims
    sc = S.make_scenario(nx, ny, nz, [5.0, 15.0, 30.0], 28.0, nxp=nxp, nyp=nyp, nzp=nzp, seed=seed)
    yy, xx = np.mgrid[0:nyp, 0:nxp]
    rel_thick = (1.0 + 0.3 * np.sin(xx / 5.0 + 0.3) * np.cos(yy / 4.0)).astype(np.float32)
    shift = gain = None
    if surfaces:
        rng = np.random.default_rng(seed)
        shift = rng.uniform(-6.0, 6.0, (sc.ntheta, ny, nx)).astype(np.float32)   # ms
        gain = rng.uniform(0.8, 1.25, (sc.ntheta, ny, nx)).astype(np.float32)
    return sc, rel_thick, shift, gain


def _tables(sc):
    from crava_gb300 import api
    lz = sc.nz * sc.dt_ms
    return api.scale_wavelet_tables(sc.wavelets, sc.A, sc.sigma0, sc.circ_corr_t, sc.err_theta_cov, sc.nz,
                                    sc.dt_ms, lz, sc.low_cut, sc.high_cut, sc.wnc), lz


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda() if a is not None else None


@pytest.mark.parametrize("dims", DIMS)
@pytest.mark.parametrize("surfaces", [False, True])
def test_divide_by_scale_wavelet_matches_oracle(cuda, oracle, dims, surfaces):
    from crava_gb300 import api
    nx, ny, nz, nxp, nyp, nzp = dims
    sc, rt, shift, gain = _case(dims, nzp + nx, surfaces)
    tab, lz = _tables(sc)
    cubes = [_dev(d) for d in sc.data]
    nbad = api.divide_by_scale_wavelet(cubes, nx, ny, nz, nxp, _dev(tab), _dev(rt), sc.dt_ms, lz, sc.low_cut,
                                       sc.high_cut, energy_threshold=-1.0, shift=_dev(shift), gain=_dev(gain))
    torch.cuda.synchronize()
    for l in range(sc.ntheta):
        ref = oracle.divide_scale_wavelet(sc.data[l], nx, ny, nz, sc.wavelets[l], sc.A[l], sc.sigma0, sc.circ_corr_t,
                                          sc.dt_ms, lz, sc.low_cut, sc.high_cut, sc.wnc, float(sc.err_theta_cov[l, l]),
                                          rt, None if shift is None else shift[l], None if gain is None else gain[l],
                                          prec="d")
        got = cubes[l].cpu().numpy()
        e = rel(got[:, :, :nxp], ref[:, :, :nxp])
        print(dims, surfaces, l, "divide vs FP64 oracle", e)
        assert e < 2e-5


@pytest.mark.parametrize("dims", DIMS[:2])
def test_divide_then_interpolate_with_dead_traces(cuda, oracle, dims):
    """Dead (all-zero) traces stay exactly zero through the division, so the energy test flags them as
    the reference does; the full step then matches the oracle's divide + interpolate."""
    from crava_gb300 import api
    nx, ny, nz, nxp, nyp, nzp = dims
    sc, rt, shift, gain = _case(dims, 3 * nzp, True)
    tab, lz = _tables(sc)
    data = [d.copy() for d in sc.data]
    dead = [(3, 4), (3, 5), (0, 0), (7, nx - 1), (ny - 1, 10), (8, 8), (9, 8), (8, 9)]
    for d in data:
        for (j, i) in dead:
            d[:, j, i] = 0.0
    cubes = [_dev(d) for d in data]
    nbad = api.divide_by_scale_wavelet(cubes, nx, ny, nz, nxp, _dev(tab), _dev(rt), sc.dt_ms, lz, sc.low_cut,
                                       sc.high_cut, energy_threshold=0.0, shift=_dev(shift), gain=_dev(gain))
    assert nbad == [len(dead)] * sc.ntheta
    for l in range(sc.ntheta):
        ref = oracle.divide_scale_wavelet(data[l], nx, ny, nz, sc.wavelets[l], sc.A[l], sc.sigma0, sc.circ_corr_t,
                                          sc.dt_ms, lz, sc.low_cut, sc.high_cut, sc.wnc, float(sc.err_theta_cov[l, l]),
                                          rt, shift[l], gain[l], prec="d")
        ref, n = oracle.interpolate_seismic(ref, nx, ny, nz, nxp, 0.0, prec="d")
        assert n == len(dead)
        got = cubes[l].cpu().numpy()
        e = rel(got[:, :, :nxp], ref[:, :, :nxp])
        print(dims, l, "divide + interpolate vs FP64 oracle", e)
        assert e < 2e-5


@pytest.mark.parametrize("dims", DIMS)
@pytest.mark.parametrize("threshold", [0.0, 0.3])
def test_interpolate_seismic_bit_exact(cuda, oracle, dims, threshold):
    """Trace energies, the flag scan, the neighbour means and the padding refill reproduce the FP32
    oracle bit for bit (threshold 0.3 also flags live traces, including runs of neighbours)."""
    from crava_gb300 import api
    nx, ny, nz, nxp, nyp, nzp = dims
    rng = np.random.default_rng(nx * ny + int(threshold * 10))
    _, rnxp = api.dims(nxp)
    cube = rng.standard_normal((nzp, nyp, rnxp)).astype(np.float32)
    cube *= rng.uniform(0.2, 1.5, (1, nyp, rnxp)).astype(np.float32)
    for (j, i) in [(2, 3), (2, 4), (2, 5), (0, 0), (ny - 1, nx - 1), (5, 0), (6, 0)]:
        cube[:, j, i] = 0.0
    ref, n_ref = oracle.interpolate_seismic(cube, nx, ny, nz, nxp, threshold, prec="f")
    t = _dev(cube)
    n = api.interpolate_seismic(t, nx, ny, nz, nxp, threshold)
    got = t.cpu().numpy()
    assert n == n_ref
    assert np.array_equal(got[:, :, :nxp], ref[:, :, :nxp]), np.abs(got[:, :, :nxp] - ref[:, :, :nxp]).max()


@pytest.mark.parametrize("dims", DIMS)
@pytest.mark.parametrize("surfaces", [False, True])
def test_multiply_by_scale_wavelet_matches_oracle(cuda, oracle, dims, surfaces):
    from crava_gb300 import api
    nx, ny, nz, nxp, nyp, nzp = dims
    sc, rt, shift, gain = _case(dims, 5 * nzp + 1, surfaces)
    tab, _ = _tables(sc)
    cubes = [_dev(d) for d in sc.data]
    api.multiply_by_scale_wavelet(cubes, nx, ny, nxp, _dev(tab), _dev(rt), sc.dt_ms, shift=_dev(shift),
                                  gain=_dev(gain))
    torch.cuda.synchronize()
    for l in range(sc.ntheta):
        ref = oracle.multiply_scale_wavelet(sc.data[l], nx, ny, sc.wavelets[l], sc.dt_ms, rt,
                                            None if shift is None else shift[l], None if gain is None else gain[l],
                                            prec="d")
        got = cubes[l].cpu().numpy()
        e = rel(got[:, :, :nxp], ref[:, :, :nxp])
        print(dims, surfaces, l, "multiply vs FP64 oracle", e)
        assert e < 2e-5


def test_scale_wavelet_rejects_bad_arguments(cuda):
    from crava_gb300 import api
    sc, rt, _, _ = _case(DIMS[0], 1, False)
    tab, lz = _tables(sc)
    cubes = [_dev(d) for d in sc.data]
    with pytest.raises(RuntimeError):   # nx above nxp
        api.divide_by_scale_wavelet(cubes, 30, sc.ny, sc.nz, sc.nxp, _dev(tab), _dev(rt), sc.dt_ms, lz, sc.low_cut,
                                    sc.high_cut)
    with pytest.raises(RuntimeError):   # 17 cubes
        api.multiply_by_scale_wavelet(cubes * 6, sc.nx, sc.ny, sc.nxp, _dev(tab), _dev(rt), sc.dt_ms)


@pytest.mark.parametrize("form", ["mixed", "plain", "fp32_3pass"])
def test_variable_thickness_inversion_matches_oracle(cuda, oracle, form):
    """A whole inversion on a simbox of non-constant thickness: scale-wavelet division and dead-trace
    interpolation of the data, the non-constant-thickness operator tables, the bin loop, and the residuals
    multiplied back by the scale wavelet, against the FP64 oracle doing the same steps."""
    from dataclasses import replace
    from crava_gb300 import synthetic as S
    from crava_gb300.pipeline import Inversion
    from conftest import oracle_pipeline
    base = S.make_scenario(40, 30, 48, [5.0, 15.0, 25.0, 35.0], 28.0, nxp=48, nyp=36, nzp=60, seed=11)
    sc = S.variable_thickness(base, amp=0.3, surfaces=True, dead_traces=6, seed=4)
    inv = Inversion(sc, forms=(form,))
    inv.restore(form)
    inv.run(form)
    torch.cuda.synchronize()
    assert inv.n_bad == [6] * sc.ntheta
    pm, res, cov = inv.results(form)
    # oracle: the same data steps in FP64, then the inversion with the GPU's operator tables
    lz = sc.nz * sc.dt_ms
    data = []
    for l in range(sc.ntheta):
        d = oracle.divide_scale_wavelet(sc.data[l], sc.nx, sc.ny, sc.nz, sc.wavelets[l], sc.A[l], sc.sigma0,
                                        sc.circ_corr_t, sc.dt_ms, lz, sc.low_cut, sc.high_cut, sc.wnc,
                                        float(sc.err_theta_cov[l, l]), sc.rel_thick, sc.wavelet_shift[l],
                                        sc.wavelet_gain[l], prec="d")
        d, n = oracle.interpolate_seismic(d, sc.nx, sc.ny, sc.nz, sc.nxp, sc.energy_threshold, prec="d")
        assert n == 6
        data.append(d)
    post64, res64, cov64, _ = oracle_pipeline(oracle, replace(sc, data=data), "d", tables=inv.tables)
    prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
    e = (rel(pm, post64), rel(pm - prior, post64 - prior), rel(res, res64), rel(cov, cov64))
    print(form, "variable thickness vs FP64 oracle (mean, update, resid, cov):", e)
    assert e[0] < 1e-6 and e[1] < 1e-4 and e[2] < 1e-4 and e[3] < 1e-4
    # the residuals back in the time domain, multiplied by the scale wavelet
    if form != "plain":
        inv.outputs(form)
        torch.cuda.synchronize()
        r_gpu = np.stack([d[:, :, :sc.nxp].cpu().numpy() for d in inv.data])
        r_ref = []
        for l in range(sc.ntheta):
            spec = res64[l]
            rr = oracle.fft3d_c2r(np.ascontiguousarray(spec), sc.nxp, oracle.DATA, "d")
            rr = oracle.multiply_scale_wavelet(rr, sc.nx, sc.ny, sc.wavelets[l], sc.dt_ms, sc.rel_thick,
                                               sc.wavelet_shift[l], sc.wavelet_gain[l], prec="d")
            r_ref.append(rr[:, :, :sc.nxp])
        er = rel(r_gpu, np.stack(r_ref))
        print(form, "residual output vs oracle", er)
        assert er < 1e-4
