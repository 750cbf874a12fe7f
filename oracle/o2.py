"""Driver of oracle/_ref/crava_o2, the harness around the reference's own
compiled Crava / Wavelet / SeismicParametersHolder / State4D classes -- TEST
INFRASTRUCTURE ONLY.  tests/golden/make_golden.py calls it where the
reference checkout exists (CRAVA_REFERENCE_SRC) to write golden fixtures;
the tests read the fixtures, never this module.

Each call writes the inputs as raw little-endian arrays plus a params.txt
into a scratch directory, runs ``crava_o2 <command> <dir>`` and reads the
outputs back (oracle/o2_harness.cpp documents every file).
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
O2_EXE = os.path.join(HERE, "_ref", "crava_o2")


def build(reference_src: str) -> str:
    subprocess.check_call(["make", "-s", "-f", os.path.join(HERE, "Makefile.o2"), f"REF={reference_src}",
                           f"-j{os.cpu_count() or 4}"], cwd=os.path.dirname(HERE))
    return O2_EXE


def _run(cmd, d):
    r = subprocess.run([O2_EXE, cmd, d], cwd=d, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"crava_o2 {cmd} failed ({r.returncode}): {r.stderr[-2000:]}")


def _params(d, **kw):
    with open(os.path.join(d, "params.txt"), "w") as f:
        for k, v in kw.items():
            f.write(f"{k} {v!r}\n")


def _w(d, name, arr, dt):
    np.ascontiguousarray(arr, dtype=dt).tofile(os.path.join(d, name))


def _r(d, name, dt, shape=None):
    a = np.fromfile(os.path.join(d, name), dtype=dt)
    return a.reshape(shape) if shape is not None else a


def inversion(sc, corr_t, min_int_fq, f_peak, wavelets=None):
    """Crava::computePostMeanResidAndFFTCov on the scenario's data and prior means, with the reference's
    own Ricker wavelets (peak frequency f_peak; or, when ``wavelets`` (n, nzp) is given, those resampled
    samples in the reference's Wavelet objects) and prior/error correlation cubes built from corr_xy and
    the temporal correlation corr_t.  Returns the reference's intermediate and final arrays (complex
    spectra as (nzp, nyp, cnxp) complex64, real cubes as (nzp, nyp, rnxp) float32)."""
    n, nxp, nyp, nzp = sc.ntheta, sc.nxp, sc.nyp, sc.nzp
    cnxp, rnxp = nxp // 2 + 1, 2 * (nxp // 2 + 1)
    shape = (nzp, nyp, rnxp)
    with tempfile.TemporaryDirectory() as d:
        _params(d, nx=sc.nx, ny=sc.ny, nz=sc.nz, nxp=nxp, nyp=nyp, nzp=nzp, ntheta=n, ncorrt=len(corr_t),
                min_int_fq=int(min_int_fq), dt=float(sc.dt_ms), fpeak=float(f_peak), low_cut=float(sc.low_cut),
                high_cut=float(sc.high_cut), wnc=float(sc.wnc), given_wavelets=int(wavelets is not None),
                grad_i=float(np.float32(getattr(sc, "corr_grad", (0.0, 0.0))[0])),
                grad_j=float(np.float32(getattr(sc, "corr_grad", (0.0, 0.0))[1])))
        if wavelets is not None:
            _w(d, "wavelets_in.f32", wavelets, np.float32)
        _w(d, "theta.f32", sc.theta_deg, np.float32)
        _w(d, "A.f32", sc.A, np.float32)
        _w(d, "etc.f64", sc.err_theta_cov, np.float64)
        _w(d, "sigma0.f32", np.asarray(sc.sigma0, dtype=np.float64).astype(np.float32), np.float32)
        _w(d, "corrxy.f64", np.asarray(sc.corr_xy, dtype=np.float32).astype(np.float64), np.float64)
        _w(d, "corrt.f32", corr_t, np.float32)
        _w(d, "data.f32", np.stack(sc.data), np.float32)
        _w(d, "mean.f32", np.stack(sc.mean), np.float32)
        _run("inversion", d)
        spec = lambda a: a.view(np.complex64).reshape((nzp, nyp, cnxp))  # noqa: E731
        out = _r(d, "output.f32", np.float32, (3 + n + 6,) + shape)
        inp = _r(d, "input_spectra.f32", np.float32, (n + 3,) + shape)
        res = {
            "wavelets": _r(d, "wavelets.f32", np.float32, (n, nzp)),
            "wavelet_norms": _r(d, "wavelet_norms.f32", np.float32),
            "circ_corr_t": _r(d, "circcorrt.f32", np.float32),
            "prior_cov_real": _r(d, "prior_cov_real.f32", np.float32, (6,) + shape),
            "errcorr_real": _r(d, "errcorr_real.f32", np.float32, shape),
            "errcorr_spec": spec(_r(d, "errcorr_spec.f32", np.float32, shape)),
            "data_spec": np.stack([spec(x) for x in inp[:n]]),
            "mean_spec": np.stack([spec(x) for x in inp[n:]]),
            "out_mean_real": out[:3],
            "out_resid": np.stack([spec(x) for x in out[3:3 + n]]),
            "out_cov": np.stack([spec(x) for x in out[3 + n:]]),
        }
        for sfx in ("", "_nct"):
            res["K" + sfx] = _r(d, f"K{sfx}.f32", np.float32).view(np.complex64).reshape(nzp, n, 3)
            for e in ("em1", "em2", "em3"):
                res[e + sfx] = _r(d, f"{e}{sfx}.f32", np.float32).view(np.complex64).reshape(nzp, n)
            res["band" + sfx] = _r(d, f"band{sfx}.u8", np.uint8)
    return res


def state4d(state27, post9, nxp):
    """State4D::merge then State4D::split.  state27: the 27 state spectra (mu_s 3, mu_d 3, static-static 6,
    static-dynamic 9, dynamic-dynamic 6), post9: the current state's posterior (mean 3, covariance in the
    order 00 01 02 11 12 22), all (nzp, nyp, cnxp) complex64.  Returns (merged 9 spectra, split 27)."""
    state27 = np.ascontiguousarray(state27, dtype=np.complex64)
    post9 = np.ascontiguousarray(post9, dtype=np.complex64)
    nzp, nyp, cnxp = state27.shape[1:]
    with tempfile.TemporaryDirectory() as d:
        _params(d, nxp=nxp, nyp=nyp, nzp=nzp)
        _w(d, "state.f32", state27.view(np.float32), np.float32)
        _w(d, "post.f32", post9.view(np.float32), np.float32)
        _run("state4d", d)
        merged = _r(d, "merged.f32", np.float32).view(np.complex64).reshape(9, nzp, nyp, cnxp)
        split = _r(d, "split.f32", np.float32).view(np.complex64).reshape(27, nzp, nyp, cnxp)
    return merged, split


def state4d_evolve(state27, nx, ny, nz, nxp, E, c, C):
    """State4D::evolve with one time step (E, C (6, 6), c (6,)) on the 27 state spectra ((nzp, nyp, cnxp)
    complex64; grids of logical size nx x ny x nz).  Returns (evolved 27 spectra, the increment correlation
    cube (nzp, nyp, rnxp) as fillInGenExpCorr writes it, and its transform)."""
    state27 = np.ascontiguousarray(state27, dtype=np.complex64)
    nzp, nyp, cnxp = state27.shape[1:]
    with tempfile.TemporaryDirectory() as d:
        _params(d, nx=nx, ny=ny, nz=nz, nxp=nxp, nyp=nyp, nzp=nzp)
        _w(d, "state.f32", state27.view(np.float32), np.float32)
        _w(d, "E.f64", E, np.float64)
        _w(d, "c.f64", c, np.float64)
        _w(d, "C.f64", C, np.float64)
        _run("state4d_evolve", d)
        ev = _r(d, "evolved.f32", np.float32).view(np.complex64).reshape(27, nzp, nyp, cnxp)
        gr = _r(d, "genexp_real.f32", np.float32).reshape(nzp, nyp, 2 * cnxp)
        gs = _r(d, "genexp_spec.f32", np.float32).view(np.complex64).reshape(nzp, nyp, cnxp)
    return ev, gr, gs


def adjustment(sc, l, corr_t, min_int_fq, f_peak, cases, error_var):
    """Crava::computeAdjustmentFactor for angle l of the scenario: the reference's Ricker (f_peak) resampled
    on the grid is the global wavelet; cases: (n, 3) of (time shift ms, gain, stretch).  Returns (the
    global wavelet samples, the filtered temporal correlation it used, (n, nzp/2+1) complex factors)."""
    cases = np.ascontiguousarray(cases, dtype=np.float32)
    nzp = sc.nzp
    with tempfile.TemporaryDirectory() as d:
        _params(d, nx=sc.nx, ny=sc.ny, nz=sc.nz, nxp=sc.nxp, nyp=sc.nyp, nzp=nzp, ncases=len(cases),
                ncorrt=len(corr_t), min_int_fq=int(min_int_fq), dt=float(sc.dt_ms), fpeak=float(f_peak),
                theta=float(sc.theta_deg[l]), error_var=float(error_var), low_cut=float(sc.low_cut),
                high_cut=float(sc.high_cut), wnc=float(sc.wnc))
        _w(d, "A.f32", sc.A[l], np.float32)
        _w(d, "sigma0.f32", np.asarray(sc.sigma0, dtype=np.float64).astype(np.float32), np.float32)
        _w(d, "corrxy.f64", np.asarray(sc.corr_xy, dtype=np.float32).astype(np.float64), np.float64)
        _w(d, "corrt.f32", corr_t, np.float32)
        _w(d, "cases.f32", cases, np.float32)
        _run("adjust", d)
        wav = _r(d, "wavelet.f32", np.float32)
        ct_f = _r(d, "corrt_filtered.f32", np.float32)
        adj = _r(d, "adjust.f32", np.float32).view(np.complex64).reshape(len(cases), nzp // 2 + 1)
    return wav, ct_f, adj


def local_noise(post, mean, nx, ny, nz, nxp, err_theta_cov, prior_var0, post_var0, scale):
    """Crava::computeG and Crava::correctAlphaBetaRho: post, mean 3 real padded cubes (nzp, nyp, rnxp) each,
    scale (ntheta, ny, nx) local noise scales.  Returns (G (ntheta, 3), the 3 corrected posterior cubes)."""
    n = len(err_theta_cov)
    nzp, nyp, rnxp = post[0].shape
    with tempfile.TemporaryDirectory() as d:
        _params(d, nx=nx, ny=ny, nz=nz, nxp=nxp, nyp=nyp, nzp=nzp, ntheta=n)
        _w(d, "etc.f64", err_theta_cov, np.float64)
        _w(d, "priorvar0.f64", prior_var0, np.float64)
        _w(d, "postvar0.f64", post_var0, np.float64)
        _w(d, "scale.f64", scale, np.float64)
        _w(d, "post.f32", np.stack(post), np.float32)
        _w(d, "mean.f32", np.stack(mean), np.float32)
        _run("localnoise", d)
        G = _r(d, "G.f64", np.float64, (n, 3))
        out = [_r(d, f"post_{q}.f32", np.float32, (nzp, nyp, rnxp)) for q in ("alpha", "beta", "rho")]
    return G, out


def fill_in_data(values, gbox, nx, ny, nz, nxp, nyp, nzp, sbox, cubetype, smooth_length):
    """FFTGrid::fillInData from a STORM grid: values (gnk, gny, gnx) on the box gbox = (gx0, gy0, gz0, glx, gly,
    glz), a constant-thickness simbox sbox = (x0, y0, z0, lx, ly, lz, rot, dx, dy, dz).  Returns (the filled cube
    (nzp, nyp, rnxp), per-column traces (ncol, gnk), state (ncol,), z0_data, dz_data, z0_grid, dz_grid (ncol,),
    the three missing/dead counts)."""
    gnk, gny, gnx = values.shape
    rnxp = 2 * (nxp // 2 + 1)
    ncol = rnxp * nyp
    gx0, gy0, gz0, glx, gly, glz = gbox
    x0, y0, z0, lx, ly, lz, rot, dx, dy, dz = sbox
    with tempfile.TemporaryDirectory() as d:
        _params(d, nx=nx, ny=ny, nz=nz, nxp=nxp, nyp=nyp, nzp=nzp, gnx=gnx, gny=gny, gnk=gnk, cubetype=int(cubetype),
                smooth_length=float(smooth_length), gx0=float(gx0), gy0=float(gy0), gz0=float(gz0), glx=float(glx),
                gly=float(gly), glz=float(glz), x0=float(x0), y0=float(y0), z0=float(z0), lx=float(lx),
                ly=float(ly), lz=float(lz), rot=float(rot), dx=float(dx), dy=float(dy), dz=float(dz))
        _w(d, "grid.f32", values, np.float32)
        _run("fillindata", d)
        cube = _r(d, "cube.f32", np.float32, (nzp, nyp, rnxp))
        traces = _r(d, "traces.f32", np.float32, (ncol, gnk))
        state = _r(d, "state.i32", np.int32)
        cols = [_r(d, f, np.float32) for f in ("z0_data.f32", "dz_data.f32", "z0_grid.f32", "dz_grid.f32")]
        counts = _r(d, "counts.i32", np.int32)
    return (cube, traces, state, *cols, counts)


def divide_scale_wavelet(sc, corr_t, min_int_fq, f_peak, thick_nodes, shift, gain, energy_threshold, dx=25.0, dy=25.0,
                         z0=1000.0):
    """Crava::divideDataByScaleWavelet on the scenario's DATA cubes over a simbox whose bottom is
    z0 + lz * thick_nodes (nj, ni nodes over the simbox area); shift, gain (ntheta, ny, nx).  Returns (the divided
    cubes, the relative thickness at every padded trace (nyp, nxp), the simbox lz, the reference's resampled
    wavelets (ntheta, nzp) and gain grids (ntheta, ny, nx) after Wavelet::setGainGrid, the filtered temporal
    correlation)."""
    n, nzp = sc.ntheta, sc.nzp
    nj, ni = thick_nodes.shape
    with tempfile.TemporaryDirectory() as d:
        _params(d, nx=sc.nx, ny=sc.ny, nz=sc.nz, nxp=sc.nxp, nyp=sc.nyp, nzp=nzp, ntheta=n, ncorrt=len(corr_t),
                min_int_fq=int(min_int_fq), dt=float(sc.dt_ms), fpeak=float(f_peak), low_cut=float(sc.low_cut),
                high_cut=float(sc.high_cut), wnc=float(sc.wnc), energy_threshold=float(energy_threshold), ni=ni,
                nj=nj, dx=float(dx), dy=float(dy), z0=float(z0))
        _w(d, "theta.f32", sc.theta_deg, np.float32)
        _w(d, "A.f32", sc.A, np.float32)
        _w(d, "etc.f64", sc.err_theta_cov, np.float64)
        _w(d, "sigma0.f32", np.asarray(sc.sigma0, dtype=np.float64).astype(np.float32), np.float32)
        _w(d, "corrxy.f64", np.asarray(sc.corr_xy, dtype=np.float32).astype(np.float64), np.float64)
        _w(d, "corrt.f32", corr_t, np.float32)
        _w(d, "data.f32", np.stack(sc.data), np.float32)
        _w(d, "thick.f64", thick_nodes, np.float64)
        _w(d, "shift.f32", shift, np.float32)
        _w(d, "gain.f32", gain, np.float32)
        _run("divide", d)
        shp = sc.data[0].shape
        out = [_r(d, f"out{l}.f32", np.float32, shp) for l in range(n)]
        rel = _r(d, "relthick.f64", np.float64, (sc.nyp, sc.nxp))
        lz = float(_r(d, "lz.f64", np.float64)[0])
        wav = _r(d, "wavelets.f32", np.float32, (n, nzp))
        gn = _r(d, "gain_normalised.f32", np.float32, (n, sc.ny, sc.nx))
        ctf = _r(d, "corrt_filtered.f32", np.float32)
        mult = [_r(d, f"mult{l}.f32", np.float32, shp) for l in range(n)]
    return out, rel, lz, wav, gn, ctf, mult


def interpolate_seismic(cube, nx, ny, nz, nxp, threshold):
    """FFTGrid::interpolateSeismic on a real padded DATA cube (nzp, nyp, rnxp); returns the result."""
    nzp, nyp, rnxp = cube.shape
    with tempfile.TemporaryDirectory() as d:
        _params(d, nx=nx, ny=ny, nz=nz, nxp=nxp, nyp=nyp, nzp=nzp, threshold=float(threshold))
        _w(d, "cube.f32", cube, np.float32)
        _run("interpolate", d)
        return _r(d, "out.f32", np.float32, (nzp, nyp, rnxp))


CRAVA_GEOM = ("x0", "y0", "dx", "dy", "il0", "xl0", "ilstepx", "ilstepy", "xlstepx", "xlstepy", "angle")


def crava_write(cube, nx, ny, nxp, geom):
    """FFTGrid::writeCravaFile of the padded real cube (nzp, nyp, rnxp) with simbox geometry geom (the 11
    values of CRAVA_GEOM); returns the file's bytes."""
    nzp, nyp, _ = cube.shape
    with tempfile.TemporaryDirectory() as d:
        _params(d, nx=nx, ny=ny, nxp=nxp, nyp=nyp, nzp=nzp, **dict(zip(CRAVA_GEOM, [float(g) for g in geom])))
        _w(d, "cube.f32", cube, np.float32)
        _run("crava_write", d)
        with open(os.path.join(d, "out.crava"), "rb") as f:
            return f.read()


def crava_read(raw, nxp, nyp, nzp):
    """FFTGrid::readCravaFile of the bytes raw into a grid of padded size nxp x nyp x nzp: the cube, or the
    reference's error text when the sizes disagree."""
    rnxp = 2 * (nxp // 2 + 1)
    with tempfile.TemporaryDirectory() as d:
        _params(d, nxp=nxp, nyp=nyp, nzp=nzp)
        with open(os.path.join(d, "in.crava"), "wb") as f:
            f.write(raw)
        _run("crava_read", d)
        if os.path.exists(os.path.join(d, "error.txt")):
            with open(os.path.join(d, "error.txt")) as f:
                return f.read()
        return _r(d, "cube_read.f32", np.float32, (nzp, nyp, rnxp))


STORM_PARAMS = ("zone", "missing", "x_min", "lx", "y_min", "ly", "z_top", "z_bot", "erosion_top", "erosion_bot",
                "angle_deg")


def storm_write(values, **hdr):
    """NRLib::StormContGrid::WriteToFile of values (nk, nj, ni) with constant surfaces, model file name
    "ModelFile" and variable name "Vp"; returns the file's bytes."""
    nk, nj, ni = values.shape
    with tempfile.TemporaryDirectory() as d:
        _params(d, ni=ni, nj=nj, nk=nk, **{k: float(hdr[k]) for k in STORM_PARAMS})
        _w(d, "values.f32", values, np.float32)
        _run("storm_write", d)
        with open(os.path.join(d, "out.storm"), "rb") as f:
            return f.read()


def storm_read(raw):
    """NRLib::StormContGrid::ReadFromFile of the bytes raw: (values (nk, nj, ni), header dict)."""
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "in.storm"), "wb") as f:
            f.write(raw)
        _run("storm_read", d)
        hdr = {}
        with open(os.path.join(d, "header.txt")) as f:
            for line in f:
                k, v = line.split()
                hdr[k] = float(v)
        v = _r(d, "values_read.f32", np.float32)
        return v.reshape(int(hdr["nk"]), int(hdr["nj"]), int(hdr["ni"])), hdr


def storm_write_surf(values, top, bot, surf_geom, **hdr):
    """StormContGrid::WriteToFile with regular top / bottom surfaces top, bot (nj, ni) float64 over surf_geom
    (x_min, y_min, lx, ly): returns {file name: bytes} for the grid and the surface files beside it."""
    nk, nj, ni = values.shape
    snj, sni = top.shape
    with tempfile.TemporaryDirectory() as d:
        _params(d, ni=ni, nj=nj, nk=nk, surf_ni=sni, surf_nj=snj, sx_min=float(surf_geom[0]),
                sy_min=float(surf_geom[1]), slx=float(surf_geom[2]), sly=float(surf_geom[3]),
                **{k: float(hdr[k]) for k in STORM_PARAMS if k not in ("z_top", "z_bot")})
        _w(d, "values.f32", values, np.float32)
        _w(d, "top.f64", top, np.float64)
        _w(d, "bot.f64", bot, np.float64)
        _run("storm_write_surf", d)
        out = {}
        for name in sorted(os.listdir(d)):
            if name.startswith("out.storm"):
                with open(os.path.join(d, name), "rb") as f:
                    out[name] = f.read()
        return out


def storm_read_surf(files):
    """StormContGrid::ReadFromFile of files["in.storm"] with its surface files beside it (files: {name: bytes}):
    (values (nk, nj, ni), {"top"/"bot": (z (nj, ni), geometry (ni, nj, x_min, y_min, lx, ly))})."""
    with tempfile.TemporaryDirectory() as d:
        for name, raw in files.items():
            with open(os.path.join(d, name), "wb") as f:
                f.write(raw)
        _run("storm_read_surf", d)
        surf = {}
        for q in ("top", "bot"):
            g = _r(d, f"{q}_geom.f64", np.float64)
            surf[q] = (_r(d, f"{q}_read.f64", np.float64).reshape(int(g[1]), int(g[0])), g)
        v = _r(d, "values_read.f32", np.float32)
    return v, surf


def closest_factorable(ns):
    ns = np.asarray(ns, dtype=np.int32)
    with tempfile.TemporaryDirectory() as d:
        _params(d, count=len(ns))
        _w(d, "n.i32", ns, np.int32)
        _run("factorable", d)
        return _r(d, "factorable.i32", np.int32)
