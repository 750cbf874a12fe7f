"""File formats either side of the path (host code, no GPU): CRAVA FFTGrid binary and STORM binary grids."""
import struct

import numpy as np
import pytest


def test_crava_file_round_trip_and_layout(native, tmp_path):
    from crava_gb300 import api
    nxp, nyp, nzp = 10, 6, 4
    _, rnxp = api.dims(nxp)
    rng = np.random.default_rng(1)
    cube = rng.standard_normal((nzp, nyp, rnxp)).astype(np.float32)
    geom = [1000.5, 2000.25, 25.0, 12.5, 100.0, 200.0, 0.5, -0.5, 0.25, 0.75, 0.1]
    p = tmp_path / "grid.crava"
    api.write_crava_file(p, cube, geom, 8, 5)
    raw = p.read_bytes()
    tag = b"crava_fftgrid_binary\n"
    assert raw.startswith(tag)
    # big-endian doubles and ints in FFTGrid::writeCravaFile order
    x0, y0, dx, dy, nx, ny = struct.unpack(">4d2i", raw[len(tag):len(tag) + 40])
    assert (x0, y0, dx, dy, nx, ny) == (1000.5, 2000.25, 25.0, 12.5, 8, 5)
    off = len(tag) + 40 + 7 * 8
    assert struct.unpack(">3i", raw[off:off + 12]) == (rnxp, nyp, nzp)
    data = np.frombuffer(raw[off + 12:], dtype=">f4")
    assert data.size == cube.size and np.array_equal(data.astype(np.float32), cube.reshape(-1))
    back, g, n = api.read_crava_file(p, nxp, nyp, nzp)
    assert np.array_equal(back, cube) and list(g) == geom and n == (8, 5)
    with pytest.raises(RuntimeError, match="padding"):
        api.read_crava_file(p, nxp + 2, nyp, nzp)


def _header(**kw):
    from crava_gb300 import api
    h = api.StormHeader()
    h.zone_number = 0
    h.model_file = b"ModelFile"
    h.missing_code = -999.25
    h.variable = b"Vp"
    h.x_min, h.lx, h.y_min, h.ly = 456000.0, 1600.0, 6780000.0, 1200.0
    h.z_top, h.z_bot, h.erosion_top, h.erosion_bot = 1800.0, 2400.0, 1800.0, 2400.0
    h.lz, h.angle_deg = 600.0, 30.0
    for k, v in kw.items():
        setattr(h, k, v)
    return h


def test_storm_round_trip_and_header_text(native, tmp_path):
    from crava_gb300 import api
    rng = np.random.default_rng(2)
    v = rng.standard_normal((5, 4, 3)).astype(np.float32)
    p = tmp_path / "vp.storm"
    api.write_storm(p, v, _header())
    raw = p.read_bytes()
    head = (b"storm_petro_binary\n\n0 ModelFile -999.25\n\nVp\n\n456000 1600 6780000 1200 1800 2400 1800 2400\n"
            b"600 30\n\n3 4 5\n")
    assert raw.startswith(head)
    body = raw[len(head):]
    assert body[-1:] == b"0" and len(body) == 4 * v.size + 1
    assert np.array_equal(np.frombuffer(body[:-1], dtype=">f4").astype(np.float32), v.reshape(-1))
    back, h = api.read_storm(p)
    assert np.array_equal(back, v)
    assert h.variable == b"Vp" and h.lx == 1600.0 and h.angle_deg == 30.0 and h.missing_code == np.float32(-999.25)


def test_storm_unsupported_forms(native, tmp_path):
    from crava_gb300 import api
    # a surface given as a file keeps its name; a surface file that is not STORM binary is refused
    p = tmp_path / "surf.storm"
    p.write_bytes(b"storm_petro_binary\n\n0 ModelFile -999\n\nVp\n\n0 100 0 100 top.irap 2400 1800 2400\n600 0\n\n1 1 1\n"
                  + struct.pack(">f", 1.0) + b"0")
    v, h = api.read_storm(p)
    assert h.z_top_file == b"top.irap" and h.z_bot == 2400.0 and v.shape == (1, 1, 1)
    (tmp_path / "top.irap").write_bytes(b"-996 2 50 50\n0 100 0 100\n")
    with pytest.raises(RuntimeError, match="not a STORM binary surface"):
        api.read_storm_surfaces(p, h)
    q = tmp_path / "ascii.storm"
    q.write_bytes(b"storm_petro_ascii\n\n0 ModelFile -999\n")
    with pytest.raises(RuntimeError, match="ASCII"):
        api.read_storm(q)


def test_storm_surface_round_trip_and_checks(native, tmp_path):
    from crava_gb300 import api
    rng = np.random.default_rng(3)
    z = rng.uniform(1000, 2000, (5, 7))
    p = tmp_path / "s.storm_top"
    api.write_storm_surface(p, api.StormSurface(z, 100.0, 200.0, 60.0, 40.0))
    raw = p.read_bytes()
    assert raw.startswith(b"STORMGRID_BINARY\n\n7 5 10 10\n100 160 200 240\n")
    assert len(raw) == len(b"STORMGRID_BINARY\n\n7 5 10 10\n100 160 200 240\n") + 8 * z.size
    s = api.read_storm_surface(p)
    np.testing.assert_array_equal(s.z, z)
    assert (s.x_min, s.y_min, s.lx, s.ly) == (100.0, 200.0, 60.0, 40.0)
    # inconsistent spacing, trailing bytes and a truncated body are refused as the reference refuses them
    bad = raw.replace(b"7 5 10 10", b"7 5 11 10")
    (tmp_path / "b1").write_bytes(bad)
    with pytest.raises(RuntimeError, match="dx"):
        api.read_storm_surface(tmp_path / "b1")
    (tmp_path / "b2").write_bytes(raw + b"x")
    with pytest.raises(RuntimeError, match="too long"):
        api.read_storm_surface(tmp_path / "b2")
    (tmp_path / "b3").write_bytes(raw[:-8])
    with pytest.raises(RuntimeError, match="truncated"):
        api.read_storm_surface(tmp_path / "b3")
