"""C-ABI surface checks that need no GPU: the library loads and exports every
declared symbol, and the host-side set-up code matches the oracle."""
import ctypes as ct

import numpy as np
import pytest

from conftest import rel


def test_library_exports_every_declared_symbol(native):
    from crava_gb300._native import header_symbols
    names = header_symbols()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, missing


def test_version_and_limits(native):
    assert native.cg_version() >= 100
    assert native.cg_fft_max_length() >= 4096


@pytest.mark.parametrize("n", [1, 2, 7, 11, 13, 80, 81, 121, 200, 257, 1000])
def test_find_closest_factorable_matches_oracle(native, oracle, n):
    assert native.cg_find_closest_factorable(n) == oracle.find_closest_factorable(n)


@pytest.mark.parametrize("case", ["inversion_c0small.npz", "inversion_c1small.npz", "inversion_n8odd.npz"])
def test_operator_tables_match_reference_fixture(native, case):
    from conftest import golden
    from crava_gb300 import api
    g = golden(case)
    t = api.operator_tables(g["wavelets"], g["A"], int(g["nz"]), int(g["nzp"]), float(g["dt_ms"]),
                            float(g["low_cut"]), float(g["high_cut"]))
    np.testing.assert_array_equal(t["band"], g["band"])
    for k in ("K", "em1", "em2", "em3"):
        scale = np.abs(g[k]).max()
        assert np.abs(t[k] - g[k]).max() <= 1e-6 * scale, k


def test_host_setup_rejects_bad_arguments(native):
    out = np.zeros(4, np.float32)
    rc = native.cg_operator_tables(0, 4, 8, None, None, 4.0, 1.0, 5.0, 55.0, None, None, None, None, None)
    assert rc == -1
    assert b"bad argument" in native.cg_last_error()
    del out


def test_workspace_rejects_bad_sizes_without_gpu(native):
    h = ct.c_void_p()
    assert native.cg_workspace_create(ct.byref(h), 0, 8, 8, 3) == -1
    assert native.cg_workspace_create(ct.byref(h), 8, 8, 8, 9) == -1
    assert b"ntheta" in native.cg_last_error()


def test_synthetic_scenario_is_seeded():
    from crava_gb300 import synthetic as S
    a = S.make_scenario(8, 6, 10, [10.0, 20.0], 30.0, nxp=10, nyp=8, nzp=12, seed=7)
    b = S.make_scenario(8, 6, 10, [10.0, 20.0], 30.0, nxp=10, nyp=8, nzp=12, seed=7)
    assert all(np.array_equal(x, y) for x, y in zip(a.data, b.data))
    assert rel(a.circ_corr_t, b.circ_corr_t) == 0


def test_circ_corr_t_matches_oracle(oracle):
    from crava_gb300 import synthetic as S
    corr = S.genexp_corr_t(40, 4.0, 20.0, 1.5)
    a = S.circ_corr_t(corr, 2, 64)
    b = oracle.circ_corr_t(corr, 2, 64, prec="d")
    assert rel(a, b) < 1e-6


def test_tuning_table_defaults_overrides_and_validation(native):
    native.cg_tune_clear()
    assert native.cg_tune_get(0, 256) == 3 and native.cg_tune_get(0, 512) == 2   # column-pass CTA target
    assert native.cg_tune_get(2, 5) == 6 and native.cg_tune_get(2, 8) == 1       # bin-kernel register cap
    assert native.cg_tune_set(0, 256, 2) == 0
    assert native.cg_tune_get(0, 256) == 2 and native.cg_tune_get(0, 200) == 3   # per-length entry wins
    assert native.cg_tune_set(1, 0, 0) == 0 and native.cg_tune_get(1, 128) == 0  # n = 0: every length
    assert native.cg_tune_set(0, 256, 7) == -1 and native.cg_tune_set(0, 256, 4) == 0  # resident-CTA targets 2-4
    assert native.cg_tune_set(1, 0, 4) == 0 and native.cg_tune_set(1, 0, 6) == -1  # column kernels 0..5
    assert native.cg_tune_get(3, 128) == 1 and native.cg_tune_set(3, 128, 0) == 0  # x-row kernel 0/1
    assert native.cg_tune_get(3, 128) == 0 and native.cg_tune_set(3, 128, 2) == -1
    assert native.cg_tune_set(9, 1, 1) == -1
    # fused-form y handling: 0 three passes, 1 fused y kernel, an even z-chunk size >= 2 the chunked pipeline
    assert native.cg_tune_get(4, 256) == 0 and native.cg_tune_set(4, 256, 16) == 0 and native.cg_tune_get(4, 256) == 16
    assert native.cg_tune_set(4, 256, 15) == -1 and native.cg_tune_set(4, 256, 8192) == -1
    assert native.cg_tune_set(4, 256, 2) == 0 and native.cg_tune_set(4, 256, 3) == -1   # 2: split y of the means
    assert native.cg_tune_set(2, 5, 5) == 0 and native.cg_tune_set(2, 5, 3) == -1       # bin kernel caps 1, 4-6
    assert native.cg_tune_get(5, 5) == 1 and native.cg_tune_set(5, 5, 0) == 0 and native.cg_tune_set(5, 5, 2) == -1
    native.cg_tune_clear()
    assert native.cg_tune_get(0, 256) == 3
