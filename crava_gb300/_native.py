"""Build and load libcravagpu.so (the sm_103a CUDA library behind include/cravagpu.h).

The library is built in-tree with nvcc (one -gencode, sm_103a only), each
translation unit compiled in parallel.  Loading never falls back to anything:
if the library is missing or fails to load, the caller gets an exception.
"""
from __future__ import annotations

import ctypes as ct
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(PKG, "_build")
LIB_PATH = os.path.join(PKG, "libcravagpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcravagpu.so")


def sources():
    cu = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = []
    if os.path.isdir(HOST):
        cpp = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp"))
    return cu, cpp


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    if os.path.isdir(HOST):
        hs += [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith((".hpp", ".h"))]
    return hs


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile every CUDA/C++ source for sm_103a and link libcravagpu.so."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp = sources()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in cu + cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            if src.endswith(".cu"):
                cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-I" + INCLUDE, "-I" + CSRC, "-c", src, "-o", obj]
            else:
                cmd = [nvcc, "-x", "c++", "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE,
                       "-I" + HOST, "-c", src, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or not os.path.exists(LIB_PATH):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    """The loaded native library; raises if it is not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run crava_gb300.build() (needs nvcc)")
        L = ct.CDLL(LIB_PATH)
        _declare(L)
        _apply_tuning(L)
        _lib = L
    return _lib


TUNING_PATH = os.path.join(PKG, "tuning.json")


def _apply_tuning(L):
    """Load the autotuner's choices (crava_gb300/autotune.py) into the library."""
    if not os.path.exists(TUNING_PATH):
        return
    import json
    try:
        with open(TUNING_PATH) as f:
            t = json.load(f)
        for n, v in t.get("cols", {}).items():
            L.cg_tune_set(1, int(n), int(v["pipe"]))
            L.cg_tune_set(0, int(n), int(v["minb"]))
            L.cg_tune_set(7, int(n), int(v.get("shape", 0)))
        for n, v in t.get("bin", {}).items():
            L.cg_tune_set(2, int(n), int(v["minb"]))
            L.cg_tune_set(8, int(n), int(v.get("runs", 0)))
        for n, v in t.get("rows", {}).items():
            L.cg_tune_set(3, int(n), int(v["kernel"]))
        for n, v in t.get("fused_y", {}).items():
            L.cg_tune_set(4, int(n), int(v["fused"]))
    except (OSError, ValueError, KeyError):
        pass  # a damaged table leaves the built-in defaults


def _declare(L):
    I, V, F, D = ct.c_int, ct.c_void_p, ct.c_float, ct.c_double
    PP = ct.POINTER(ct.c_void_p)
    sig = {
        "cg_last_error": ([], ct.c_char_p),
        "cg_version": ([], I),
        "cg_fft_max_length": ([], I),
        "cg_fft3d_r2c": ([V, I, I, I, I, V], I),
        "cg_fft3d_c2r": ([V, I, I, I, I, V], I),
        "cg_fft3d_r2c_batch": ([PP, I, I, I, I, I, V], I),
        "cg_fft3d_c2r_batch": ([PP, I, I, I, I, I, V], I),
        "cg_fft3d_r2c_f64": ([V, I, I, I, I, V], I),
        "cg_fft3d_c2r_f64": ([V, I, I, I, I, V], I),
        "cg_fft3d_r2c_noalloc": ([V, I, I, I, I, V], I),
        "cg_fft3d_c2r_noalloc": ([V, I, I, I, I, V], I),
        "cg_fft3d_r2c_host": ([V, I, I, I, I], I),
        "cg_fft3d_c2r_host": ([V, I, I, I, I], I),
        "cg_workspace_create": ([ct.POINTER(V), I, I, I, I], I),
        "cg_workspace_destroy": ([V], None),
        "cg_workspace_set_model": ([V, V], I),
        "cg_workspace_set_model_async": ([V, V, V], I),
        "cg_condition_histogram": ([V, V, V, I, V], I),
        "cg_alloc_calls": ([], ct.c_long),
        "cg_vintage4d": ([V, V, V, V, V, V, V, V, V, I, V, V], I),
        "cg_workspace_stats": ([V, ct.POINTER(I), ct.POINTER(I), ct.POINTER(I)], I),
        "cg_workspace_reset_stats": ([V, V], I),
        "cg_invert_bins_plain": ([V, PP, PP, PP, V, V], I),
        "cg_prior_spectra": ([V, V, V, I, V], I),
        "cg_prior_spectra_grad": ([V, V, V, F, F, I, V], I),
        "cg_invert_bins_fused": ([V, PP, PP, PP, I, V], I),
        "cg_invert_cubes_fused": ([V, PP, PP, PP, I, V], I),
        "cg_invert_bins_fused_f64": ([V, PP, PP, PP, V], I),
        "cg_operator_tables": ([I, I, I, V, V, F, F, F, F, V, V, V, V, V], I),
        "cg_find_closest_factorable": ([I], I),
        "cg_fill_param_corr": ([V, I, I, I, V, V, F, F, F, V], I),
        "cg_fill_err_corr": ([V, I, I, I, V, F, F, V], I),
        "cg_posterior_cholesky": ([PP, V, I, I, I, V, V], I),
        "cg_simulate_fields": ([V, PP, PP, I, I, ct.c_uint64, I, I, I, PP, V], I),
        "cg_state4d_merge": ([PP, PP, PP, PP, PP, PP, PP, I, I, I, V], I),
        "cg_state4d_split": ([PP, PP, PP, PP, PP, PP, PP, I, I, I, V, V], I),
        "cg_state4d_evolve": ([PP, PP, PP, PP, PP, V, V, V, V, I, I, I, V], I),
        "cg_fill_genexp_corr": ([V, I, I, I, ct.c_double, ct.c_double, ct.c_double, F, F, V], I),
        "cg_scale": ([V, ct.c_long, F, V], I),
        "cg_add": ([V, V, ct.c_long, V], I),
        "cg_host_register": ([V, ct.c_size_t], I),
        "cg_copy": ([V, V, ct.c_size_t, V], I),
        "cg_exp_transform": ([V, ct.c_long, V], I),
        "cg_fill_in_data": ([V, I, I, I, I, I, V, I, V, V, V, V, F, F, V, V], I),
        "cg_operator_tables_ex": ([I, I, I, V, V, F, F, F, F, I, V, V, V, V, V], I),
        "cg_scale_wavelet_table_size": ([I], I),
        "cg_scale_wavelet_tables": ([I, I, I, V, V, V, V, V, F, F, F, F, F, V], I),
        "cg_divide_by_scale_wavelet": ([PP, I, I, I, I, I, I, I, V, V, V, V, F, F, F, F, F, V, V], I),
        "cg_multiply_by_scale_wavelet": ([PP, I, I, I, I, I, I, V, V, V, V, F, V], I),
        "cg_interpolate_seismic": ([V, I, I, I, I, I, I, F, V, V], I),
        "cg_correct_alpha_beta_rho": ([PP, PP, I, I, I, I, I, I, I, V, V, V, V, V, V, V], I),
        "cg_apply_trace_matrices": ([PP, PP, V, I, I, I, I, I, I, V], I),
        "cg_crava_file_write": ([ct.c_char_p, V, I, I, I, V, V], I),
        "cg_crava_file_read": ([ct.c_char_p, V, I, I, I, V, V], I),
        "cg_storm_write": ([ct.c_char_p, V, I, I, I, V], I),
        "cg_storm_read_header": ([ct.c_char_p, V, V, V, V], I),
        "cg_storm_read": ([ct.c_char_p, V, ct.c_long], I),
        "cg_storm_surface_write": ([ct.c_char_p, V, I, I, ct.c_double, ct.c_double, ct.c_double, ct.c_double], I),
        "cg_storm_surface_read_header": ([ct.c_char_p, V, V, V, V, V, V], I),
        "cg_storm_surface_read": ([ct.c_char_p, V, ct.c_long], I),
        "cg_log_transform": ([V, ct.c_long, V], I),
        "cg_fft3d_c2r_exp_batch": ([PP, I, I, I, I, I, V], I),
        "cg_cov_origin": ([PP, I, I, I, I, V, V, V], I),
        "cg_host_access": ([], I),
        "cg_host_unregister": ([V], I),
        "cg_inversion_create": ([ct.POINTER(V), I, I, I, I, I, I, V], I),
        "cg_inversion_destroy": ([V], None),
        "cg_inversion_run_host": ([V, PP, PP, PP, PP, V, I], I),
        "cg_inversion_submit_host": ([V, PP, PP, PP, PP, PP, PP, V, I], I),
        "cg_inversion_wait": ([V], I),
        "cg_inversion_stats": ([V, ct.POINTER(I), ct.POINTER(I), ct.POINTER(I)], I),
        "cg_batch_create": ([ct.POINTER(V), V, I, I], I),
        "cg_batch_destroy": ([V], None),
        "cg_batch_load": ([V, I, PP, PP], I),
        "cg_batch_reset": ([V, V], I),
        "cg_batch_run": ([V, I, I, V], I),
        "cg_batch_read": ([V, I, PP, PP, PP], I),
        "cg_batch_set_simulation": ([V, I, I, ct.c_ulonglong], I),
        "cg_batch_read_fields": ([V, I, I, PP], I),
        "cg_batch_bins": ([V], ct.c_long),
        "cg_tune_set": ([I, I, I], I),
        "cg_tune_get": ([I, I], I),
        "cg_tune_clear": ([], I),
        "cg_trace_enable": ([I], I),
        "cg_device_faults": ([ct.POINTER(I)], I),
        "cg_trace_collect": ([], I),
        "cg_trace_entry": ([I, ct.c_char_p, I, ct.POINTER(ct.c_long), ct.POINTER(D), ct.POINTER(D)], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name, None)
        if f is None:
            continue
        f.argtypes = args
        f.restype = res
    _ = (F, D)


def check(rc: int, what: str = ""):
    if rc != 0:
        msg = lib().cg_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed with status {rc}: {msg}")


def header_symbols() -> list[str]:
    """Function names declared in include/cravagpu.h."""
    import re
    names = []
    for fn in sorted(os.listdir(INCLUDE)):
        if not fn.endswith(".h"):
            continue
        txt = open(os.path.join(INCLUDE, fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(?:int|void|const char\s*\*)\s*\**\s*(cg_\w+)\s*\(", txt):
            names.append(m.group(1))
    return sorted(set(names))


def trace_enable(on: bool = True):
    check(lib().cg_trace_enable(1 if on else 0), "cg_trace_enable")


def device_faults() -> int:
    """1 when a kernel's bounded wait gave up since the last call (the word is cleared), else 0."""
    v = ct.c_int(0)
    check(lib().cg_device_faults(ct.byref(v)), "cg_device_faults")
    return v.value


def trace_collect():
    """{kernel name: (launches, total ms, total algorithmic bytes)} since trace_enable."""
    L = lib()
    n = L.cg_trace_collect()
    if n < 0:
        check(n, "cg_trace_collect")
    out = {}
    for i in range(n):
        buf = ct.create_string_buffer(128)
        la, ms, by = ct.c_long(), ct.c_double(), ct.c_double()
        check(L.cg_trace_entry(i, buf, 128, ct.byref(la), ct.byref(ms), ct.byref(by)), "cg_trace_entry")
        out[buf.value.decode()] = (la.value, ms.value, by.value)
    return out
