"""The C++ host layer (FFTGrid / Crava mirror behind cg_inversion_*) with host buffers."""
import numpy as np
import pytest
import torch

from conftest import oracle_pipeline, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form", ["plain", "fp32", "mixed"])
def test_host_buffers_inversion_matches_oracle(cuda, oracle, form):
    from crava_gb300 import api
    from crava_gb300 import synthetic as S
    sc = S.scaled_config1(48, 40, 64, seed=8)
    inv = api.HostInversion(sc)
    data = [d.copy() for d in sc.data]
    mean = [m.copy() for m in sc.mean]
    cov = [np.zeros_like(sc.data[0]) for _ in range(6)]
    kw = {}
    if form == "plain":
        s0 = sc.sigma0.astype(np.float32)
        kw["prior_cov_real"] = [oracle.fill_param_corr(sc.nxp, sc.nyp, sc.nzp, sc.corr_xy, sc.circ_corr_t, 0, 0,
                                                       float(s0[p, q])) for (p, q) in
                                [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]]
        kw["err_corr_real"] = oracle.fill_err_corr(sc.nxp, sc.nyp, sc.nzp, sc.corr_xy)
    inv.run(data, mean, cov, form=form, **kw)
    tables = api.operator_tables(sc.wavelets, sc.A, sc.nz, sc.nzp, sc.dt_ms, sc.low_cut, sc.high_cut)
    post64, res64, cov64, _ = oracle_pipeline(oracle, sc, "d", tables=tables)
    pm = np.stack([m[:, :, :sc.nxp] for m in mean])
    res = np.stack([d.view(np.complex64) for d in data])
    cv = np.stack([c.view(np.complex64) for c in cov])
    prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
    e = (rel(pm, post64), rel(pm - prior, post64 - prior), rel(res, res64), rel(cv, cov64))
    print(form, "host-buffer inversion vs FP64 oracle (mean, update, resid, cov):", e, inv.stats())
    assert e[0] < 1e-6 and e[1] < 1e-4 and e[2] < 1e-4 and e[3] < 1e-4
    # a second call on the same context reuses its device cubes
    data2 = [d.copy() for d in sc.data]
    mean2 = [m.copy() for m in sc.mean]
    inv.run(data2, mean2, cov, form=form, **kw)
    assert rel(np.stack([m[:, :, :sc.nxp] for m in mean2]), pm) < 1e-6


def test_kernel_copy_between_host_and_device(cuda, native):
    """cg_copy moves page-locked host memory with a kernel (no copy engine), both directions."""
    from crava_gb300 import _native
    n = (1 << 20) + 12
    h = torch.randn(n).pin_memory()
    d = torch.empty(n, device="cuda")
    back = torch.zeros(n).pin_memory()
    _native.check(native.cg_copy(d.data_ptr(), h.data_ptr(), n * 4, None), "h2d")
    _native.check(native.cg_copy(back.data_ptr(), d.data_ptr(), n * 4, None), "d2h")
    torch.cuda.synchronize()
    assert torch.equal(d.cpu(), h) and torch.equal(back, h)
    assert native.cg_copy(d.data_ptr() + 4, h.data_ptr(), 64, None) == -1      # misaligned
    assert native.cg_copy(d.data_ptr(), h.data_ptr(), 20, None) == -1          # size not a multiple of 16
    assert native.cg_copy(None, h.data_ptr(), 16, None) == -1
    assert native.cg_host_access() >= 0


def test_submit_wait_pipeline_equals_synchronous_calls(cuda):
    """Two contexts used in turn through cg_inversion_submit_host / cg_inversion_wait (out of place, inputs
    untouched) give bit-identical outputs to one synchronous in-place cg_inversion_run_host per input set."""
    from crava_gb300 import api
    from crava_gb300 import synthetic as S
    scs = [S.scaled_config1(48, 40, 64, seed=s) for s in (11, 12, 13)]
    ctx = [api.HostInversion(scs[0]), api.HostInversion(scs[0])]
    n = scs[0].ntheta
    pinned = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()  # noqa: E731
    ins = [[pinned(x) for x in list(sc.data) + list(sc.mean)] for sc in scs]
    keep = [[x.clone() for x in s] for s in ins]
    outs = [[torch.zeros_like(ins[0][0]).pin_memory() for _ in range(n + 3 + 6)] for _ in scs]
    got = []
    for i, sc in enumerate(scs):
        c = ctx[i % 2]
        if i >= 2:
            c.wait()
            got.append([x.clone() for x in outs[i - 2]])
        c.submit(ins[i][:n], ins[i][n:], outs[i][:n], outs[i][n:n + 3], outs[i][n + 3:], "mixed")
    for i in (1, 2):
        ctx[i % 2].wait()
        got.append([x.clone() for x in outs[i]])
    for i in range(3):
        assert all(torch.equal(a, b) for a, b in zip(ins[i], keep[i])), "inputs must stay untouched"
        data = [x.numpy().copy() for x in keep[i][:n]]
        mean = [x.numpy().copy() for x in keep[i][n:]]
        cov = [np.zeros_like(data[0]) for _ in range(6)]
        ctx[0].run(data, mean, cov, "mixed")
        ref = data + mean + cov
        assert all(np.array_equal(g.numpy(), r) for g, r in zip(got[i], ref)), i
