"""Batched uneven inversions (cg_batch_*): per-cube results, graph replay, oracle parity."""
import numpy as np
import pytest

from conftest import oracle_pipeline, rel

pytestmark = pytest.mark.gpu


def _scenarios():
    from crava_gb300 import synthetic as S
    # uneven sizes, stack counts and physics; 90/75/35 exercise the generic transform kernels
    return [
        S.make_scenario(40, 36, 70, [0.0, 20.0], 30.0, nxp=48, nyp=45, nzp=90, sn=3.0, seed=31),
        S.make_scenario(60, 50, 60, [0.0, 10.0, 20.0, 30.0], 20.0, nxp=80, nyp=64, nzp=75, sn=5.0, seed=32),
        S.make_scenario(20, 28, 30, [5.0, 15.0, 25.0, 35.0, 40.0, 45.0, 50.0], 40.0, nxp=27, nyp=35, nzp=40,
                        sn=2.5, std_scale=1.3, seed=33),
        S.make_scenario(100, 80, 100, [10.0, 20.0, 30.0], 25.0, nxp=128, nyp=100, nzp=128, sn=4.0, seed=34),
    ]


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_matches_single_cube_inversions(cuda, use_graph):
    from crava_gb300 import api
    scs = _scenarios()
    b = api.Batch(scs, nstreams=3)
    assert b.bins == sum(sc.nbins for sc in scs)
    outs = []
    for rep in range(2):  # a replay must give the same answer as the first run
        b.reset()
        b.run("mixed", use_graph=use_graph)
        outs.append([b.read(i) for i in range(len(scs))])
    for i, sc in enumerate(scs):
        inv = api.HostInversion(sc)
        data = [d.copy() for d in sc.data]
        mean = [m.copy() for m in sc.mean]
        cov = [np.zeros_like(sc.data[0]) for _ in range(6)]
        inv.run(data, mean, cov, form="mixed")
        pm = np.stack([m[:, :, :sc.nxp] for m in mean])
        res = np.stack([d.view(np.complex64) for d in data])
        cv = np.stack([c.view(np.complex64) for c in cov])
        for o in outs:
            bpm, bres, bcov = o[i]
            assert np.array_equal(bpm, pm), i
            assert np.array_equal(bres, res), i
            assert np.array_equal(bcov, cv), i


def test_batch_cube_matches_fp64_oracle(cuda, oracle):
    from crava_gb300 import api
    scs = _scenarios()
    b = api.Batch(scs, nstreams=2)
    b.reset()
    b.run("mixed", use_graph=True)
    for i in (0, 2):
        sc = scs[i]
        pm, res, cov = b.read(i)
        tables = api.operator_tables(sc.wavelets, sc.A, sc.nz, sc.nzp, sc.dt_ms, sc.low_cut, sc.high_cut)
        post64, res64, cov64, _ = oracle_pipeline(oracle, sc, "d", tables=tables)
        prior = np.stack([m[:, :, :sc.nxp] for m in sc.mean]).astype(np.float64)
        e = (rel(pm, post64), rel(pm - prior, post64 - prior), rel(res, res64), rel(cov, cov64))
        print("batch cube", i, (sc.nxp, sc.nyp, sc.nzp, sc.ntheta), "vs FP64 oracle:", e)
        assert e[0] < 1e-6 and e[1] < 1e-4 and e[2] < 1e-4 and e[3] < 1e-4


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_simulation_matches_single_cube(cuda, use_graph):
    """Realisations drawn inside the batch equal the single-cube chain on the same posterior and seed."""
    import torch
    from crava_gb300 import api
    scs = _scenarios()
    b = api.Batch(scs, nstreams=3)
    nreal = {0: 2, 2: 3, 3: 1}
    for i, n in nreal.items():
        b.set_simulation(i, n, seed=100 + i)
    for rep in range(2):
        b.reset()
        b.run("mixed", use_graph=use_graph)
        got = {i: [b.read_fields(i, r) for r in range(n)] for i, n in nreal.items()}
        for i, n in nreal.items():
            sc = scs[i]
            inv = api.HostInversion(sc)
            data = [d.copy() for d in sc.data]
            mean = [m.copy() for m in sc.mean]
            cov = [np.zeros_like(sc.data[0]) for _ in range(6)]
            inv.run(data, mean, cov, form="mixed")
            chol, nfail = api.posterior_cholesky([torch.from_numpy(c).cuda() for c in cov], sc.nxp)
            fields = [torch.empty_like(torch.from_numpy(sc.mean[0])).cuda() for _ in range(3 * n)]
            api.simulate_fields(chol, fields, sc.nxp, seed=100 + i,
                                post_mean=[torch.from_numpy(m).cuda() for m in mean])
            torch.cuda.synchronize()
            for r in range(n):
                for p in range(3):
                    want = fields[3 * r + p].cpu().numpy()[:, :, :sc.nxp]
                    assert np.array_equal(got[i][r][p][:, :, :sc.nxp], want), (rep, i, r, p)
                # a realisation is not the posterior mean
                assert not np.array_equal(got[i][r][0][:, :, :sc.nxp], mean[0][:, :, :sc.nxp])
    # realisations are per-seed: two different seeds give different fields
    assert not np.array_equal(got[2][0][0], got[2][1][0])
    with pytest.raises(Exception):
        b.read_fields(1, 0)
    with pytest.raises(Exception):
        b.read_fields(0, 2)
    # removing the simulation keeps the inversion results
    b.set_simulation(0, 0)
    b.reset()
    b.run("mixed", use_graph=use_graph)
    with pytest.raises(Exception):
        b.read_fields(0, 0)
