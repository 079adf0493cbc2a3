"""GPU tests of robust scenarios: one launch over scenarios that differ in setup shift (shifted
voxel edges, tps_env's XShift/YShift/ZShift, moqui/base/environments/mqi_tps_env.hpp:475-477) and
density scale (DensityScaling, mqi_tps_env.hpp:766-769) equals separate single-scenario runs, and
statistical stopping over plan passes."""
import numpy as np
import pytest

from moquimc_gb300 import capi, phantom as ph, workloads

pytestmark = pytest.mark.gpu

SCEN = [((0.0, 0.0, 0.0), 1.0), ((3.0, 0.0, 0.0), 1.035), ((0.0, -3.0, 0.0), 0.965), ((0.0, 0.0, 3.0), 1.0)]


def _edges(wl, shift):
    """Edges of the shifted box: the origin moves, then the edges are formed from it."""
    p = tuple(np.float32(a) + np.float32(b) for a, b in zip(wl.pxyz, shift))
    return ph.phantom_box_edges(wl.lxyz, p, wl.nxyz)


def _setup(make, wl, edges, rho):
    c = make()
    c.set_physics(wl.physics_debug)
    cid = c.add_child(*edges)
    c.set_density(cid, rho)
    return c, cid


def test_scenarios_equal_separate_runs(gpu_ctx_factory):
    wl = workloads.c2(histories=6000)
    probe = gpu_ctx_factory()
    rho0 = probe.hu_to_density(wl.hu.ravel())
    n = 6000
    v = wl.vertices(n, 13)
    # one launch over all scenarios
    c, cid = _setup(gpu_ctx_factory, wl, _edges(wl, SCEN[0][0]), rho0)
    dose = c.add_scorer(cid, capi.DOSE_W)
    es = [_edges(wl, s) for s, _ in SCEN]
    c.set_scenarios(cid, [e[0] for e in es], [e[1] for e in es], [e[2] for e in es], [k for _, k in SCEN])
    c.set_vertices(v)
    c.transport(0, n, 21)
    tally = c.tally(dose).reshape(len(SCEN), -1)
    st = c.stats()
    assert st["histories"] == n * len(SCEN)
    steps = 0
    for k, (shift, scale) in enumerate(SCEN):
        rho = (rho0 * np.float32(scale)).astype(np.float32)    # one FP32 product per voxel
        d, did = _setup(gpu_ctx_factory, wl, es[k], rho)
        sid = d.add_scorer(did, capi.DOSE_W)
        d.set_vertices(v)
        d.transport(0, n, 21)
        ref = d.tally(sid)
        steps += d.stats()["steps"]
        np.testing.assert_array_equal(np.flatnonzero(tally[k]), np.flatnonzero(ref))
        np.testing.assert_allclose(tally[k], ref, rtol=1e-12, atol=1e-300)
    assert st["steps"] == steps
    # the scenarios differ from one another
    assert not np.allclose(tally[0], tally[1])


def test_scenario_statistics_report_the_worst(gpu_ctx_factory):
    wl = workloads.c2(histories=4000)
    probe = gpu_ctx_factory()
    rho0 = probe.hu_to_density(wl.hu.ravel())
    c, cid = _setup(gpu_ctx_factory, wl, wl.edges(), rho0)
    d1, d2 = c.add_stat_scorers(cid)
    es = [_edges(wl, s) for s, _ in SCEN[:3]]
    c.set_scenarios(cid, [e[0] for e in es], [e[1] for e in es], [e[2] for e in es], [k for _, k in SCEN[:3]])
    c.set_vertices(wl.vertices(4000, 2))
    c.transport(0, 4000, 3)
    s1 = c.tally(d1).reshape(3, -1)
    s2 = c.tally(d2).reshape(3, -1)
    got, _ = c.stat_uncertainty(d1, d2, 4000, 0.5)
    per = []
    for k in range(3):
        sc = s1[k] > 0
        m = s1[k][sc] / 4000
        var = ((s2[k][sc] / 4000 - m * m) / 3999).astype(np.float32)
        sig = np.sqrt(np.maximum(var, 0)).astype(np.float32)
        mean = m.astype(np.float32)
        sel = mean.astype(np.float64) > mean.max() * np.float64(np.float32(0.5))
        per.append(float(np.mean((sig[sel] / mean[sel]).astype(np.float64))))
    assert abs(got - max(per)) <= 1e-6 * max(per)
    # removing the scenarios restores one tally per scorer
    c.set_scenarios(cid, [], [], [])
    assert len(c.tally(d1)) == len(s1[0])


def test_run_plan_until_stat(gpu_ctx_factory):
    wl = workloads.c2(histories=1000)
    c = gpu_ctx_factory()
    c.set_physics(False)
    cid = c.add_child(*wl.edges())
    c.set_hu(cid, wl.hu)
    dose = c.add_scorer(cid, capi.DOSE_W)
    d1, d2 = c.add_stat_scorers(cid)
    sp = np.zeros(2, capi.SPOT_DTYPE)
    sp["energy"] = [120.0, 140.0]
    sp["mean"][:, 2] = 0.5
    sp["sigma"][:, :2] = 4.0
    sp["rot"] = np.eye(3, dtype=np.float32).ravel()
    sp["histories"] = [3000, 2000]
    N = c.set_spot_plan(sp)
    passes, got = c.run_plan_until_stat(d1, d2, 0.04, 0.5, 40, 17)
    assert got <= 0.04 and passes > 1
    prev = got * np.sqrt(passes / (passes - 1))
    assert prev > 0.04 * 0.9
    # the dose scorer holds one pass worth of dose: the stat dose (all passes) / passes
    total = c.tally(dose).sum()
    assert abs(total - c.tally(d1)[1:].sum() / passes) <= 1e-9 * total
    assert c.stats()["histories"] == N * passes
