"""GPU tests of the statistics path: the reference's estimator (calculate_standard_deviation +
tps_env::calculate_stat), the batch estimator, statistical stopping, and the scoring rules that
depend on whether a node carries the statistics pair."""
import numpy as np
import pytest

from moquimc_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _ctx(wl, make):
    c = make()
    c.set_physics(wl.physics_debug)
    cid = c.add_child(*wl.edges())
    c.set_hu(cid, wl.hu)
    return c, cid


def _ref_estimate(s1, s2, n, thr):
    """The reference's estimator in numpy: sigma stored as float, mean as float, mean of
    sigma/mean over voxels with mean > thr * max (mqi_variables.hpp:38-45, mqi_tps_env.hpp:1409-1425)."""
    sc = s1 > 0
    m = s1[sc] / n
    v = ((s2[sc] / n - m * m) / (n - 1)).astype(np.float32)
    v = np.where(v > 0, v, np.float32(0))
    sig = np.sqrt(v).astype(np.float32)
    mean = m.astype(np.float32)
    sel = mean.astype(np.float64) > mean.max() * np.float64(np.float32(thr))
    return float(np.mean((sig[sel] / mean[sel]).astype(np.float64))), int(sel.sum())


def test_reference_estimator_matches_numpy(gpu_ctx_factory):
    wl = workloads.c2()
    c, cid = _ctx(wl, gpu_ctx_factory)
    dose = c.add_scorer(cid, capi.DOSE_W)
    d1, d2 = c.add_stat_scorers(cid)
    n = 50_000
    c.set_vertices(wl.vertices(n, 21))
    c.transport(0, n, 99)
    s1, s2 = c.tally(d1), c.tally(d2)
    for thr in (0.5, 0.1):
        got, nv = c.stat_uncertainty(d1, d2, n, thr)
        exp, nexp = _ref_estimate(s1, s2, n, thr)
        assert nv == nexp
        assert abs(got - exp) <= 1e-6 * exp
    # the stat dose equals the dose scorer except at voxel 0, which only the stat gate admits
    plain = c.tally(dose)
    np.testing.assert_allclose(s1[1:], plain[1:], rtol=1e-9, atol=1e-300)
    assert plain[0] == 0.0


@pytest.mark.parametrize("mode", [0, 1])
def test_dose_and_stat_pair_mode_matches_the_generic_scoring(gpu_ctx_factory, mode):
    """A dose scorer followed by the statistics pair runs a kernel instance of its own (the generic
    per-scorer loop folded away); with a fourth scorer added the same run takes the generic loop.
    The dose, dose and dose^2 tallies agree to FP64 summation order, inline and split."""
    wl = workloads.c2()
    n = 30_000
    v = wl.vertices(n, 31)
    out = []
    for extra in (False, True):
        c, cid = _ctx(wl, gpu_ctx_factory)
        c.set_post_step_mode(mode)
        dose = c.add_scorer(cid, capi.DOSE_W)
        d1, d2 = c.add_stat_scorers(cid)
        if extra:
            c.add_scorer(cid, capi.EDEP)
        c.set_vertices(v)
        c.transport(0, n, 1234)
        out.append((c.tally(dose), c.tally(d1), c.tally(d2), c.stats()["steps"]))
    for a, b in zip(out[0][:3], out[1][:3]):
        assert a.sum() > 0
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-300)
    assert out[0][3] == out[1][3]


def test_estimate_falls_like_one_over_sqrt_n(gpu_ctx_factory):
    wl = workloads.c2()
    c, cid = _ctx(wl, gpu_ctx_factory)
    d1, d2 = c.add_stat_scorers(cid)
    c.set_vertices(wl.vertices(100_000, 3))
    c.transport(0, 25_000, 1)
    a, _ = c.stat_uncertainty(d1, d2, 25_000, 0.5)
    c.transport(0, 100_000, 2)
    b, _ = c.stat_uncertainty(d1, d2, 125_000, 0.5)
    assert 0.35 < b / a < 0.55     # sqrt(25000/125000) = 0.447


def test_batch_estimator_matches_numpy(gpu_ctx_factory):
    wl = workloads.c2()
    c, cid = _ctx(wl, gpu_ctx_factory)
    dose = c.add_scorer(cid, capi.DOSE_W)
    B, n = 6, 20_000
    c.set_vertices(wl.vertices(B * n, 31))
    batches = []
    for b in range(B):
        c.transport(b * n, (b + 1) * n, 1000 + b)
        batches.append(c.tally(dose))
        c.batch_accumulate(dose)
        assert c.tally(dose).sum() == 0.0
    x = np.array(batches)
    got, nv, nb = c.batch_uncertainty(dose, 0.5)
    assert nb == B
    mean = x.mean(0)
    var = (np.mean(x * x, 0) - mean * mean) / (B - 1)
    rel = np.sqrt(np.maximum(var, 0) / B) / np.where(mean > 0, mean, 1)
    sel = mean > 0.5 * mean.max()
    assert nv == sel.sum()
    assert abs(got - rel[sel].mean()) <= 1e-9 * rel[sel].mean()
    np.testing.assert_allclose(c.batch_mean(dose), mean, rtol=1e-12, atol=1e-300)


def test_run_until_stat_stops_at_the_criterion(gpu_ctx_factory):
    wl = workloads.c2()
    c, cid = _ctx(wl, gpu_ctx_factory)
    dose = c.add_scorer(cid, capi.DOSE_W)
    d1, d2 = c.add_stat_scorers(cid)
    per_run = 20_000
    c.set_vertices(wl.vertices(per_run, 5))
    done, got = c.run_until_stat(d1, d2, per_run, 0.03, 0.5, 50, 7)
    assert got <= 0.03 and done % per_run == 0 and done > per_run
    # one more run would have been unnecessary: the estimate before the last run was above 3%
    est_prev = got * np.sqrt(done / (done - per_run))
    assert est_prev > 0.03 * 0.9
    # the dose scorer is scaled back to one run's worth of histories (calculate_average_results)
    total = c.tally(dose).sum()
    assert abs(total - c.tally(d1)[1:].sum() * per_run / done) <= 1e-9 * total


def test_double_scoring_quirk_and_stat_kernel(gpu_ctx_factory):
    """moqui's non-stat kernel inserts scorers 0..n-3 twice per step when a node has >= 3 scorers
    (mqi_transport.hpp:204-225); its _stat kernel, used when the statistics pair is present,
    inserts each once."""
    wl = workloads.c2(histories=5000)
    n = 5000
    v = wl.vertices(n, 9)
    res = {}
    for tag in ("one", "three", "three_stat"):
        c, cid = _ctx(wl, gpu_ctx_factory)
        s0 = c.add_scorer(cid, capi.DOSE_W)
        if tag != "one":
            c.add_scorer(cid, capi.EDEP)
            c.add_scorer(cid, capi.EDEP)
        if tag == "three_stat":
            c.add_stat_scorers(cid)
        c.set_vertices(v)
        c.transport(0, n, 123)
        res[tag] = c.tally(s0)
    np.testing.assert_allclose(res["three"], 2.0 * res["one"], rtol=1e-9, atol=1e-300)
    np.testing.assert_allclose(res["three_stat"], res["one"], rtol=1e-9, atol=1e-300)
