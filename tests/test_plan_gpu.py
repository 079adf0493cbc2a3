"""GPU tests of spot plans: device-side beamlet sampling (moqui's beamsource + beamlet + phsp_6d,
moqui/base/mqi_beamsource.hpp:48-112, mqi_beamlet.hpp:80-90, distributions/mqi_phsp6d.hpp:61-79)
and the equivalence of one batched plan call with per-spot calls and with explicit vertices."""
import numpy as np
import pytest

from moquimc_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _rot(axis, deg):
    a = np.deg2rad(deg)
    c, s = np.cos(a), np.sin(a)
    if axis == "x":
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
    if axis == "y":
        return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])


def _plan(histories):
    sp = np.zeros(len(histories), capi.SPOT_DTYPE)
    sp["histories"] = histories
    sp["energy"] = [150.0, 120.0, 180.0][: len(histories)]
    sp["energy_sigma"] = [0.0, 1.5, 0.8][: len(histories)]
    sp["mean"] = [[0.0, 0.0, 0.5, 0.0, 0.0], [10.0, -5.0, 0.5, 0.01, -0.02], [-8.0, 6.0, 0.5, 0.0, 0.0]][: len(histories)]
    sp["sigma"] = [[4.0, 4.0, 0.0, 0.0, 0.0], [3.0, 5.0, 0.2, 0.003, 0.004], [2.0, 2.0, 0.0, 0.002, 0.002]][: len(histories)]
    sp["corr"] = [[0.0, 0.0], [0.6, -0.4], [0.2, 0.2]][: len(histories)]
    rots = [np.eye(3), _rot("z", 30.0), _rot("x", 4.0) @ _rot("z", -20.0)]
    sp["rot"] = np.array([r.ravel() for r in rots[: len(histories)]], np.float32)
    sp["trans"] = [[0.0, 0.0, 0.0], [1.0, 2.0, 0.0], [0.0, 0.0, -1.0]][: len(histories)]
    return sp


def _ctx(wl, make):
    c = make()
    c.set_physics(wl.physics_debug)
    cid = c.add_child(*wl.edges())
    c.set_hu(cid, wl.hu)
    return c, cid


def test_plan_sampling_moments(gpu_ctx_factory):
    n = 400_000
    sp = _plan([n, n, n])
    c = gpu_ctx_factory()
    assert c.set_spot_plan(sp) == 3 * n
    v, sid = c.sample_plan(0, 3 * n, 17)
    np.testing.assert_array_equal(sid, np.repeat(np.arange(3, dtype=np.uint32), n))
    for s in range(3):
        S = sp[s]
        R = S["rot"].reshape(3, 3).astype(np.float64)
        vs = v[sid == s]
        # back to the beam frame: p = R^T (x - T), d = R^T x'
        p = (vs["pos"].astype(np.float64) - S["trans"]) @ R
        d = vs["dir"].astype(np.float64) @ R
        se = 5.0 / np.sqrt(n)    # 5 standard errors, in units of sigma
        for k in range(3):
            sig = float(S["sigma"][k])
            if sig == 0.0:
                np.testing.assert_allclose(p[:, k], S["mean"][k], atol=2e-4)
            else:
                assert abs(p[:, k].mean() - S["mean"][k]) < se * sig
                assert abs(p[:, k].std() / sig - 1.0) < 5.0 * np.sqrt(0.5 / n)
        for k, j in ((3, 0), (4, 1)):
            sig = float(S["sigma"][k])
            if sig == 0.0:
                np.testing.assert_allclose(d[:, j], S["mean"][k], atol=1e-6)
                continue
            assert abs(d[:, j].mean() - S["mean"][k]) < se * sig
            assert abs(d[:, j].std() / sig - 1.0) < 5.0 * np.sqrt(0.5 / n)
            rho = np.corrcoef(p[:, j], d[:, j])[0, 1]
            assert abs(rho - S["corr"][j]) < 5.0 * (1 - S["corr"][j] ** 2) / np.sqrt(n)
        # z' = -sqrt(1 - x'^2 - y'^2): unit direction pointing down the beam axis
        np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=2e-6)
        assert (d[:, 2] < 0).all()
        ke = vs["ke"].astype(np.float64)
        if S["energy_sigma"] == 0.0:
            assert (vs["ke"] == S["energy"]).all()
        else:
            assert abs(ke.mean() - S["energy"]) < se * S["energy_sigma"]
            assert abs(ke.std() / S["energy_sigma"] - 1.0) < 5.0 * np.sqrt(0.5 / n)
    # the sample depends on (seed, history) only: a sub-range reproduces the same vertices
    v2, sid2 = c.sample_plan(n - 5, n + 5, 17)
    np.testing.assert_array_equal(v2.view(np.uint8), v[n - 5:n + 5].view(np.uint8))
    np.testing.assert_array_equal(sid2, sid[n - 5:n + 5])
    v3, _ = c.sample_plan(0, 10, 18)
    assert not np.array_equal(v3["pos"], v[:10]["pos"])


def test_plan_edges(gpu_ctx_factory):
    c = gpu_ctx_factory()
    sp = _plan([5, 0, 7])
    assert c.set_spot_plan(sp) == 12
    _, sid = c.sample_plan(0, 12, 1)
    np.testing.assert_array_equal(sid, [0] * 5 + [2] * 7)      # an empty spot gets no history
    with pytest.raises(capi.MqiError):
        c.sample_plan(0, 13, 1)
    wl = workloads.c2(histories=100)
    c2, _ = _ctx(wl, gpu_ctx_factory)
    with pytest.raises(capi.MqiError):
        c2.transport_plan(0, 1, 1)                              # no plan yet
    c2.set_spot_plan(sp)
    with pytest.raises(capi.MqiError):
        c2.transport_plan(0, 13, 1)
    c2.transport_plan(3, 3, 1)                                  # empty range
    assert c2.stats()["histories"] == 0


def test_plan_equals_explicit_vertices(gpu_ctx_factory):
    """mqi_transport_plan == mqi_set_vertices(sampled vertices, spot ids) + mqi_transport: the
    transport streams are keyed by the history index, so both runs take identical steps; the FP64
    tallies differ only by atomic summation order."""
    wl = workloads.c2(histories=30_000)
    sp = _plan([12_000, 8_000, 10_000])
    res = []
    for mode in ("plan", "vertices"):
        c, cid = _ctx(wl, gpu_ctx_factory)
        d = c.add_scorer(cid, capi.DOSE_W)
        N = c.set_spot_plan(sp)
        if mode == "plan":
            c.transport_plan(0, N, 77)
        else:
            v, sid = c.sample_plan(0, N, 77)
            c.set_vertices(v, sid)
            c.transport(0, N, 77)
        st = c.stats()
        res.append((c.tally(d), st["steps"], st["tracks"], st["secondaries"]))
    a, b = res
    assert a[1:] == b[1:]
    np.testing.assert_allclose(a[0], b[0], rtol=1e-12, atol=1e-300)


def test_per_spot_calls_equal_one_batched_call(gpu_ctx_factory):
    wl = workloads.c2(histories=30_000)
    sp = _plan([12_000, 8_000, 10_000])
    res = []
    for mode in ("batched", "per_spot"):
        c, cid = _ctx(wl, gpu_ctx_factory)
        d = c.add_scorer(cid, capi.DOSE_W)
        N = c.set_spot_plan(sp)
        if mode == "batched":
            c.transport_plan(0, N, 5)
        else:
            cum = c.plan_cum
            for s in range(len(sp)):
                c.transport_plan(int(cum[s]), int(cum[s + 1]), 5)
        st = c.stats()
        res.append((c.tally(d), st["steps"], st["histories"]))
    a, b = res
    assert a[1:] == b[1:]
    np.testing.assert_allclose(a[0], b[0], rtol=1e-12, atol=1e-300)


def test_streamed_graph_equals_generations(gpu_ctx_factory):
    """The device top-up + graph-captured waves and the generation loop run the same tracks: equal
    step counts and tallies equal up to FP64 summation order, for vertices and plans, and with
    chunks smaller than the run so that the top-up interleaves new histories with daughters."""
    wl = workloads.c2(histories=30_000)
    sp = _plan([12_000, 8_000, 10_000])
    v = wl.vertices(20_000, 4)
    res = {}
    for mode in ("generations", "streamed", "streamed2"):
        c, cid = _ctx(wl, gpu_ctx_factory)
        d = c.add_scorer(cid, capi.DOSE_W)
        c.set_tuning(primary_chunk=4096)
        c.set_launch_mode(0 if mode == "generations" else 1, 2 if mode == "streamed2" else 8)
        N = c.set_spot_plan(sp)
        c.transport_plan(0, N, 31)
        c.set_vertices(v)
        c.transport(0, len(v), 32)
        st = c.stats()
        res[mode] = (c.tally(d), st["steps"], st["histories"], st["secondaries"])
    a = res["generations"]
    for m in ("streamed", "streamed2"):
        b = res[m]
        assert a[1:] == b[1:]
        np.testing.assert_allclose(a[0], b[0], rtol=1e-12, atol=1e-300)


def test_autotune_keeps_tallies_and_picks_a_candidate(gpu_ctx_factory):
    wl = workloads.c2(histories=20_000)
    c, cid = _ctx(wl, gpu_ctx_factory)
    d = c.add_scorer(cid, capi.DOSE_W)
    c.set_vertices(wl.vertices(20_000, 8))
    c.transport(0, 5_000, 3)
    before, st = c.tally(d), c.stats()
    res = c.autotune(0, 20_000, 9)
    assert len(res) == 8 and (res["histories_per_s"] > 0).all()   # one queue size: all exceed the sample
    np.testing.assert_array_equal(c.tally(d), before)
    assert c.stats() == st
    # the chosen setting runs the same tracks as the default one
    c.transport(5_000, 10_000, 3)
    e, eid = _ctx(wl, gpu_ctx_factory)
    f = e.add_scorer(eid, capi.DOSE_W)
    e.set_vertices(wl.vertices(20_000, 8))
    e.transport(0, 10_000, 3)
    np.testing.assert_allclose(c.tally(d), e.tally(f), rtol=1e-12, atol=1e-300)
