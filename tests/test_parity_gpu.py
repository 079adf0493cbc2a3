"""GPU parity tests: the CUDA path, called through the C ABI, against the golden vectors of the
reference's own CPU build and against the C restatement run on the same random streams.

Tolerances:
* integer/index work (voxel walks, HU -> density): bit-exact;
* tabulated physics: identical table lookups, <= 2e-6 relative where the reference uses double
  intermediates;
* dose (FP32 stepping, FP64 tally) vs the reference: per depth bin within 2% or 3 sigma of the
  combined statistical uncertainty in bins above 10% of the maximum (>= 95% of bins), R80 within
  0.2 mm;
* GPU vs the C restatement on identical Philox streams: total energy within 1e-4, and at least 99%
  of the dose in voxels that agree to 1e-3 (rare FP32 ulp differences in libm functions can flip
  a branch of a single history).
"""
import numpy as np
import pytest

from moquimc_gb300 import capi
from moquimc_gb300 import phantom as ph
from moquimc_gb300 import workloads

pytestmark = pytest.mark.gpu


def _ctx_for(wl, make, scorer=capi.DOSE_W):
    c = make()
    c.set_physics(wl.physics_debug)
    cid = c.add_child(*wl.edges())
    c.set_hu(cid, wl.hu)
    sid = c.add_scorer(cid, scorer)
    return c, cid, sid


@pytest.mark.parametrize("name", ["phantom", "ct"])
def test_raywalk_gpu_bit_exact(golden, gpu_ctx_factory, name):
    g = golden("raywalk.npz")
    b, n = g[f"{name}_bounds"], g[f"{name}_n"]
    edges = [ph.uniform_edges(float(b[2 * a]), float(b[2 * a + 1]), int(n[a])) for a in range(3)]
    c = gpu_ctx_factory()
    cid = c.add_child(*edges)
    off, cnb, dist, cells = c.trace_rays(cid, g[f"{name}_rays"], int(g[f"{name}_max_steps"]))
    np.testing.assert_array_equal(off, g[f"{name}_offsets"])
    np.testing.assert_array_equal(cnb.astype(np.uint32), g[f"{name}_cnb"])
    np.testing.assert_array_equal(dist.view(np.uint32), g[f"{name}_dist_bits"])
    nx, ny = int(n[0]), int(n[1])
    np.testing.assert_array_equal(cells[:, 0] + nx * (cells[:, 1] + ny * cells[:, 2]), cnb.astype(np.int64))


def test_physics_probe_gpu(golden, gpu_ctx_factory):
    p = golden("physics.npz")
    c = gpu_ctx_factory()
    out = c.eval_physics(p["energies"])
    for k, name in enumerate(["cs_ion", "cs_pp", "cs_poe", "cs_poi", "dedx"]):
        np.testing.assert_allclose(out[:, k], p[name], rtol=1e-6, atol=0, err_msg=name)
        assert np.mean(out[:, k] == p[name]) > 0.99, name
    np.testing.assert_allclose(out[:, 5], p["beta_sq"], rtol=2e-6, atol=1e-9)
    np.testing.assert_allclose(out[:, 6], p["te_max"], rtol=2e-6, atol=1e-12)
    np.testing.assert_allclose(out[:, 7], p["momentum"], rtol=1e-6)


def test_hu_to_density_gpu_bit_exact(golden, gpu_ctx_factory):
    p = golden("physics.npz")
    c = gpu_ctx_factory()
    rho = c.hu_to_density(p["hu"].astype(np.int16))
    np.testing.assert_array_equal(rho.view(np.uint32), p["hu_rho"].view(np.uint32))
    rho2 = c.hu_to_density(p["hu"].astype(np.int16), scale=1.035)
    np.testing.assert_array_equal(rho2, (p["hu_rho"] * np.float32(1.035)).astype(np.float32))


_GRIDS = {}


def _oracle_grid(oracle, wl):
    import hashlib

    key = (wl.name, tuple(wl.nxyz), tuple(wl.lxyz), tuple(wl.pxyz), hashlib.md5(wl.hu.tobytes()).hexdigest())
    if key not in _GRIDS:
        hu = np.unique(wl.hu)
        lut = np.array([oracle.hu_to_density(int(h)) for h in hu], np.float32)
        rho = lut[np.searchsorted(hu, wl.hu)].reshape(-1)
        _GRIDS[key] = oracle.Grid(*wl.edges(), rho)
    return _GRIDS[key]


def _laterally_coarse(wl, k):
    """The same depth structure on k x k coarser lateral voxels (cheap per-history tallies)."""
    nx, ny, nz = wl.nxyz
    wl.hu = np.ascontiguousarray(wl.hu[:, ::k, ::k])
    wl.nxyz = (nx // k, ny // k, nz)
    return wl


@pytest.mark.parametrize("wname", ["c1", "c2"])
def test_gpu_matches_oracle_history_by_history(oracle, gpu_ctx_factory, wname):
    """Same Philox streams on the GPU and in the C restatement: each history deposits the same
    energy to 1e-4 unless an FP32 ulp difference between CUDA's and libm's transcendental functions
    flips one discrete decision along it, which must stay rare."""
    wl = _laterally_coarse(workloads.WORKLOADS[wname](histories=200), 10 if wname == "c1" else 16)
    n, seed = 200, 0xC0FFEE
    v = wl.vertices(n, 11)
    c, cid, sid = _ctx_for(wl, gpu_ctx_factory, capi.EDEP)
    c.set_vertices(v)
    e_gpu = np.zeros(n)
    steps = 0
    for h in range(n):
        c.reset()
        c.transport(h, h + 1, seed)
        e_gpu[h] = c.tally(sid).sum()
        st = c.stats()
        # the oracle pops each deposit-only daughter and counts its one step; the GPU scores
        # them where they are created
        steps += st["steps"] + st["local_daughters"]
    _, e_ora, ost = oracle.transport(_oracle_grid(oracle, wl), v, 0, n, seed, wl.physics_debug, scorer=1,
                                     per_history=True)
    same = np.abs(e_gpu - e_ora) <= 1e-4 * np.maximum(e_ora, 1e-9)
    assert same.mean() >= 0.95, (same.mean(), np.flatnonzero(~same)[:10])
    assert abs(e_gpu.sum() - e_ora.sum()) <= 0.02 * e_ora.sum()
    assert abs(steps - ost["steps"]) <= 0.02 * ost["steps"]


def test_tabulated_calibration_matches_oracle_history_by_history(oracle, gpu_ctx_factory):
    """A custom calibration (mqi_set_calibration: SPR(rho, E) and X0(rho) tables; here moqui's
    default curves scaled by 1.05 and 0.9) on the slab phantom: the GPU and the restatement on the
    same Philox streams, history by history as above; then the default curves back."""
    wl = _laterally_coarse(workloads.c2(histories=200), 16)
    n, seed = 200, 0xCA11B
    table = capi.CalibTable.sample(lambda r, e: 1.05 * oracle.spr(r, e, False), lambda r: 0.9 * oracle.x0(r, False),
                                   1.0e-4, 1.0e-5, 241, 0.5, 0.5, 500)
    v = wl.vertices(n, 13)
    c, cid, sid = _ctx_for(wl, gpu_ctx_factory, capi.EDEP)
    c.set_calibration(table)
    c.set_vertices(v)
    e_gpu = np.zeros(n)
    for h in range(n):
        c.reset()
        c.transport(h, h + 1, seed)
        e_gpu[h] = c.tally(sid).sum()
    grid = _oracle_grid(oracle, wl)
    _, e_ora, _ = oracle.transport(grid, v, 0, n, seed, wl.physics_debug, scorer=1, per_history=True, calib=table)
    _, e_def, _ = oracle.transport(grid, v, 0, n, seed, wl.physics_debug, scorer=1, per_history=True)
    same = np.abs(e_gpu - e_ora) <= 1e-4 * np.maximum(e_ora, 1e-9)
    assert same.mean() >= 0.95, (same.mean(), np.flatnonzero(~same)[:10])
    assert not np.allclose(e_ora, e_def, rtol=1e-3)   # the tables did change the transport
    c.set_calibration(None)
    c.reset()
    c.transport(0, n, seed)
    assert abs(c.tally(sid).sum() / e_def.sum() - 1.0) <= 0.02


def test_calibration_arguments_are_checked(gpu_ctx_factory):
    c = gpu_ctx_factory()
    lib = c.lib
    spr = np.ones(4, np.float32)
    x0 = np.ones(2, np.float32)
    bad = [
        (capi.CALIB_TABLE, 1, 0.0, 1.0, 2, 0.0, 1.0, spr, x0),              # one density node
        (capi.CALIB_TABLE, 2, 0.0, 0.0, 2, 0.0, 1.0, spr, x0),              # zero pitch
        (capi.CALIB_TABLE, 2, 0.0, 1.0, 2, 0.0, 1.0, None, x0),             # no SPR table
        (capi.CALIB_TABLE, 2, 0.0, 1.0, 2, 0.0, 1.0, spr, -x0),             # X0 <= 0
        (7, 2, 0.0, 1.0, 2, 0.0, 1.0, spr, x0),                              # unknown calibration
    ]
    for mode, nr, r0, dr, ne, e0, de, s_, x_ in bad:
        rc = lib.mqi_set_calibration(c.h, mode, nr, r0, dr, ne, e0, de,
                                     None if s_ is None else s_.ctypes.data, x_.ctypes.data)
        assert rc == capi.MQI_ERR_INVALID
    nan = spr.copy()
    nan[1] = np.nan
    assert lib.mqi_set_calibration(c.h, capi.CALIB_TABLE, 2, 0.0, 1.0, 2, 0.0, 1.0, nan.ctypes.data,
                                   x0.ctypes.data) == capi.MQI_ERR_INVALID
    assert lib.mqi_set_calibration(c.h, capi.CALIB_TABLE, 2, 0.0, 1.0, 2, 0.0, 1.0, spr.ctypes.data,
                                   x0.ctypes.data) == capi.MQI_OK


def test_gpu_matches_oracle_in_aggregate(oracle, gpu_ctx_factory):
    """Full-resolution phantom example, 4 x 3000 histories on each side: the depth-dose curves of
    the GPU and of the C restatement agree within 2% or 3 sigma, and R80 within 0.2 mm (the
    standard error of each side's R80 is about 0.03 mm at 12 000 histories).  (Voxel-for-voxel equality on the
    same streams does not hold: a 1-ulp difference between CUDA's and libm's powf in the stopping
    power ratio flips near-ties such as a 1.0 mm boundary distance against a 1.0 mm step limit,
    and the extra step shifts the track's Philox block counter.)"""
    wl = workloads.c1()
    each, seed = 3000, 0xBEEF
    c, cid, sid = _ctx_for(wl, gpu_ctx_factory, capi.DOSE_W)
    grid = _oracle_grid(oracle, wl)
    g_b, o_b = [], []
    for b in range(4):
        v = wl.vertices(each, 12 + b)
        c.reset()
        c.set_vertices(v)
        c.transport(0, each, seed + b)
        g_b.append(ph.depth_dose(c.tally(sid), wl.nxyz) / each)
        ora, _, ost = oracle.transport(grid, v, 0, each, seed + b, True, scorer=2)
        o_b.append(ph.depth_dose(ora, wl.nxyz) / each)
        assert c.stats()["histories"] == each == ost["histories"]
    g_b, o_b = np.array(g_b), np.array(o_b)
    gm, gs = g_b.mean(0), g_b.std(0, ddof=1) / 2
    om, os_ = o_b.mean(0), o_b.std(0, ddof=1) / 2
    sel = om > 0.1 * om.max()
    ok = (np.abs(gm - om) <= 0.02 * om) | (np.abs(gm - om) <= 3 * np.sqrt(gs ** 2 + os_ ** 2))
    assert ok[sel].mean() >= 0.95
    assert abs(ph.r80(gm, 1.0) - ph.r80(om, 1.0)) <= 0.2, (ph.r80(gm, 1.0), ph.r80(om, 1.0))


def test_gpu_fp32_matches_the_fp64_oracle(oracle, gpu_ctx_factory):
    """Slab phantom: FP32 stepping with FP64 dose and dose^2 tallies against the all-FP64 oracle
    (the restatement built with -DMQO_FP64) on the same vertices and the same Philox streams,
    8 x 2000 histories.  Depth dose and depth dose^2 within 2% or 3 sigma in bins above 10% of the
    maximum, R80 within 0.2 mm, and the total dose within 0.2%: FP32 arithmetic moves the dose by
    much less than the statistics do."""
    wl = workloads.c2()
    each, batches = 2000, 8
    c = gpu_ctx_factory()
    c.set_physics(wl.physics_debug)
    cid = c.add_child(*wl.edges())
    c.set_hu(cid, wl.hu)
    s_d = c.add_scorer(cid, capi.DOSE_W)
    s_d2 = c.add_scorer(cid, capi.DOSE_W2)
    grid = _oracle_grid(oracle, wl)
    g = {"d": [], "d2": []}
    o = {"d": [], "d2": []}
    tot_g = tot_o = 0.0
    for b in range(batches):
        v = wl.vertices(each, 7100 + b)
        seed = 0xF64 + b
        c.reset()
        c.set_vertices(v)
        c.transport(0, each, seed)
        dg, d2g = c.tally(s_d), c.tally(s_d2)
        do, _, _ = oracle.transport(grid, v, 0, each, seed, wl.physics_debug, scorer=2, fp64=True)
        d2o, _, _ = oracle.transport(grid, v, 0, each, seed, wl.physics_debug, scorer=3, fp64=True)
        g["d"].append(ph.depth_dose(dg, wl.nxyz) / each)
        g["d2"].append(ph.depth_dose(d2g, wl.nxyz) / each)
        o["d"].append(ph.depth_dose(do, wl.nxyz) / each)
        o["d2"].append(ph.depth_dose(d2o, wl.nxyz) / each)
        tot_g += dg.sum()
        tot_o += do.sum()
    for k in ("d", "d2"):
        gb, ob = np.array(g[k]), np.array(o[k])
        gm, gs = gb.mean(0), gb.std(0, ddof=1) / np.sqrt(batches)
        om, os_ = ob.mean(0), ob.std(0, ddof=1) / np.sqrt(batches)
        sel = om > 0.1 * om.max()
        ok = (np.abs(gm - om) <= 0.02 * om) | (np.abs(gm - om) <= 3 * np.sqrt(gs ** 2 + os_ ** 2))
        assert ok[sel].mean() >= 0.95, (k, ok[sel].mean())
        if k == "d":
            assert abs(ph.r80(gm, 1.0) - ph.r80(om, 1.0)) <= 0.2, (ph.r80(gm, 1.0), ph.r80(om, 1.0))
    assert abs(tot_g / tot_o - 1.0) <= 2e-3, tot_g / tot_o


def _gpu_idd_batches(wl, make, batches, each, seed0):
    c, cid, sid = _ctx_for(wl, make)
    out, coarse = [], []
    for b in range(batches):
        c.reset()
        c.set_vertices(wl.vertices(each, seed0 + b))
        c.transport(0, each, seed0 * 7919 + b)
        d = c.tally(sid)
        out.append(ph.depth_dose(d, wl.nxyz) / each)
        coarse.append(d)
    return np.array(out), coarse


def _coarse(d, nxyz, b):
    nx, ny, nz = nxyz
    return d.reshape(nz, ny, nx).reshape(nz // b[2], b[2], ny // b[1], b[1], nx // b[0], b[0]).sum(axis=(1, 3, 5))


@pytest.mark.parametrize("wname,fixture", [("c1", "dose_c1.npz"), ("c2", "dose_c2.npz")])
def test_gpu_dose_matches_reference(golden, gpu_ctx_factory, wname, fixture):
    gd = golden(fixture)
    wl = workloads.WORKLOADS[wname]()
    each = int(gd["histories_per_batch"])
    idd, doses = _gpu_idd_batches(wl, gpu_ctx_factory, 8, each, 2024)
    ref = gd["idd"]
    rm, rs = ref.mean(0), ref.std(0, ddof=1) / np.sqrt(len(ref))
    tm, ts = idd.mean(0), idd.std(0, ddof=1) / np.sqrt(len(idd))
    sel = rm > 0.1 * rm.max()
    ok = (np.abs(tm - rm) <= 0.02 * rm) | (np.abs(tm - rm) <= 3 * np.sqrt(rs ** 2 + ts ** 2))
    assert ok[sel].mean() >= 0.95, ok[sel].mean()
    dz = wl.lxyz[2] / wl.nxyz[2]
    assert abs(ph.r80(tm, dz) - ph.r80(rm, dz)) <= 0.2, (ph.r80(tm, dz), ph.r80(rm, dz))
    # per-voxel (coarse bins) dose
    b = tuple(int(x) for x in gd["coarse_bins"])
    gc = np.array([_coarse(d, wl.nxyz, b) / each for d in doses])
    rc = gd["coarse"]
    gm, gs = gc.mean(0), gc.std(0, ddof=1) / np.sqrt(len(gc))
    cm, cs = rc.mean(0), rc.std(0, ddof=1) / np.sqrt(len(rc))
    sel = cm > 0.1 * cm.max()
    ok = (np.abs(gm - cm) <= 0.02 * cm) | (np.abs(gm - cm) <= 3 * np.sqrt(gs ** 2 + cs ** 2))
    assert ok[sel].mean() >= 0.95, ok[sel].mean()


def test_slicing_and_launch_shape_do_not_change_results(gpu_ctx_factory):
    wl = workloads.c1()
    n = 3000
    v = wl.vertices(n, 5)
    res = []
    for tune in ({}, {"slice_steps": 37}, {"block": 128, "blocks_per_sm": 4, "slice_steps": 5}):
        c, cid, sid = _ctx_for(wl, gpu_ctx_factory)
        if tune:
            c.set_tuning(**tune)
        c.set_vertices(v)
        c.transport(0, n, 99)
        res.append((c.tally(sid), c.stats()))
    base, st0 = res[0]
    for d, st in res[1:]:
        np.testing.assert_allclose(d, base, rtol=1e-9, atol=1e-300)
        assert st["steps"] == st0["steps"] and st["histories"] == n


@pytest.mark.parametrize("wname,dbg", [("c1", True), ("c2", False)])
def test_post_step_modes_and_queue_sort_give_the_same_tracks(gpu_ctx_factory, wname, dbg):
    """Nuclear post-steps inside the wave (mode 0) or in the post-step kernel (mode 1), with the
    queue sorted by energy bin before every wave or never, run the same tracks on the same random
    numbers: identical step counts and tallies to FP64 summation order, in both physics builds."""
    wl = workloads.WORKLOADS[wname]()
    wl.physics_debug = dbg
    n = 20_000
    v = wl.vertices(n, 21)
    res = []
    for mode, sort_min in ((0, 0), (1, 0), (1, 1), (0, 1)):
        c, cid, sid = _ctx_for(wl, gpu_ctx_factory)
        c.set_post_step_mode(mode)
        c.set_queue_sort(sort_min)
        c.set_launch_mode(streamed=0)          # queue generations: the wave count is the waves run
        c.set_vertices(v)
        c.transport(0, n, 77)
        res.append((c.tally(sid), c.stats()))
    d0, st0 = res[0]
    for d1, st1 in res[1:]:
        np.testing.assert_allclose(d1, d0, rtol=1e-9, atol=1e-300)
        for k in ("steps", "histories", "secondaries", "local_daughters", "dropped"):
            assert st1[k] == st0[k], k
    assert res[1][1]["waves"] > st0["waves"]   # each nuclear interaction ends its track's wave


def test_slicing_on_a_deep_grid(gpu_ctx_factory):
    """Tracks re-queued mid-grid resume in the voxel they stopped in, at every slice index: a
    700-slice water column (0.4 mm slices; the beam enters at slice 699 and 200 MeV protons stop
    near slice 50, so every track crosses slices 512-699), sliced every 5 steps, gives the
    unsliced tallies."""
    wl = workloads.Workload("deep_water_column", (40.0, 40.0, 280.0), (0.0, 0.0, -140.0), (20, 20, 700),
                            np.zeros((700, 20, 20), np.int16), 200.0, "gaussian", (3.0, 3.0), (0.0, 0.0, 0.5),
                            2000, False)
    n = 2000
    v = wl.vertices(n, 11)
    res = []
    for tune in ({}, {"slice_steps": 5}):
        c, cid, sid = _ctx_for(wl, gpu_ctx_factory)
        if tune:
            c.set_tuning(**tune)
        c.set_vertices(v)
        c.transport(0, n, 321)
        res.append((c.tally(sid), c.stats()))
    (d0, st0), (d1, st1) = res
    assert d0.reshape(700, 20, 20)[600:].sum() > 0.0 and d0.reshape(700, 20, 20)[:100].sum() > 0.0
    np.testing.assert_allclose(d1, d0, rtol=1e-9, atol=1e-300)
    assert st1["steps"] == st0["steps"] and st1["histories"] == n


def test_chunked_primaries_match_single_chunk(gpu_ctx_factory):
    wl = workloads.c2(histories=5000)
    n = 5000
    v = wl.vertices(n, 6)
    out = []
    for chunk in (0, 777):
        c, cid, sid = _ctx_for(wl, gpu_ctx_factory)
        if chunk:
            c.set_tuning(primary_chunk=chunk)
        c.set_vertices(v)
        c.transport(0, n, 4242)
        out.append(c.tally(sid))
    np.testing.assert_allclose(out[1], out[0], rtol=1e-9, atol=1e-300)


def test_history_ranges_add_up(gpu_ctx_factory):
    """transport(0, n) equals transport(0, k) + transport(k, n): histories are independent."""
    wl = workloads.c1()
    n = 2000
    v = wl.vertices(n, 8)
    c, cid, sid = _ctx_for(wl, gpu_ctx_factory)
    c.set_vertices(v)
    c.transport(0, n, 5)
    whole = c.tally(sid)
    c.reset()
    c.transport(0, 700, 5)
    c.transport(700, n, 5)
    np.testing.assert_allclose(c.tally(sid), whole, rtol=1e-9, atol=1e-300)


def test_edge_cases(gpu_ctx_factory):
    wl = workloads.c1()
    c, cid, sid = _ctx_for(wl, gpu_ctx_factory)
    v = wl.vertices(64, 1)
    c.set_vertices(v)
    c.transport(5, 5, 1)                      # empty range is a no-op
    assert c.tally(sid).sum() == 0.0
    miss = v.copy()
    miss["pos"][:, 0] = 500.0                 # beam line outside the phantom: no dose
    c.set_vertices(miss)
    c.transport(0, 64, 1)
    assert c.tally(sid).sum() == 0.0
    assert c.stats()["histories"] == 64
    inside = v.copy()
    inside["pos"][:, 2] = -100.0              # starts inside the grid
    c.set_vertices(inside)
    c.transport(0, 64, 1)
    idd = ph.depth_dose(c.tally(sid), wl.nxyz)
    assert idd[:99].sum() == 0.0 and idd[100:].sum() > 0.0
    with pytest.raises(capi.MqiError):
        c.transport(0, 65, 1)                 # beyond the vertices
    with pytest.raises(capi.MqiError):
        c.add_scorer(7, capi.DOSE_W)          # no such child
    with pytest.raises(capi.MqiError):
        c.add_scorer(cid, 99)                 # unknown plug-in
    c.reset()
    assert c.tally(sid).sum() == 0.0 and c.stats()["histories"] == 0


def test_queue_overflow_is_reported(gpu_ctx_factory):
    """A queue sized below what a generation needs is detected on the device (bounds-checked
    append) and reported as MQI_ERR_OVERFLOW; nothing is written out of bounds."""
    wl = workloads.c1()
    c, cid, sid = _ctx_for(wl, gpu_ctx_factory)
    c.set_physics(False)
    c.set_tuning(primary_chunk=1)             # queue capacity 3 tracks
    v = wl.vertices(2000, 2)
    c.set_vertices(v)
    with pytest.raises(capi.MqiError) as e:
        c.transport(0, 2000, 3)
    assert e.value.code == -6
    c.set_tuning(primary_chunk=4096)          # the context stays usable
    c.reset()
    c.transport(0, 2000, 3)
    assert c.stats()["histories"] == 2000


def test_transport_before_setup_is_a_state_error(gpu_ctx_factory):
    c = gpu_ctx_factory()
    with pytest.raises(capi.MqiError) as e:
        c.transport(0, 0, 1)
    assert e.value.code == -4


def test_gpu_dose_matches_reference_on_the_synthetic_ct(golden, gpu_ctx_factory):
    """Three Gaussian spots on the synthetic CT (heterogeneous HU field, 0.98 x 0.98 x 2 mm,
    release physics) against the reference CPU build: depth dose and a coarse dose in the column
    around each spot within 2% or 3 sigma in bins above 10% of the maximum, R80 within 0.2 mm."""
    gd = golden("dose_c3.npz")
    half, bins = int(gd["crop"]), tuple(int(b) for b in gd["bins"])
    wl = workloads.c3()
    each = int(gd["histories_per_batch"])
    c = gpu_ctx_factory()
    c.set_physics(False)
    cid = c.add_child(*wl.edges())
    c.set_hu(cid, wl.hu)
    sid = c.add_scorer(cid, capi.DOSE_W)
    for k, (x, y, e) in enumerate(gd["spots"]):
        idd, crs = [], []
        for b in range(8):
            c.reset()
            rng = np.random.default_rng(7000 + 10 * k + b)
            c.set_vertices(ph.gaussian_spot_vertices(each, rng, float(e), (float(x), float(y), 195.0), (4.0, 4.0)))
            c.transport(0, each, 99 + 10 * k + b)
            d = c.tally(sid)
            idd.append(ph.depth_dose(d, wl.nxyz) / each)
            crs.append(ph.column_crop(d, wl.lxyz, wl.nxyz, float(x), float(y), half, bins) / each)
        for mine, ref in ((np.array(idd), gd[f"idd{k}"]), (np.array(crs), gd[f"coarse{k}"])):
            tm, ts = mine.mean(0), mine.std(0, ddof=1) / np.sqrt(len(mine))
            rm, rs = ref.mean(0), ref.std(0, ddof=1) / np.sqrt(len(ref))
            sel = rm > 0.1 * rm.max()
            ok = (np.abs(tm - rm) <= 0.02 * rm) | (np.abs(tm - rm) <= 3 * np.sqrt(rs ** 2 + ts ** 2))
            assert ok[sel].mean() >= 0.95, (k, ok[sel].mean())
        tm, rm = np.array(idd).mean(0), gd[f"idd{k}"].mean(0)
        assert abs(ph.r80(tm, 2.0) - ph.r80(rm, 2.0)) <= 0.2, (k, ph.r80(tm, 2.0), ph.r80(rm, 2.0))


@pytest.mark.parametrize("stype", [capi.EDEP, capi.DOSE_W2, capi.DOSE_M, capi.LETD_NUM, capi.LETD_DEN, capi.LETT_NUM,
                                   capi.LETT_DEN, capi.EDEP_PRIMARY, capi.EDEP_SECONDARY])
def test_scorer_plugins_match_the_oracle(oracle, gpu_ctx_factory, stype):
    """Every enum'd scorer callback (scorers/mqi_scorer_energy_deposit.hpp:12-177) against the C
    restatement run on the same Philox streams, history by history.  A history agrees to 1e-4
    unless an ulp-level difference (CUDA's and libm's powf in the SPR, say) flipped a near-tie
    along it: the flip moves deposits between voxels, which conserves energy but not the
    non-linear scorers (dose^2, the LET numerators), so those differ in more histories -- by a
    few 1e-4 typically, by up to a few percent when a step crosses the LET cut of 25."""
    wl = _laterally_coarse(workloads.c2(histories=150), 16)
    n, seed = 150, 0xD0CE
    c, cid, sid = _ctx_for(wl, gpu_ctx_factory, stype)
    v = wl.vertices(n, 41)
    c.set_vertices(v)
    g = np.zeros(n)
    for h in range(n):
        c.reset()
        c.transport(h, h + 1, seed)
        g[h] = c.tally(sid).sum()
    _, o, _ = oracle.transport(_oracle_grid(oracle, wl), v, 0, n, seed, wl.physics_debug, scorer=int(stype),
                               per_history=True)
    assert o.sum() > 0
    rel = np.abs(g - o) / np.maximum(np.abs(o), 1e-30)
    # a flip that moves a deposit between voxels leaves an energy sum alone, changes the scorers
    # that depend on the voxel or the step a little, and the squared or LET-cut ones most
    if stype in (capi.EDEP, capi.EDEP_PRIMARY, capi.EDEP_SECONDARY):
        share = 0.99
    elif stype in (capi.DOSE_W2, capi.LETD_NUM):
        share = 0.8
    else:
        share = 0.95
    print(f"scorer {int(stype)}: {(rel <= 1e-4).mean():.3f} of histories within 1e-4, {(rel <= 5e-2).mean():.3f} within 5e-2")
    assert (rel <= 1e-4).mean() >= share, ((rel <= 1e-4).mean(), np.flatnonzero(rel > 1e-4)[:10])
    assert (rel <= 5e-2).mean() >= 0.99, np.sort(rel)[-6:]
    assert abs(g.sum() - o.sum()) <= 1e-2 * abs(o.sum())
