"""Scorer callbacks and ROI mappings against the reference's own code.

Fixtures are computed by the reference's CPU build (driver modes `hits` and `roi`):
* the ten fp_compute_hit callbacks (moqui/base/scorers/mqi_scorer_energy_deposit.hpp:12-177) on
  seeded step states in a grid with uneven edges and densities from vacuum to bone, including
  zero-length steps, zero deposits and secondaries;
* roi_t::idx and roi_t::get_mask_idx (moqui/base/mqi_roi.hpp:47-71, 87-160) for INDIRECT and
  CONTOUR maps on random voxels.

CPU tests check the reference's numbers against the formulas written out here (FP32 operands,
FP64 accumulation where the reference forms doubles), so the fixture means what the kernels assume.
GPU tests evaluate the transport's own device functions (mqi_eval_hits, mqi_eval_roi) on the same
inputs: ROI indices and every callback but dose_to_water bit-exact; dose_to_water (and the Dij
value) within 4e-7 relative, its square within 8e-7: the kernel forms the per-step dose in FP32
(the constant 1.60218e-10 rounded to FP32, a product and a quotient rounded to FP32: three roundings
of 2^-24 at most) where the reference forms it in double, and CUDA's powf in the stopping-power
ratio is within 2 ulp of the host's.
"""
import numpy as np
import pytest

from moquimc_gb300 import capi, phantom as ph

F = np.float32
TYPES = {"energy_deposit": capi.EDEP, "energy_deposit_primary": capi.EDEP_PRIMARY,
         "energy_deposit_secondary": capi.EDEP_SECONDARY, "dose_to_water": capi.DOSE_W,
         "dose_to_water_square": capi.DOSE_W2, "dose_to_medium": capi.DOSE_M, "LETd_weight1": capi.LETD_NUM,
         "LETd_weight2": capi.LETD_DEN, "LETt_weight1": capi.LETT_NUM, "LETt_weight2": capi.LETT_DEN}


def _case(seed=21, n=20000):
    rng = np.random.default_rng(seed)
    nxyz = (20, 16, 12)
    xe = np.cumsum(np.concatenate([[-30.0], rng.uniform(0.5, 4.0, nxyz[0])])).astype(F)
    ye = np.cumsum(np.concatenate([[-20.0], rng.uniform(0.5, 4.0, nxyz[1])])).astype(F)
    ze = np.cumsum(np.concatenate([[-40.0], rng.uniform(0.5, 4.0, nxyz[2])])).astype(F)
    nv = int(np.prod(nxyz))
    rho = rng.uniform(1e-4, 2.2e-3, nv).astype(F)
    rho[rng.random(nv) < 0.1] = F(1e-9)                   # vacuum voxels
    rho[rng.random(nv) < 0.1] = F(0.001)                  # water (the debug shortcut)
    cnb = rng.integers(0, nv, n).astype(np.uint32)
    steps = np.zeros((n, 9), F)
    steps[:, 0] = rng.uniform(0.05, 250.0, n)
    steps[:, 1] = rng.exponential(0.5, n) * (rng.random(n) > 0.05)
    steps[:, 2] = rng.exponential(0.1, n) * (rng.random(n) < 0.2)
    steps[:, 3:6] = rng.uniform(-30.0, 30.0, (n, 3))
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    length = rng.exponential(1.0, n) * (rng.random(n) > 0.05)  # some zero-length steps
    steps[:, 6:9] = (steps[:, 3:6] + d * length[:, None]).astype(F)
    primary = (rng.random(n) < 0.7).astype(np.int32)
    return nxyz, (xe, ye, ze), rho, steps, cnb, primary


@pytest.fixture(scope="module", params=[False, True], ids=["release", "debug"])
def hits(request, oracle):
    if not oracle.ref_available():
        pytest.skip("the reference's staged sources are not present")
    nxyz, edges, rho, steps, cnb, primary = _case()
    ref = oracle.ref_hits(nxyz, *edges, rho, steps, cnb, primary, debug=request.param)
    return request.param, nxyz, edges, rho, steps, cnb, primary, ref


def _volume(edges, nxyz, cnb):
    xe, ye, ze = edges
    nx, ny = nxyz[0], nxyz[1]
    i, j, k = cnb % nx, (cnb // nx) % ny, cnb // (nx * ny)
    return ((xe[i + 1] - xe[i]) * (ye[j + 1] - ye[j])).astype(F) * (ze[k + 1] - ze[k])


def test_reference_callbacks_follow_the_formulas(hits):
    dbg, nxyz, edges, rho, steps, cnb, primary, ref = hits
    dE, ldE = steps[:, 1], steps[:, 2]
    np.testing.assert_array_equal(ref["energy_deposit"], (dE + ldE).astype(F).astype(np.float64))
    np.testing.assert_array_equal(ref["energy_deposit_primary"], np.where(primary != 0, dE, 0).astype(np.float64))
    np.testing.assert_array_equal(ref["energy_deposit_secondary"], np.where(primary == 0, dE, 0).astype(np.float64))
    r = rho[cnb]
    vol = _volume(edges, nxyz, cnb)
    dm = np.where(primary != 0, dE.astype(np.float64) * 1.60218e-13 * 1000.0 / (vol * r).astype(F), 0.0)
    np.testing.assert_array_equal(ref["dose_to_medium"], dm)
    dd = (steps[:, 6:9] - steps[:, 3:6]).astype(F)
    sq = (dd * dd).astype(F).astype(np.float64)
    length = np.sqrt((sq[:, 0] + sq[:, 1]) + sq[:, 2])
    dens = (r * F(1000.0)).astype(F).astype(np.float64)
    ok = length > 0
    with np.errstate(divide="ignore", invalid="ignore"):
        let = dE.astype(np.float64) / length / dens
        np.testing.assert_array_equal(ref["LETt_weight2"], np.where(ok, length, 0.0))
        np.testing.assert_array_equal(ref["LETt_weight1"], np.where(ok, length * let, 0.0))
        np.testing.assert_array_equal(ref["LETd_weight2"], np.where(ok & (let < 25.0), dE.astype(np.float64), 0.0))
        np.testing.assert_array_equal(ref["LETd_weight1"], np.where(ok & (let < 25.0), dE * let, 0.0))
    dw = ref["dose_to_water"]
    assert (dw[r < F(1e-7)] == 0).all() and (dw[r >= F(1e-7)] >= 0).all()
    np.testing.assert_allclose(ref["dose_to_water_square"], dw * dw, rtol=1e-15, atol=0)


@pytest.mark.gpu
def test_device_callbacks_match_the_reference(hits, gpu_ctx_factory):
    dbg, nxyz, edges, rho, steps, cnb, primary, ref = hits
    c = gpu_ctx_factory()
    c.set_physics(dbg)
    cid = c.add_child(*edges)
    c.set_density(cid, rho)
    for name, t in TYPES.items():
        got = c.eval_hits(cid, t, steps, cnb, primary)
        if name == "dose_to_water":
            np.testing.assert_allclose(got, ref[name], rtol=4e-7, atol=0, err_msg=name)
            np.testing.assert_allclose(c.eval_hits(cid, capi.DIJ, steps, cnb, primary), ref[name], rtol=4e-7, atol=0)
            assert np.mean(got == ref[name]) < 1.0   # formed in FP32: not the double result
        elif name == "dose_to_water_square":
            np.testing.assert_allclose(got, ref[name], rtol=8e-7, atol=0, err_msg=name)
        else:
            np.testing.assert_array_equal(got, ref[name], err_msg=name)


def _contour(rng, nv, n_runs=40):
    starts = np.sort(rng.choice(np.arange(50, nv - 50), n_runs, replace=False)).astype(np.uint32)
    gaps = np.diff(np.concatenate([starts, [nv]]))
    stride = np.minimum(rng.integers(1, 60, n_runs), gaps).astype(np.uint32)
    acc = np.cumsum(stride).astype(np.uint32)
    return starts, stride, acc


@pytest.fixture(scope="module")
def roi_case(oracle):
    if not oracle.ref_available():
        pytest.skip("the reference's staged sources are not present")
    rng = np.random.default_rng(33)
    nxyz = (30, 20, 10)
    nv = int(np.prod(nxyz))
    vox = rng.integers(0, nv, 20000).astype(np.uint32)
    start, stride, acc = _contour(rng, nv)
    contour = (start, stride, acc) + oracle.ref_roi(capi.ROI_CONTOUR, nv, start, stride, acc, vox)
    ind = np.full(nv, 0xFFFFFFFF, np.uint32)
    sel = rng.random(nv) < 0.3
    ind[sel] = np.arange(int(sel.sum()), dtype=np.uint32)
    indirect = (ind,) + oracle.ref_roi(capi.ROI_INDIRECT, nv, ind, None, None, vox)
    return nxyz, vox, contour, indirect


def test_reference_roi_maps(roi_case):
    nxyz, vox, (start, stride, acc, idx, mask), (ind, iidx, imask) = roi_case
    v = vox.astype(np.int64)
    run = np.searchsorted(start, v, side="right") - 1
    first = start[np.maximum(run, 0)].astype(np.int64)
    inside = (run >= 0) & (v - first < stride[np.maximum(run, 0)])
    prev = np.where(run > 0, acc[np.maximum(run - 1, 0)], 0).astype(np.int64)
    expect = np.where(inside, v - first + prev, -1)
    np.testing.assert_array_equal(mask, expect)
    above = vox >= start[0]   # below the first run the reference's idx reads before its array
    np.testing.assert_array_equal(idx[above], np.where(inside, 1, -1)[above])
    np.testing.assert_array_equal(iidx, ind[vox].astype(np.int32))
    np.testing.assert_array_equal(imask, ind[vox].astype(np.int32))


@pytest.mark.gpu
def test_device_roi_maps_match_the_reference(roi_case, gpu_ctx_factory):
    nxyz, vox, (start, stride, acc, idx, mask), (ind, iidx, imask) = roi_case
    c = gpu_ctx_factory()
    edges = [ph.uniform_edges(0.0, float(n), n) for n in nxyz]
    cid = c.add_child(*edges)
    c.set_density(cid, np.full(int(np.prod(nxyz)), 0.001, np.float32))
    sc = c.add_scorer(cid, capi.DOSE_W, capi.ROI_CONTOUR, start=start, stride=stride, acc=acc)
    si = c.add_scorer(cid, capi.DOSE_W, capi.ROI_INDIRECT, start=ind)
    gi, gm = c.eval_roi(sc, vox)
    np.testing.assert_array_equal(gm, mask)
    above = vox >= start[0]
    np.testing.assert_array_equal(gi[above], idx[above])
    assert (gi[~above] == -1).all()            # the transport does not score there
    gi, gm = c.eval_roi(si, vox)
    np.testing.assert_array_equal(gi, iidx)
    np.testing.assert_array_equal(gm, imask)
