"""GPU tests of the Dij scorer: the (voxel, spot) table against the reference's own insertion and
writer replaying the GPU's recorded insertions (bit-exact sparsity pattern for identical tracks),
and against per-spot dense runs, the CSR layouts, the products D.w and D^T.g against dense
references, the torch.autograd.Function against central finite differences, and the table-full
error."""
import numpy as np
import pytest

from moquimc_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _spots(n_spots, histories, seed=0, energy=(110.0, 170.0), pitch=6.0):
    rng = np.random.default_rng(seed)
    sp = np.zeros(n_spots, capi.SPOT_DTYPE)
    side = int(np.ceil(np.sqrt(n_spots)))
    for s in range(n_spots):
        sp[s]["mean"][:3] = [(s % side - 0.5 * (side - 1)) * pitch, (s // side - 0.5 * (side - 1)) * pitch, 0.5]
    sp["sigma"][:, 0] = 4.0
    sp["sigma"][:, 1] = 4.0
    sp["energy"] = rng.uniform(*energy, n_spots).astype(np.float32)
    sp["rot"] = np.eye(3, dtype=np.float32).ravel()
    sp["histories"] = histories
    return sp


def _ctx(make, wl):
    c = make()
    c.set_physics(wl.physics_debug)
    cid = c.add_child(*wl.edges())
    c.set_hu(cid, wl.hu)
    return c, cid


@pytest.fixture(scope="module")
def wl():
    return workloads.c2(histories=10_000)


def _csr(op):
    import scipy.sparse as sps

    indptr, indices, data = op.csr()
    return sps.csr_matrix((data, indices, indptr), shape=(op.n_spots, op.n_voxels))


def test_dij_rows_equal_per_spot_dense_runs(gpu_ctx_factory, wl):
    sp = _spots(3, [4000, 2500, 3500], seed=1)
    c, cid = _ctx(gpu_ctx_factory, wl)
    dij = c.add_dij_scorer(cid, capacity=1 << 22)
    N = c.set_spot_plan(sp)
    c.transport_plan(0, N, 11)
    op = c.dij_build(dij)
    indptr, indices, data = op.csr()
    assert indptr[0] == 0 and indptr[-1] == op.nnz == len(indices)
    info = c.dij_info(dij)
    assert info["occupied"] == op.nnz and info["table_slots"] == 1 << 22
    cum = c.plan_cum
    for s in range(len(sp)):
        d, did = _ctx(gpu_ctx_factory, wl)
        dose = d.add_scorer(did, capi.DOSE_W)
        d.set_spot_plan(sp)
        d.transport_plan(int(cum[s]), int(cum[s + 1]), 11)       # the same histories, the same tracks
        ref = d.tally(dose)
        row = slice(int(indptr[s]), int(indptr[s + 1]))
        vox = indices[row].astype(np.int64)
        assert (np.diff(vox) > 0).all()                           # voxels ascending within a row
        np.testing.assert_array_equal(vox, np.flatnonzero(ref))   # bit-exact sparsity pattern
        np.testing.assert_allclose(data[row], ref[vox], rtol=2.0 ** -23, atol=0)


def test_dij_sparsity_matches_the_reference_table(gpu_ctx_factory, oracle, tmp_path):
    """Bit-exact Dij sparsity against the reference's own code for identical tracks: every
    insertion the GPU makes during a plan transport on a heterogeneous CT crop (air, tissue noise)
    is recorded, replayed in the same order through the reference's insert_hashtable (CPU branch,
    mqi_transport.hpp:68-111) and written by its save_to_npz (mqi_io.hpp:249-320).  The reference
    file's (spot, voxel) key set equals the GPU matrix's, its values agree to the matrix's FP32
    rounding, and the GPU table holds one slot per key."""
    if not oracle.ref_available():
        pytest.skip("the reference's staged sources are not present")
    nxyz, dxyz = (96, 96, 100), (0.98, 0.98, 2.0)
    hu = workloads.ct_hu(nxyz, dxyz, semi=(40.0, 35.0, 90.0), seed=12)
    from moquimc_gb300 import phantom as ph

    lxyz = tuple(float(np.float32(n * d)) for n, d in zip(nxyz, dxyz))
    edges = ph.phantom_box_edges(lxyz, (0.0, 0.0, 0.0), nxyz)
    sp = _spots(6, [800, 500, 1200, 300, 900, 600], seed=9, energy=(90.0, 160.0), pitch=12.0)
    sp["mean"][:, 2] = 99.5                                     # just outside the grid's top face
    c = gpu_ctx_factory()
    c.set_physics(False)
    cid = c.add_child(*edges)
    c.set_hu(cid, hu)
    dij = c.add_dij_scorer(cid, capacity=1 << 22)
    c.dij_record_hits(dij, 1 << 24)
    N = c.set_spot_plan(sp)
    c.transport_plan(0, N, 17)
    vox, spot, val = c.dij_hits(dij)
    assert len(vox) > 100_000 and (val > 0).all()
    op = c.dij_build(dij)
    indptr, indices, data = op.csr()
    path = oracle.ref_dij(vox, spot, val, 1 << 22, len(sp), nxyz, str(tmp_path))
    z = np.load(path)
    assert list(z["shape"]) == [len(sp), int(np.prod(nxyz))]
    for s in range(len(sp)):
        rv = z["indices"][z["indptr"][s]:z["indptr"][s + 1]].astype(np.int64)
        rd = z["data"][z["indptr"][s]:z["indptr"][s + 1]]
        order = np.argsort(rv)
        gv = indices[indptr[s]:indptr[s + 1]].astype(np.int64)
        np.testing.assert_array_equal(gv, rv[order])           # the key set, bit-exact
        np.testing.assert_allclose(data[indptr[s]:indptr[s + 1]], rd[order], rtol=2.0 ** -23, atol=0)
    assert c.dij_info(dij)["occupied"] == len(z["indices"]) == op.nnz


def test_dij_products_match_dense_references(gpu_ctx_factory, wl):
    import scipy.sparse as sps  # noqa: F401

    sp = _spots(9, 1500, seed=2)
    c, cid = _ctx(gpu_ctx_factory, wl)
    dij = c.add_dij_scorer(cid, capacity=1 << 23)
    N = c.set_spot_plan(sp)
    c.transport_plan(0, N, 3)
    op = c.dij_build(dij, scale=1e6)
    A = _csr(op).astype(np.float64)                              # [n_spots, n_voxels] = D^T
    rng = np.random.default_rng(5)
    w = rng.uniform(0.5, 1.5, op.n_spots)
    g = rng.standard_normal(op.n_voxels)
    ref_d = A.T @ w
    ref_g = A @ g
    d64 = c.dij_matvec(dij, w.astype(np.float64), op.n_voxels)
    np.testing.assert_allclose(d64, ref_d, rtol=1e-12, atol=1e-12 * np.abs(ref_d).max())
    d32 = c.dij_matvec(dij, w.astype(np.float32), op.n_voxels)
    np.testing.assert_allclose(d32, ref_d, rtol=1e-5, atol=1e-6 * np.abs(ref_d).max())
    g64 = c.dij_rmatvec(dij, g.astype(np.float64), op.n_spots)
    np.testing.assert_allclose(g64, ref_g, rtol=1e-11, atol=1e-11 * np.abs(ref_g).max())
    g32 = c.dij_rmatvec(dij, g.astype(np.float32), op.n_spots)
    np.testing.assert_allclose(g32, ref_g, rtol=1e-4, atol=1e-5 * np.abs(ref_g).max())
    # fixed reduction orders: repeated products give identical bits (the backward's warps take its
    # segments from a shared cursor, in whatever order they get there)
    for _ in range(3):
        np.testing.assert_array_equal(c.dij_rmatvec(dij, g.astype(np.float32), op.n_spots), g32)
        np.testing.assert_array_equal(c.dij_rmatvec(dij, g.astype(np.float64), op.n_spots), g64)
        np.testing.assert_array_equal(c.dij_matvec(dij, w.astype(np.float32), op.n_voxels), d32)
    # unit weights reproduce the dense dose of the same run (FP32 matrix entries)
    e, eid = _ctx(gpu_ctx_factory, wl)
    dose = e.add_scorer(eid, capi.DOSE_W)
    e.set_spot_plan(sp)
    e.transport_plan(0, N, 3)
    dense = e.tally(dose) * 1e6
    np.testing.assert_allclose(c.dij_matvec(dij, np.ones(op.n_spots), op.n_voxels), dense, rtol=1e-6,
                               atol=1e-9 * dense.max())


def test_dij_products_with_long_voxel_rows(gpu_ctx_factory, wl):
    """3000 one-history spots on one axis through voxel centres: the voxels near the entrance get
    rows of nearly 3000 entries, longer than what one forward block stages (the rows' run then
    exceeds the staging buffer and is summed from global memory), beside short rows that are
    staged."""
    sp = _spots(3000, 1, seed=4, energy=(140.0, 141.0))
    sp["mean"][:, :2] = 0.5
    sp["sigma"][:, :2] = 0.02
    c, cid = _ctx(gpu_ctx_factory, wl)
    dij = c.add_dij_scorer(cid, capacity=1 << 23)
    N = c.set_spot_plan(sp)
    c.transport_plan(0, N, 9)
    op = c.dij_build(dij, scale=1e6)
    A = _csr(op).astype(np.float64)
    row_len = np.diff(A.T.tocsr().indptr)
    assert row_len.max() > 2048 and (row_len > 0).sum() > 100
    rng = np.random.default_rng(6)
    w = rng.uniform(0.5, 1.5, op.n_spots)
    ref_d = A.T @ w
    d32 = c.dij_matvec(dij, w.astype(np.float32), op.n_voxels)
    np.testing.assert_allclose(d32, ref_d, rtol=1e-5, atol=1e-6 * np.abs(ref_d).max())
    d64 = c.dij_matvec(dij, w.astype(np.float64), op.n_voxels)
    np.testing.assert_allclose(d64, ref_d, rtol=1e-12, atol=1e-12 * np.abs(ref_d).max())
    g = rng.standard_normal(op.n_voxels)
    g32 = c.dij_rmatvec(dij, g.astype(np.float32), op.n_spots)
    np.testing.assert_allclose(g32, A @ g, rtol=1e-4, atol=1e-5 * np.abs(A @ g).max())


def test_dij_autograd_matches_finite_differences(gpu_ctx_factory, wl):
    """Quadratic objective on D.w: the hand-written D^T.g backward against central differences
    (h = 1e-3) evaluated with the FP64 forward product, and against the dense gradient."""
    torch = pytest.importorskip("torch")
    from moquimc_gb300 import dij as dijmod

    sp = _spots(16, 1200, seed=3)
    c, cid = _ctx(gpu_ctx_factory, wl)
    sid = c.add_dij_scorer(cid, capacity=1 << 23)
    N = c.set_spot_plan(sp)
    c.transport_plan(0, N, 9)
    op = c.dij_build(sid, scale=1e9)
    dev = torch.device("cuda:0")
    w = torch.full((op.n_spots,), 1.0, device=dev, dtype=torch.float32, requires_grad=True)
    d0 = op.matvec(w.detach())
    target = torch.zeros(op.n_voxels, dtype=torch.bool, device=dev)
    hot = d0 > 0.3 * d0.max()
    target[hot] = True
    presc = float(d0[hot].mean()) * 1.2

    def objective(dose):
        return ((dose[target] - presc) ** 2).sum() + 0.1 * (torch.relu(dose[~target] - 0.5 * presc) ** 2).sum()

    f = objective(dijmod.dose(op, w))
    f.backward()
    grad = w.grad.double().cpu().numpy()
    h = 1e-3
    fd = np.empty(op.n_spots)
    w64 = w.detach().double()
    for s in range(op.n_spots):
        e = torch.zeros_like(w64)
        e[s] = h
        fp = objective(op.matvec(w64 + e)).item()
        fm = objective(op.matvec(w64 - e)).item()
        fd[s] = (fp - fm) / (2 * h)
    rel = np.abs(grad - fd) / np.maximum(np.abs(fd), 1e-12 * np.abs(fd).max())
    assert rel.max() < 1e-4, rel
    # dense reference gradient: D^T . dobjective/ddose in numpy FP64
    A = _csr(op).astype(np.float64)
    dose64 = A.T @ np.ones(op.n_spots)
    tg = target.cpu().numpy()
    gd = np.where(tg, 2 * (dose64 - presc), 0.2 * np.maximum(dose64 - 0.5 * presc, 0.0))
    np.testing.assert_allclose(grad, A @ gd, rtol=1e-4, atol=1e-6 * np.abs(A @ gd).max())


def test_dij_products_are_ordered_with_torch_work(gpu_ctx_factory, wl):
    """Chained device products on torch's default stream equal the synchronous host path."""
    torch = pytest.importorskip("torch")
    sp = _spots(9, 1500, seed=7)
    c, cid = _ctx(gpu_ctx_factory, wl)
    sid = c.add_dij_scorer(cid, capacity=1 << 23)
    N = c.set_spot_plan(sp)
    c.transport_plan(0, N, 4)
    op = c.dij_build(sid, scale=1e6)
    dev = torch.device("cuda:0")
    host_d = c.dij_matvec(sid, np.ones(op.n_spots, np.float32), op.n_voxels)
    host_g = c.dij_rmatvec(sid, host_d, op.n_spots)
    for _ in range(3):
        d = op.matvec(torch.ones(op.n_spots, device=dev))
        g = op.rmatvec(d * 1.0)
        np.testing.assert_array_equal(d.cpu().numpy(), host_d)
        np.testing.assert_allclose(g.cpu().numpy(), host_g, rtol=1e-6)


def test_dij_save_npz_loads_as_scipy_csr(gpu_ctx_factory, wl, tmp_path):
    sps = pytest.importorskip("scipy.sparse")
    sp = _spots(2, 500, seed=4)
    c, cid = _ctx(gpu_ctx_factory, wl)
    sid = c.add_dij_scorer(cid, capacity=1 << 20)
    c.set_spot_plan(sp)
    c.transport_plan(0, 1000, 1)
    op = c.dij_build(sid)
    op.save_npz(str(tmp_path / "dij.npz"))
    m = sps.load_npz(str(tmp_path / "dij.npz"))
    assert m.shape == (2, op.n_voxels) and m.nnz == op.nnz and m.has_sorted_indices
    indptr, indices, data = op.csr()
    np.testing.assert_array_equal(m.indices, indices)
    np.testing.assert_array_equal(m.data, data)


def test_dij_table_full_is_an_error(gpu_ctx_factory, wl):
    sp = _spots(1, 100, seed=5)
    c, cid = _ctx(gpu_ctx_factory, wl)
    sid = c.add_dij_scorer(cid, capacity=256)
    c.set_spot_plan(sp)
    with pytest.raises(capi.MqiError) as ei:
        c.transport_plan(0, 100, 1)
    assert ei.value.code == capi.MQI_ERR_OVERFLOW
    # the context stays usable
    c.reset()
    assert c.dij_info(sid)["occupied"] == 0
