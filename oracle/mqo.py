"""ctypes binding of the C restatement (oracle/mqi_oracle.c) and runners for the reference's own
CPU build (oracle/_ref/bin).  TEST INFRASTRUCTURE: only tests, the smoke check and the bench's
CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import struct
import subprocess
import tempfile
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys_path_added = False


def _build():
    import sys

    sys.path.insert(0, HERE)
    import build_oracle  # noqa: E402

    return build_oracle


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("xe", C.c_void_p), ("ye", C.c_void_p),
                ("ze", C.c_void_p), ("rho", C.c_void_p)]


class _Calib(C.Structure):
    _fields_ = [("n_rho", C.c_uint32), ("n_e", C.c_uint32), ("rho0", C.c_float), ("drho", C.c_float),
                ("e0", C.c_float), ("de", C.c_float), ("spr", C.c_void_p), ("x0", C.c_void_p)]


class _Cfg(C.Structure):
    _fields_ = [("physics_debug", C.c_int), ("scorer", C.c_int), ("calib", C.POINTER(_Calib))]


class _Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("histories", "tracks", "steps", "pushed", "dropped")]


_libs = {}


def lib(fp64: bool = False):
    """The C restatement: FP32 stepping, or the all-FP64 build (same source, -DMQO_FP64)."""
    if fp64 not in _libs:
        path = _build().build_restatement(fp64=fp64)
        L = C.CDLL(path)
        L.mqo_transport.restype = C.c_int
        L.mqo_transport.argtypes = [C.POINTER(_Grid), C.POINTER(_Cfg), C.c_void_p, C.c_uint64, C.c_uint64,
                                    C.c_uint64, C.c_void_p, C.c_void_p, C.POINTER(_Stats)]
        L.mqo_eval_physics.restype = None
        L.mqo_eval_physics.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
        L.mqo_spr.restype = C.c_float
        L.mqo_spr.argtypes = [C.c_float, C.c_float, C.c_int]
        L.mqo_x0.restype = C.c_float
        L.mqo_x0.argtypes = [C.c_float, C.c_int]
        L.mqo_hu_to_density.restype = C.c_float
        L.mqo_hu_to_density.argtypes = [C.c_int]
        L.mqo_sample.restype = C.c_int
        L.mqo_sample.argtypes = [C.c_int, C.c_float, C.c_float, C.c_uint64, C.c_uint64, C.c_int, C.c_void_p]
        L.mqo_philox.restype = None
        L.mqo_philox.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.mqo_trace_ray.restype = C.c_int
        L.mqo_trace_ray.argtypes = [C.POINTER(_Grid), C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        _libs[fp64] = L
    return _libs[fp64]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Grid:
    def __init__(self, xe, ye, ze, rho):
        self.xe = np.ascontiguousarray(xe, np.float32)
        self.ye = np.ascontiguousarray(ye, np.float32)
        self.ze = np.ascontiguousarray(ze, np.float32)
        self.rho = np.ascontiguousarray(rho, np.float32).reshape(-1)
        self.c = _Grid(len(self.xe) - 1, len(self.ye) - 1, len(self.ze) - 1, _p(self.xe).value, _p(self.ye).value,
                       _p(self.ze).value, _p(self.rho).value)


def transport(grid: Grid, vertices: np.ndarray, h0: int, h1: int, seed: int, physics_debug: bool, scorer: int = 2,
              per_history: bool = False, fp64: bool = False, calib=None):
    """Run the C restatement (the all-FP64 build with fp64; `calib` an object with n_rho, n_e, rho0,
    drho, e0, de, spr, x0 for tabulated SPR / X0 curves); returns (tally, per_history_sums or None,
    stats dict)."""
    v = np.ascontiguousarray(vertices).view(np.float32).reshape(-1, 7)
    tally = np.zeros(grid.rho.size, np.float64)
    ph = np.zeros(h1 - h0, np.float64) if per_history else None
    st = _Stats()
    cfg = _Cfg(int(physics_debug), scorer, None)
    if calib is not None:
        spr = np.ascontiguousarray(calib.spr, np.float32)
        x0 = np.ascontiguousarray(calib.x0, np.float32)
        cal = _Calib(calib.n_rho, calib.n_e, calib.rho0, calib.drho, calib.e0, calib.de, _p(spr).value, _p(x0).value)
        cfg.calib = C.pointer(cal)
    rc = lib(fp64).mqo_transport(C.byref(grid.c), C.byref(cfg), _p(v), h0, h1, seed, _p(tally),
                             None if ph is None else _p(ph), C.byref(st))
    if rc != 0:
        raise RuntimeError(f"mqo_transport failed: {rc}")
    return tally, ph, {n: int(getattr(st, n)) for n, _ in st._fields_}


def eval_physics(energies: np.ndarray, fp64: bool = False) -> np.ndarray:
    e = np.ascontiguousarray(energies, np.float32)
    out = np.empty((len(e), 8), np.float32)
    lib(fp64).mqo_eval_physics(_p(e), len(e), _p(out))
    return out


def spr(rho: float, ke: float, dbg: bool) -> float:
    return lib().mqo_spr(rho, ke, int(dbg))


def x0(rho: float, dbg: bool) -> float:
    return lib().mqo_x0(rho, int(dbg))


def hu_to_density(hu: int) -> float:
    return lib().mqo_hu_to_density(int(hu))


def philox(counter, key) -> np.ndarray:
    """One Philox4x32-10 block of the restatement's generator."""
    c = np.ascontiguousarray(counter, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().mqo_philox(_p(c), _p(k), _p(out))
    return out


SAMPLE_QUANTITIES = {0: ("along_dE", "along_cos"), 1: ("delta_Te",), 2: ("pp_dE", "pp_cos3", "pp_cos4"),
                     3: ("poe_dE", "poe_cos3"), 4: ("poi_n", "poi_e2", "poi_dep")}


def sample(process: int, ke: float, n: int, seed: int, rho: float = 0.001, physics_debug: bool = False) -> dict:
    """The restatement's draws of one process (mqo_sample): {quantity name: float32 array of n}."""
    names = SAMPLE_QUANTITIES[process]
    out = np.zeros(len(names) * n, np.float32)
    rc = lib().mqo_sample(process, ke, rho, n, seed, int(physics_debug), _p(out))
    if rc != 0:
        raise RuntimeError(f"mqo_sample failed: {rc}")
    return {k: out[i * n:(i + 1) * n] for i, k in enumerate(names)}


def ref_sample(n: int, seed: int, debug: bool = False) -> dict:
    """The reference's own draws (driver mode `sample`): {(energy, quantity name): float32 array}
    at 10, 50 and 150 MeV in water."""
    names = ["along_dE", "along_cos", "delta_Te", "pp_dE", "pp_cos3", "pp_cos4", "poe_dE", "poe_cos3", "poi_n",
             "poi_e2", "poi_dep"]
    with tempfile.TemporaryDirectory() as td:
        o = os.path.join(td, "sample.bin")
        subprocess.run([ref_binary(debug), "sample", o, str(n), str(seed)], check=True, capture_output=True)
        vecs = read_vecs(o, [np.float32] * (3 * len(names)))
    return {(e, k): vecs[i * len(names) + j] for i, e in enumerate((10.0, 50.0, 150.0)) for j, k in enumerate(names)}


def trace_rays(grid: Grid, rays: np.ndarray, max_steps: int):
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    offs = [0]
    cnbs, dists, cells = [], [], []
    cnb = np.zeros(max_steps, np.uint64)
    dist = np.zeros(max_steps, np.float32)
    cell = np.zeros((max_steps, 3), np.int32)
    for r in rays:
        r = np.ascontiguousarray(r)
        k = lib().mqo_trace_ray(C.byref(grid.c), _p(r), max_steps, _p(cnb), _p(dist), _p(cell))
        cnbs.append(cnb[:k].copy())
        dists.append(dist[:k].copy())
        cells.append(cell[:k].copy())
        offs.append(offs[-1] + k)
    cat = lambda xs, dt, shp: np.concatenate(xs) if xs else np.zeros(shp, dt)  # noqa: E731
    return (np.asarray(offs, np.int64), cat(cnbs, np.uint64, (0,)), cat(dists, np.float32, (0,)),
            cat(cells, np.int32, (0, 3)))


# ---- the reference's own CPU build ------------------------------------------------------------

def ref_available() -> bool:
    b = _build()
    return os.path.exists(b.ref_binary(True)) or b.build_reference()


def ref_binary(debug: bool) -> str:
    b = _build()
    path = b.ref_binary(debug)
    if not os.path.exists(path):
        b.build_reference()
    return path


def write_vecs(path, arrays):
    """Arrays in the drivers' vector format: a u64 element count, then the elements."""
    with open(path, "wb") as f:
        for a in arrays:
            a = np.ascontiguousarray(a)
            f.write(struct.pack("<Q", a.size))
            f.write(a.tobytes())


def ref_dij(voxel, spot, value, capacity: int, n_spots: int, nxyz, out_dir: str, scale: float = 1.0,
            name: str = "ref_dij") -> str:
    """Replay Dij insertions (voxel, spot, value) through the reference's insert_hashtable into a
    table of `capacity` slots and write it with the reference's save_to_npz; returns the npz path."""
    hits = os.path.join(out_dir, name + "_hits.bin")
    write_vecs(hits, [np.asarray(voxel, np.uint32), np.asarray(spot, np.uint32), np.asarray(value, np.float64)])
    subprocess.run([ref_binary(False), "dij", hits, str(int(capacity)), str(int(n_spots)), *map(str, nxyz), repr(scale),
                    out_dir, name], check=True, capture_output=True)
    return os.path.join(out_dir, name + ".npz")


HIT_FUNCTIONS = ("energy_deposit", "energy_deposit_primary", "energy_deposit_secondary", "dose_to_water",
                 "dose_to_water_square", "dose_to_medium", "LETd_weight1", "LETd_weight2", "LETt_weight1",
                 "LETt_weight2")


def ref_hits(nxyz, xe, ye, ze, rho, steps, cnb, primary, debug: bool = False) -> dict:
    """The reference's scorer callbacks on step states (driver mode `hits`): {name: float64 array}."""
    with tempfile.TemporaryDirectory() as td:
        i, o = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_vecs(i, [np.asarray(nxyz, np.int32), np.asarray(xe, np.float32), np.asarray(ye, np.float32),
                       np.asarray(ze, np.float32), np.asarray(rho, np.float32).reshape(-1),
                       np.asarray(steps, np.float32).reshape(-1), np.asarray(cnb, np.uint32),
                       np.asarray(primary, np.int32)])
        subprocess.run([ref_binary(debug), "hits", i, o], check=True, capture_output=True)
        vecs = read_vecs(o, [np.float64] * len(HIT_FUNCTIONS))
    return dict(zip(HIT_FUNCTIONS, vecs))


def ref_roi(method: int, original_length: int, start, stride, acc, voxels):
    """roi_t::idx and get_mask_idx from the reference's own roi_t (driver mode `roi`)."""
    with tempfile.TemporaryDirectory() as td:
        i, o = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_vecs(i, [np.asarray([method, original_length], np.int32), np.asarray(start, np.uint32),
                       np.asarray(stride if stride is not None else [], np.uint32),
                       np.asarray(acc if acc is not None else [], np.uint32), np.asarray(voxels, np.uint32)])
        subprocess.run([ref_binary(False), "roi", i, o], check=True, capture_output=True)
        idx, mask = read_vecs(o, [np.int32, np.int32])
    return idx, mask


def write_rays(path, grid_bounds, nxyz, max_steps, rays):
    with open(path, "wb") as f:
        f.write(np.asarray(grid_bounds, np.float32).tobytes())
        f.write(np.asarray(nxyz, np.int32).tobytes())
        f.write(struct.pack("<I", max_steps))
        r = np.ascontiguousarray(rays, np.float32).reshape(-1)
        f.write(struct.pack("<Q", r.size))
        f.write(r.tobytes())


def read_vecs(path, dtypes):
    out = []
    with open(path, "rb") as f:
        for dt in dtypes:
            n = struct.unpack("<Q", f.read(8))[0]
            out.append(np.frombuffer(f.read(n * np.dtype(dt).itemsize), dtype=dt).copy())
    return out


def ref_trace_rays(grid_bounds, nxyz, rays, max_steps):
    with tempfile.TemporaryDirectory() as td:
        i, o = os.path.join(td, "rays.bin"), os.path.join(td, "out.bin")
        write_rays(i, grid_bounds, nxyz, max_steps, rays)
        subprocess.run([ref_binary(True), "raywalk", i, o], check=True, capture_output=True)
        off, cnb, dist, cells = read_vecs(o, [np.int64, np.uint64, np.float32, np.int32])
    return off, cnb, dist, cells.reshape(-1, 3)


def ref_phantom_cmd(debug: bool, lxyz, pxyz, nxyz, energy, position, size, histories, phantom_path, out_dir, seed,
                    beam="uniform", beamline: Optional[str] = None):
    cmd = [ref_binary(debug), "phantom", "--lxyz", *map(str, lxyz), "--pxyz", *map(str, pxyz), "--nxyz",
           *map(str, nxyz), "--spot_energy", str(energy), "0", "--spot_position", *map(str, position),
           "--spot_size", *map(str, size), "--histories", str(histories), "--phantom_path", phantom_path,
           "--output_prefix", out_dir, "--random_seed", str(seed), "--beam", beam, "--json",
           os.path.join(out_dir, "run.json")]
    if beamline:
        cmd += ["--beamline", beamline]
    return cmd


def write_beamline_file(path: str, devices) -> None:
    """Write devices (moquimc_gb300.beamline.children_from_devices tuples) in the format of
    ref_driver's --beamline option."""
    with open(path, "w") as f:
        for d in devices:
            if d[0] == "rangeshifter":
                _, lo, hi, dens, ang, tr = d
                box = [lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]]
                f.write("rangeshifter " + " ".join(repr(float(np.float32(v))) for v in (*box, dens, *ang, *tr)) + "\n")
            else:
                _, center, volume, openings, ang, tr = d
                vals = [*center, *volume, *ang, *tr]
                f.write("aperture " + " ".join(repr(float(np.float32(v))) for v in vals) + f" {len(openings)}")
                for poly in openings:
                    p = np.asarray(poly, np.float32)
                    f.write(f" {len(p)} " + " ".join(repr(float(v)) for v in p.reshape(-1)))
                f.write("\n")


def _beamline_children(beamline: Optional[str]) -> int:
    if not beamline:
        return 0
    with open(beamline) as f:
        return sum(1 for line in f if line.split())


def ref_phantom_parallel(debug: bool, lxyz, pxyz, nxyz, energy, position, size, histories_each, n_proc, hu,
                         seed0, beam="uniform", workdir: Optional[str] = None, beamline: Optional[str] = None):
    """Run n_proc reference CPU processes (distinct seeds) in parallel; returns (summed dose, list of
    per-process run records, per-process doses)."""
    td = workdir or tempfile.mkdtemp(prefix="mqi_ref_")
    ph = os.path.join(td, "phantom.raw")
    np.ascontiguousarray(hu, np.int16).tofile(ph)
    procs, dirs = [], []
    for p in range(n_proc):
        od = os.path.join(td, f"p{p}")
        os.makedirs(od, exist_ok=True)
        dirs.append(od)
        cmd = ref_phantom_cmd(debug, lxyz, pxyz, nxyz, energy, position, size, histories_each, ph, od, seed0 + p, beam,
                              beamline)
        log = open(os.path.join(od, "log.txt"), "w")
        procs.append(subprocess.Popen(cmd, stdout=log, stderr=subprocess.STDOUT))
        log.close()
    rcs = [q.wait() for q in procs]
    # The reference CPU build has crashed with SIGSEGV, rarely and not reproducibly with the same
    # seed when rerun alone; a process that dies by a signal is rerun once with the same seed.
    for i, r in enumerate(rcs):
        if r < 0:
            cmd = ref_phantom_cmd(debug, lxyz, pxyz, nxyz, energy, position, size, histories_each, ph, dirs[i],
                                  seed0 + i, beam, beamline)
            with open(os.path.join(dirs[i], "log_retry.txt"), "w") as log:
                rcs[i] = subprocess.run(cmd, stdout=log, stderr=subprocess.STDOUT).returncode
    if any(rcs):
        bad = [i for i, r in enumerate(rcs) if r]
        with open(os.path.join(dirs[bad[0]], "log.txt"), errors="replace") as f:
            tail = f.read()[-3000:]
        raise RuntimeError(f"reference oracle failed: {rcs}\n{tail}")
    n = int(np.prod(nxyz))
    doses, recs = [], []
    for od in dirs:
        doses.append(np.fromfile(os.path.join(od, f"{_beamline_children(beamline)}_water_dE_total.raw"),
                                 dtype=np.float64, count=n))
        with open(os.path.join(od, "run.json")) as f:
            recs.append(json.load(f))
    return np.sum(doses, axis=0), recs, doses


def ref_phantom_voxel_stats(debug: bool, lxyz, pxyz, nxyz, energy, position, size, histories_each, n_batches,
                            hu, seed0, beam="uniform", n_parallel: Optional[int] = None):
    """Per-voxel batch statistics of the reference CPU build: n_batches processes of
    histories_each histories with distinct seeds, run n_parallel at a time; returns the per-voxel
    sums of the batch doses and of their squares (float64 volumes, x fastest)."""
    n = int(np.prod(nxyz))
    s1 = np.zeros(n)
    s2 = np.zeros(n)
    n_parallel = n_parallel or max(os.cpu_count() or 1, 1)
    done = 0
    while done < n_batches:
        k = min(n_parallel, n_batches - done)
        with tempfile.TemporaryDirectory(prefix="mqi_refvox_") as td:
            _, _, doses = ref_phantom_parallel(debug, lxyz, pxyz, nxyz, energy, position, size, histories_each, k, hu,
                                               seed0 + done, beam, workdir=td)
            for d in doses:
                s1 += d
                s2 += d * d
        done += k
    return s1, s2


def ref_gpu_available(debug: bool = True) -> bool:
    """True when the reference GPU driver builds here (staged copy and nvcc present)."""
    return bool(_build().build_reference_gpu(debug))


def ref_gpu_phantom(debug: bool, lxyz, pxyz, nxyz, energy, position, size, histories, hu, seed, beam="uniform",
                    workdir: Optional[str] = None, phantom_path: Optional[str] = None):
    """One run of the reference's own CUDA kernel (oracle/ref_gpu_driver.cu, physics-debug build or
    not) on a phantom; returns (dose, run record with the CUDA-event kernel time)."""
    binary = _build().build_reference_gpu(debug)
    if not binary:
        raise RuntimeError("reference GPU driver unavailable (no staged reference copy or no nvcc)")
    td = workdir or tempfile.mkdtemp(prefix="mqi_refgpu_")
    if phantom_path is None:
        phantom_path = os.path.join(td, "phantom.raw")
        np.ascontiguousarray(hu, np.int16).tofile(phantom_path)
    cmd = [binary] + ref_phantom_cmd(debug, lxyz, pxyz, nxyz, energy, position, size, histories, phantom_path, td,
                                     seed, beam)[2:]
    with open(os.path.join(td, "log.txt"), "w") as log:
        rc = subprocess.run(cmd, stdout=log, stderr=subprocess.STDOUT).returncode
    if rc != 0:
        with open(os.path.join(td, "log.txt"), errors="replace") as f:
            raise RuntimeError(f"reference GPU run failed ({rc}):\n{f.read()[-3000:]}")
    n = int(np.prod(nxyz))
    dose = np.fromfile(os.path.join(td, "0_water_dE_total.raw"), dtype=np.float64, count=n)
    with open(os.path.join(td, "run.json")) as f:
        return dose, json.load(f)
