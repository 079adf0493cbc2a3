"""ctypes binding of libmqigpu.so (include/mqi_gpu.h).

This is the thin Python layer over the C ABI; it adds no compute of its own.  The library must have
been built (``moquimc_gb300.build.build_library``); loading fails loudly otherwise -- there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import build as _build

MQI_OK = 0
(MQI_ERR_INVALID, MQI_ERR_CUDA, MQI_ERR_NOMEM, MQI_ERR_STATE, MQI_ERR_UNSUPPORTED, MQI_ERR_OVERFLOW,
 MQI_ERR_DEVICE) = range(-1, -8, -1)
ERRORS = {
    -1: "MQI_ERR_INVALID", -2: "MQI_ERR_CUDA", -3: "MQI_ERR_NOMEM", -4: "MQI_ERR_STATE",
    -5: "MQI_ERR_UNSUPPORTED", -6: "MQI_ERR_OVERFLOW", -7: "MQI_ERR_DEVICE",
}

# scorer types (mqi_scorer_type)
EDEP, DOSE_W, DOSE_W2, DOSE_M = 1, 2, 3, 4
LETD_NUM, LETD_DEN, LETT_NUM, LETT_DEN = 5, 6, 7, 8
EDEP_PRIMARY, EDEP_SECONDARY, DIJ = 9, 10, 11
# roi methods
ROI_DIRECT, ROI_INDIRECT, ROI_CONTOUR = 0, 1, 2
# calibration curves
CALIB_DEFAULT, CALIB_TABLE = 0, 1

# every exported symbol declared in include/mqi_gpu.h
EXPORTS = (
    "mqi_create", "mqi_destroy", "mqi_last_error", "mqi_set_stream", "mqi_set_physics",
    "mqi_add_child", "mqi_set_density", "mqi_set_hu", "mqi_add_scorer", "mqi_set_vertices",
    "mqi_transport", "mqi_get_tally", "mqi_reset_tallies", "mqi_get_stats", "mqi_hu_to_density",
    "mqi_trace_rays", "mqi_eval_physics", "mqi_set_tuning", "mqi_transport_noalloc", "mqi_version",
    "mqi_add_stat_scorers", "mqi_stat_uncertainty", "mqi_batch_accumulate", "mqi_batch_uncertainty",
    "mqi_get_batch_mean", "mqi_scale_tally", "mqi_run_until_stat", "mqi_set_spot_plan", "mqi_transport_plan",
    "mqi_sample_plan", "mqi_add_dij_scorer", "mqi_dij_build", "mqi_dij_get_csr", "mqi_dij_info",
    "mqi_dij_matvec", "mqi_dij_rmatvec", "mqi_set_scenarios", "mqi_run_plan_until_stat", "mqi_set_launch_mode",
    "mqi_autotune", "mqi_set_calibration", "mqi_philox4x32_10", "mqi_dij_record_hits", "mqi_dij_get_hits",
    "mqi_eval_hits", "mqi_eval_roi", "mqi_set_post_step_mode", "mqi_set_queue_sort",
)

VERTEX_DTYPE = np.dtype([("ke", "<f4"), ("pos", "<f4", (3,)), ("dir", "<f4", (3,))])
# mqi_tune_result (include/mqi_gpu.h)
TUNE_DTYPE = np.dtype([("block", "<i4"), ("blocks_per_sm", "<i4"), ("streamed", "<i4"), ("graph_waves", "<i4"),
                       ("primary_chunk", "<u4"), ("pad", "<u4"), ("histories_per_s", "<f8")])
# mqi_spot (include/mqi_gpu.h): 26 floats, then the 64-bit history count at byte 104
SPOT_DTYPE = np.dtype({"names": ["energy", "energy_sigma", "mean", "sigma", "corr", "rot", "trans", "histories"],
                       "formats": ["<f4", "<f4", ("<f4", (5,)), ("<f4", (5,)), ("<f4", (2,)), ("<f4", (9,)),
                                   ("<f4", (3,)), "<u8"],
                       "offsets": [0, 4, 8, 28, 48, 56, 92, 104], "itemsize": 112})


class CalibTable:
    """SPR(rho, E) and X0(rho) on uniform grids: spr has shape (n_rho, n_e), x0 shape (n_rho,);
    rho in g/mm^3, E in MeV, X0 in mm (mqi_set_calibration)."""

    def __init__(self, rho0: float, drho: float, e0: float, de: float, spr, x0):
        self.spr = np.ascontiguousarray(spr, np.float32)
        self.x0 = np.ascontiguousarray(x0, np.float32)
        if self.spr.ndim != 2 or self.x0.shape != (self.spr.shape[0],):
            raise ValueError("spr must be (n_rho, n_e) and x0 (n_rho,)")
        self.n_rho, self.n_e = self.spr.shape
        self.rho0, self.drho, self.e0, self.de = float(rho0), float(drho), float(e0), float(de)

    @classmethod
    def sample(cls, spr_fn, x0_fn, rho0, drho, n_rho, e0, de, n_e):
        """Tabulate curves given as functions (spr_fn(rho, E), x0_fn(rho)) on the grids."""
        rho = (rho0 + drho * np.arange(n_rho)).astype(np.float32)
        e = (e0 + de * np.arange(n_e)).astype(np.float32)
        spr = np.array([[spr_fn(float(r), float(x)) for x in e] for r in rho], np.float32)
        x0 = np.array([x0_fn(float(r)) for r in rho], np.float32)
        return cls(rho0, drho, e0, de, spr, x0)


class MqiStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "histories", "tracks", "steps", "secondaries", "local_daughters", "dropped", "waves",
        "device_errors", "kernel_launches", "wave_launches")] + [("wave_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {n: (float if n == "wave_ms" else int)(getattr(self, n)) for n, _ in self._fields_}


class MqiError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib: Optional[C.CDLL] = None


def library_path() -> str:
    return _build.LIB


def load(path: Optional[str] = None) -> C.CDLL:
    """Load libmqigpu.so and declare the signatures.  Raises if the library was not built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or library_path()
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    vp, i32, u32, u64, f32 = C.c_void_p, C.c_int, C.c_uint32, C.c_uint64, C.c_float
    P = C.POINTER
    sig = {
        "mqi_create": (i32, [i32, P(vp)]),
        "mqi_destroy": (i32, [vp]),
        "mqi_last_error": (C.c_char_p, [vp]),
        "mqi_set_stream": (i32, [vp, vp]),
        "mqi_set_physics": (i32, [vp, i32, i32]),
        "mqi_set_calibration": (i32, [vp, i32, u32, f32, f32, u32, f32, f32, vp, vp]),
        "mqi_add_child": (i32, [vp, i32, i32, i32, vp, vp, vp, vp, vp, P(i32)]),
        "mqi_set_density": (i32, [vp, i32, vp, i32]),
        "mqi_set_hu": (i32, [vp, i32, vp, f32, i32]),
        "mqi_add_scorer": (i32, [vp, i32, i32, i32, u32, vp, vp, vp, P(i32)]),
        "mqi_set_vertices": (i32, [vp, vp, vp, u64, i32]),
        "mqi_transport": (i32, [vp, u64, u64, u64]),
        "mqi_get_tally": (i32, [vp, i32, vp, P(u64), i32]),
        "mqi_reset_tallies": (i32, [vp]),
        "mqi_get_stats": (i32, [vp, P(MqiStats)]),
        "mqi_hu_to_density": (i32, [vp, vp, vp, u64, f32, i32]),
        "mqi_trace_rays": (i32, [vp, i32, vp, u64, u32, vp, vp, vp, vp, u64, P(u64)]),
        "mqi_eval_physics": (i32, [vp, vp, u64, vp]),
        "mqi_set_tuning": (i32, [vp, i32, i32, i32, i32]),
        "mqi_transport_noalloc": (i32, [i32, i32, i32, vp, vp, vp, vp, vp, u64, i32, i32, u64, vp, vp]),
        "mqi_version": (C.c_char_p, []),
        "mqi_philox4x32_10": (i32, [vp, vp, vp]),
        "mqi_dij_record_hits": (i32, [vp, i32, u64]),
        "mqi_eval_hits": (i32, [vp, i32, i32, vp, vp, vp, u64, vp]),
        "mqi_set_post_step_mode": (i32, [vp, i32]),
        "mqi_set_queue_sort": (i32, [vp, u32]),
        "mqi_eval_roi": (i32, [vp, i32, vp, u64, vp, vp]),
        "mqi_dij_get_hits": (i32, [vp, i32, vp, vp, vp, P(u64)]),
        "mqi_add_stat_scorers": (i32, [vp, i32, i32, u32, vp, vp, vp, P(i32), P(i32)]),
        "mqi_stat_uncertainty": (i32, [vp, i32, i32, u64, f32, P(C.c_double), P(u64)]),
        "mqi_batch_accumulate": (i32, [vp, i32]),
        "mqi_batch_uncertainty": (i32, [vp, i32, f32, P(C.c_double), P(u64), P(u64)]),
        "mqi_get_batch_mean": (i32, [vp, i32, vp, P(u64), i32]),
        "mqi_scale_tally": (i32, [vp, i32, C.c_double]),
        "mqi_run_until_stat": (i32, [vp, i32, i32, u64, f32, f32, u64, u64, P(u64), P(C.c_double)]),
        "mqi_set_spot_plan": (i32, [vp, vp, u32, P(u64)]),
        "mqi_transport_plan": (i32, [vp, u64, u64, u64]),
        "mqi_sample_plan": (i32, [vp, u64, u64, u64, vp, vp]),
        "mqi_add_dij_scorer": (i32, [vp, i32, i32, u32, vp, vp, vp, u64, P(i32)]),
        "mqi_dij_build": (i32, [vp, i32, u32, C.c_double, P(u64)]),
        "mqi_dij_get_csr": (i32, [vp, i32, vp, vp, vp, i32]),
        "mqi_dij_info": (i32, [vp, i32, P(u64), P(u64), P(u64), P(u64)]),
        "mqi_dij_matvec": (i32, [vp, i32, vp, vp, i32, i32]),
        "mqi_dij_rmatvec": (i32, [vp, i32, vp, vp, i32, i32]),
        "mqi_set_scenarios": (i32, [vp, i32, u32, vp, vp, vp, vp]),
        "mqi_set_launch_mode": (i32, [vp, i32, i32]),
        "mqi_autotune": (i32, [vp, i32, u64, u64, u64, vp, u32, P(u32)]),
        "mqi_run_plan_until_stat": (i32, [vp, i32, i32, f32, f32, u64, u64, P(u64), P(C.c_double)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def philox4x32_10(counter, key) -> np.ndarray:
    """One block of the engine's generator computed by the library on the host (no GPU needed):
    four uint32 words of Philox4x32-10 for counter (4 words) under key (2 words)."""
    lib = load()
    c = np.ascontiguousarray(counter, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    rc = lib.mqi_philox4x32_10(c.ctypes.data, k.ctypes.data, out.ctypes.data)
    if rc != MQI_OK:
        raise MqiError(rc, lib.mqi_last_error(None).decode())
    return out


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Context:
    """One engine context on one CUDA device (mqi_create ... mqi_destroy)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        self._check(self.lib.mqi_create(device, C.byref(h)), None)
        self.h = h
        self.children: list[tuple[int, int, int]] = []
        self.scorers: list[int] = []
        self._dij_child: dict[int, int] = {}
        self.plan_cum = np.zeros(1, np.uint64)

    def _check(self, rc: int, h) -> None:
        if rc != MQI_OK:
            msg = self.lib.mqi_last_error(h)
            raise MqiError(rc, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.mqi_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- setup ----
    def set_physics(self, physics_debug: bool, score_local_deposit: bool = True) -> None:
        self._check(self.lib.mqi_set_physics(self.h, int(physics_debug), int(score_local_deposit)), self.h)

    def set_calibration(self, table=None) -> None:
        """Tabulated SPR(rho, E) / X0(rho) curves (a CalibTable), or None for moqui's default
        curves (spr_default / radiation_length_default)."""
        if table is None:
            self._check(self.lib.mqi_set_calibration(self.h, CALIB_DEFAULT, 0, 0.0, 0.0, 0, 0.0, 0.0, None, None), self.h)
            return
        spr = np.ascontiguousarray(table.spr, np.float32)
        x0 = np.ascontiguousarray(table.x0, np.float32)
        self._check(self.lib.mqi_set_calibration(self.h, CALIB_TABLE, table.n_rho, table.rho0, table.drho, table.n_e,
                                                 table.e0, table.de, spr.ctypes.data, x0.ctypes.data), self.h)

    def set_tuning(self, block: int = 0, blocks_per_sm: int = 0, slice_steps: int = -1, primary_chunk: int = 0) -> None:
        self._check(self.lib.mqi_set_tuning(self.h, block, blocks_per_sm, slice_steps, primary_chunk), self.h)

    def autotune(self, h0: int, h1: int, seed: int = 1, plan: bool = False) -> np.ndarray:
        """Time every candidate launch configuration on histories [h0, h1) and keep the fastest;
        returns the measurements (TUNE_DTYPE)."""
        res = np.zeros(64, TUNE_DTYPE)
        n = C.c_uint32(0)
        self._check(self.lib.mqi_autotune(self.h, int(plan), h0, h1, seed, _ptr(res), len(res), C.byref(n)), self.h)
        return res[: n.value]

    def set_post_step_mode(self, mode: int) -> None:
        """Nuclear post-steps: 0 inside the wave, 1 in the post-step kernel, -1 by run size."""
        self._check(self.lib.mqi_set_post_step_mode(self.h, mode), self.h)

    def set_queue_sort(self, min_entries: int) -> None:
        """Sort the queue by energy bin before waves of at least min_entries entries (0: never)."""
        self._check(self.lib.mqi_set_queue_sort(self.h, min_entries), self.h)

    def set_launch_mode(self, streamed: int = -1, graph_waves: int = 0) -> None:
        self._check(self.lib.mqi_set_launch_mode(self.h, streamed, graph_waves), self.h)

    def set_stream(self, stream_ptr: Optional[int]) -> None:
        """Run the context's work on a cudaStream_t handle (1 = the legacy default stream;
        None = a stream of the context's own)."""
        self._check(self.lib.mqi_set_stream(self.h, stream_ptr), self.h)
        self._stream_handle = stream_ptr

    def add_child(self, xe, ye, ze, rot_fwd=None, translation=None) -> int:
        xe = np.ascontiguousarray(xe, dtype=np.float32)
        ye = np.ascontiguousarray(ye, dtype=np.float32)
        ze = np.ascontiguousarray(ze, dtype=np.float32)
        rf = None if rot_fwd is None else np.ascontiguousarray(rot_fwd, dtype=np.float32).reshape(9)
        tr = None if translation is None else np.ascontiguousarray(translation, dtype=np.float32).reshape(3)
        cid = C.c_int(-1)
        self._check(self.lib.mqi_add_child(self.h, len(xe) - 1, len(ye) - 1, len(ze) - 1, _ptr(xe), _ptr(ye),
                                           _ptr(ze), _ptr(rf), _ptr(tr), C.byref(cid)), self.h)
        self.children.append((len(xe) - 1, len(ye) - 1, len(ze) - 1))
        return cid.value

    def set_density(self, child: int, rho: np.ndarray) -> None:
        rho = np.ascontiguousarray(rho, dtype=np.float32)
        self._check(self.lib.mqi_set_density(self.h, child, _ptr(rho), 0), self.h)

    def set_density_device(self, child: int, dev_ptr: int) -> None:
        self._check(self.lib.mqi_set_density(self.h, child, C.c_void_p(dev_ptr), 1), self.h)

    def set_hu(self, child: int, hu: np.ndarray, density_scale: float = 1.0) -> None:
        hu = np.ascontiguousarray(hu, dtype=np.int16)
        self._check(self.lib.mqi_set_hu(self.h, child, _ptr(hu), C.c_float(density_scale), 0), self.h)

    def add_scorer(self, child: int, stype: int, roi_method: int = ROI_DIRECT, start=None, stride=None,
                   acc=None) -> int:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.uint32) for a in (start, stride, acc)]
        length = 0 if arrs[1] is None else len(arrs[1])
        sid = C.c_int(-1)
        self._check(self.lib.mqi_add_scorer(self.h, child, stype, roi_method, length, _ptr(arrs[0]), _ptr(arrs[1]),
                                            _ptr(arrs[2]), C.byref(sid)), self.h)
        self.scorers.append(sid.value)
        return sid.value

    def set_vertices(self, vertices: np.ndarray, spot_ids: Optional[np.ndarray] = None) -> None:
        v = np.ascontiguousarray(vertices)
        if v.dtype != VERTEX_DTYPE:
            v = np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(-1, 7)).view(VERTEX_DTYPE).reshape(-1)
        s = None if spot_ids is None else np.ascontiguousarray(spot_ids, dtype=np.uint32)
        self._check(self.lib.mqi_set_vertices(self.h, _ptr(v), _ptr(s), len(v), 0), self.h)
        self.n_vertices = len(v)

    def set_vertices_device(self, dev_ptr: int, n: int, spot_dev_ptr: Optional[int] = None) -> None:
        self._check(self.lib.mqi_set_vertices(self.h, C.c_void_p(dev_ptr),
                                              None if spot_dev_ptr is None else C.c_void_p(spot_dev_ptr), n, 1),
                    self.h)
        self.n_vertices = n

    # ---- run ----
    def transport(self, h0: int, h1: int, seed: int) -> None:
        self._check(self.lib.mqi_transport(self.h, h0, h1, seed & 0xFFFFFFFFFFFFFFFF), self.h)

    def tally(self, scorer: int) -> np.ndarray:
        n = C.c_uint64(0)
        self._check(self.lib.mqi_get_tally(self.h, scorer, None, C.byref(n), 0), self.h)
        out = np.empty(n.value, dtype=np.float64)
        self._check(self.lib.mqi_get_tally(self.h, scorer, _ptr(out), C.byref(n), 0), self.h)
        return out

    def tally_to_device(self, scorer: int, dev_ptr: int) -> None:
        n = C.c_uint64(0)
        self._check(self.lib.mqi_get_tally(self.h, scorer, C.c_void_p(dev_ptr), C.byref(n), 1), self.h)

    def reset(self) -> None:
        self._check(self.lib.mqi_reset_tallies(self.h), self.h)

    def stats(self) -> dict:
        s = MqiStats()
        self._check(self.lib.mqi_get_stats(self.h, C.byref(s)), self.h)
        return s.as_dict()

    # ---- probes ----
    def hu_to_density(self, hu: np.ndarray, scale: float = 1.0) -> np.ndarray:
        hu = np.ascontiguousarray(hu, dtype=np.int16)
        out = np.empty(hu.shape, dtype=np.float32)
        self._check(self.lib.mqi_hu_to_density(self.h, _ptr(hu), _ptr(out), hu.size, C.c_float(scale), 0), self.h)
        return out

    def trace_rays(self, child: int, rays: np.ndarray, max_steps: int):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        n = len(rays)
        cap = n * max_steps
        off = np.zeros(n + 1, dtype=np.int64)
        cnb = np.zeros(cap, dtype=np.uint64)
        dist = np.zeros(cap, dtype=np.float32)
        cells = np.zeros((cap, 3), dtype=np.int32)
        tot = C.c_uint64(0)
        self._check(self.lib.mqi_trace_rays(self.h, child, _ptr(rays), n, max_steps, _ptr(off), _ptr(cnb), _ptr(dist),
                                            _ptr(cells), cap, C.byref(tot)), self.h)
        t = tot.value
        return off, cnb[:t], dist[:t], cells[:t]

    def eval_physics(self, energies: np.ndarray) -> np.ndarray:
        e = np.ascontiguousarray(energies, dtype=np.float32)
        out = np.empty((len(e), 8), dtype=np.float32)
        self._check(self.lib.mqi_eval_physics(self.h, _ptr(e), len(e), _ptr(out)), self.h)
        return out

    # ---- raw-pointer variants (pinned host or device buffers owned by the caller) ----
    def eval_hits(self, child: int, stype: int, steps: np.ndarray, cnb: np.ndarray, primary: np.ndarray) -> np.ndarray:
        """The device's scorer callback on step states (9 floats each), voxels and primary flags."""
        st = np.ascontiguousarray(steps, np.float32).reshape(-1, 9)
        cb = np.ascontiguousarray(cnb, np.uint32)
        pr = np.ascontiguousarray(primary, np.int32)
        out = np.empty(len(cb), np.float64)
        self._check(self.lib.mqi_eval_hits(self.h, child, stype, _ptr(st), _ptr(cb), _ptr(pr), len(cb), _ptr(out)),
                    self.h)
        return out

    def eval_roi(self, scorer: int, voxels: np.ndarray):
        """The device's roi_t::idx and get_mask_idx of a scorer's ROI for the given voxels."""
        v = np.ascontiguousarray(voxels, np.uint32)
        idx = np.empty(len(v), np.int32)
        mask = np.empty(len(v), np.int32)
        self._check(self.lib.mqi_eval_roi(self.h, scorer, _ptr(v), len(v), _ptr(idx), _ptr(mask)), self.h)
        return idx, mask

    def set_vertices_ptr(self, ptr: int, n: int, on_device: bool) -> None:
        self._check(self.lib.mqi_set_vertices(self.h, C.c_void_p(ptr), None, n, int(on_device)), self.h)
        self.n_vertices = n

    def tally_to_ptr(self, scorer: int, ptr: int, on_device: bool) -> None:
        n = C.c_uint64(0)
        self._check(self.lib.mqi_get_tally(self.h, scorer, C.c_void_p(ptr), C.byref(n), int(on_device)), self.h)

    # ---- statistics ----
    def add_stat_scorers(self, child: int, roi_method: int = ROI_DIRECT, start=None, stride=None, acc=None,
                         mask_size: int = 0) -> tuple[int, int]:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.uint32) for a in (start, stride, acc)]
        length = mask_size if roi_method == ROI_INDIRECT else (0 if arrs[1] is None else len(arrs[1]))
        a, b = C.c_int(-1), C.c_int(-1)
        self._check(self.lib.mqi_add_stat_scorers(self.h, child, roi_method, length, _ptr(arrs[0]), _ptr(arrs[1]),
                                                  _ptr(arrs[2]), C.byref(a), C.byref(b)), self.h)
        self.scorers += [a.value, b.value]
        return a.value, b.value

    def stat_uncertainty(self, dose_id: int, dose2_id: int, n_histories: int, threshold: float) -> tuple[float, int]:
        v, n = C.c_double(0), C.c_uint64(0)
        self._check(self.lib.mqi_stat_uncertainty(self.h, dose_id, dose2_id, n_histories, C.c_float(threshold),
                                                  C.byref(v), C.byref(n)), self.h)
        return v.value, n.value

    def batch_accumulate(self, scorer: int) -> None:
        self._check(self.lib.mqi_batch_accumulate(self.h, scorer), self.h)

    def batch_uncertainty(self, scorer: int, threshold: float) -> tuple[float, int, int]:
        v, n, b = C.c_double(0), C.c_uint64(0), C.c_uint64(0)
        self._check(self.lib.mqi_batch_uncertainty(self.h, scorer, C.c_float(threshold), C.byref(v), C.byref(n),
                                                   C.byref(b)), self.h)
        return v.value, n.value, b.value

    def batch_mean(self, scorer: int) -> np.ndarray:
        n = C.c_uint64(0)
        self._check(self.lib.mqi_get_batch_mean(self.h, scorer, None, C.byref(n), 0), self.h)
        out = np.empty(n.value, np.float64)
        self._check(self.lib.mqi_get_batch_mean(self.h, scorer, _ptr(out), C.byref(n), 0), self.h)
        return out

    def scale_tally(self, scorer: int, weight: float) -> None:
        self._check(self.lib.mqi_scale_tally(self.h, scorer, C.c_double(weight)), self.h)

    def run_until_stat(self, dose_id: int, dose2_id: int, histories_per_run: int, criteria: float, threshold: float,
                       max_runs: int, seed: int) -> tuple[int, float]:
        done, got = C.c_uint64(0), C.c_double(0)
        self._check(self.lib.mqi_run_until_stat(self.h, dose_id, dose2_id, histories_per_run, C.c_float(criteria),
                                                C.c_float(threshold), max_runs, seed, C.byref(done), C.byref(got)),
                    self.h)
        return done.value, got.value

    # ---- spot plans ----
    def set_spot_plan(self, spots: np.ndarray) -> int:
        sp = np.ascontiguousarray(spots, dtype=SPOT_DTYPE)
        tot = C.c_uint64(0)
        self._check(self.lib.mqi_set_spot_plan(self.h, _ptr(sp), len(sp), C.byref(tot)), self.h)
        self.plan_histories = tot.value
        self.plan_cum = np.concatenate([[0], np.cumsum(sp["histories"].astype(np.uint64))])
        return tot.value

    def transport_plan(self, h0: int, h1: int, seed: int) -> None:
        self._check(self.lib.mqi_transport_plan(self.h, h0, h1, seed & 0xFFFFFFFFFFFFFFFF), self.h)

    def sample_plan(self, h0: int, h1: int, seed: int):
        """Vertices and spot ids mqi_transport_plan starts for histories [h0, h1)."""
        v = np.empty(h1 - h0, dtype=VERTEX_DTYPE)
        sid = np.empty(h1 - h0, dtype=np.uint32)
        self._check(self.lib.mqi_sample_plan(self.h, h0, h1, seed & 0xFFFFFFFFFFFFFFFF, _ptr(v), _ptr(sid)), self.h)
        return v, sid

    # ---- Dij ----
    def add_dij_scorer(self, child: int, capacity: int = 0, roi_method: int = ROI_DIRECT) -> int:
        out = C.c_int(-1)
        self._check(self.lib.mqi_add_dij_scorer(self.h, child, roi_method, 0, None, None, None, capacity,
                                                C.byref(out)), self.h)
        self.scorers.append(out.value)
        self._dij_child[out.value] = child
        return out.value

    def dij_record_hits(self, scorer: int, capacity: int) -> None:
        """Record every insertion into the Dij table from now on (capacity 0: stop)."""
        self._check(self.lib.mqi_dij_record_hits(self.h, scorer, capacity), self.h)

    def dij_hits(self, scorer: int):
        """The recorded insertions: (voxel uint32, spot uint32, value float64) in issue order."""
        n = C.c_uint64(0)
        self._check(self.lib.mqi_dij_get_hits(self.h, scorer, None, None, None, C.byref(n)), self.h)
        vox = np.empty(n.value, np.uint32)
        spot = np.empty(n.value, np.uint32)
        val = np.empty(n.value, np.float64)
        self._check(self.lib.mqi_dij_get_hits(self.h, scorer, _ptr(vox), _ptr(spot), _ptr(val), C.byref(n)), self.h)
        return vox, spot, val

    def dij_build(self, scorer: int, n_spots: int = 0, scale: float = 1.0):
        """Build the Dij matrix; returns a dij.DijOperator."""
        from .dij import DijOperator

        nnz = C.c_uint64(0)
        self._check(self.lib.mqi_dij_build(self.h, scorer, n_spots, scale, C.byref(nnz)), self.h)
        n_vox = int(np.prod(self.children[self._dij_child[scorer]]))
        ns = n_spots or len(self.plan_cum) - 1
        return DijOperator(self, scorer, ns, n_vox, nnz.value)

    def dij_info(self, scorer: int) -> dict:
        v = [C.c_uint64(0) for _ in range(4)]
        self._check(self.lib.mqi_dij_info(self.h, scorer, *[C.byref(x) for x in v]), self.h)
        return dict(zip(("table_slots", "occupied", "nnz", "voxel_rows"), (x.value for x in v)))

    def dij_matvec(self, scorer: int, w: np.ndarray, n_voxels: int) -> np.ndarray:
        fp64 = w.dtype == np.float64
        w = np.ascontiguousarray(w, np.float64 if fp64 else np.float32)
        out = np.empty(n_voxels, w.dtype)
        self._check(self.lib.mqi_dij_matvec(self.h, scorer, _ptr(w), _ptr(out), int(fp64), 0), self.h)
        return out

    def dij_rmatvec(self, scorer: int, g: np.ndarray, n_spots: int) -> np.ndarray:
        fp64 = g.dtype == np.float64
        g = np.ascontiguousarray(g, np.float64 if fp64 else np.float32)
        out = np.empty(n_spots, g.dtype)
        self._check(self.lib.mqi_dij_rmatvec(self.h, scorer, _ptr(g), _ptr(out), int(fp64), 0), self.h)
        return out

    # ---- robust scenarios ----
    def set_scenarios(self, child: int, xe_list, ye_list, ze_list, density_scale=None) -> None:
        """One (xe, ye, ze) edge set per scenario and optional density scales; [] removes them."""
        n = len(xe_list)
        if n <= 1:
            self._check(self.lib.mqi_set_scenarios(self.h, child, 0, None, None, None, None), self.h)
            self.n_scen = 1
            return
        xe = np.ascontiguousarray(np.stack(xe_list), np.float32)
        ye = np.ascontiguousarray(np.stack(ye_list), np.float32)
        ze = np.ascontiguousarray(np.stack(ze_list), np.float32)
        sc = None if density_scale is None else np.ascontiguousarray(density_scale, np.float32)
        self._check(self.lib.mqi_set_scenarios(self.h, child, n, _ptr(xe), _ptr(ye), _ptr(ze), _ptr(sc)), self.h)
        self.n_scen = n

    def run_plan_until_stat(self, dose_id: int, dose2_id: int, criteria: float, threshold: float,
                            max_passes: int, seed: int) -> tuple[int, float]:
        p, a = C.c_uint64(0), C.c_double(0)
        self._check(self.lib.mqi_run_plan_until_stat(self.h, dose_id, dose2_id, C.c_float(criteria),
                                                     C.c_float(threshold), max_passes, seed & 0xFFFFFFFFFFFFFFFF,
                                                     C.byref(p), C.byref(a)), self.h)
        return p.value, a.value
