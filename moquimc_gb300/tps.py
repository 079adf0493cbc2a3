"""A treatment-planning environment over the C ABI: moqui's tps_env input keys, without DICOM.

moqui's tps_env (moqui/base/environments/mqi_tps_env.hpp) reads an input file of "Key value" lines
(mqi::file_parser, moqui/base/mqi_file_handler.hpp:220-420), reads the CT, plan and structures from
a DICOM directory, and per beam: builds the world (beamline children, then the CT child with
DensityScaling and X/Y/ZShift), the scorers named by `Scorer` (plus the Dose_stat / DoseSquare_stat
pair when StoppingStatistics is on), a beam source from the machine model, transports, and writes
`<beam>_<child>_<scorer>` volumes scaled by ParticlesPerHistory x RBE x NumberOfFraction
(save_reshaped_files, :1851-1900) or the Dij as npz.

The DICOM reader is out of scope here, so the CT (HU volume and voxel edges) and the beams (spots,
angles, isocentre, source distance, beamline devices) are given as arrays; everything else follows
the input file with moqui's keys and defaults.
"""
from __future__ import annotations

import os
import time
from dataclasses import dataclass, field
from typing import Dict, List, Sequence

import numpy as np

from . import beamline as bl
from . import capi
from .machine import PBSMachine, coordinate_rotation


_WS = " \f\n\r\t\v"   # what moqui's trim_copy trims (its delimiter literal ends at an embedded NUL)
_LIBC = None


def _libc():
    global _LIBC
    if _LIBC is None:
        import ctypes
        import ctypes.util

        _LIBC = ctypes.CDLL(ctypes.util.find_library("c"))
        _LIBC.atof.restype = ctypes.c_double
        _LIBC.atof.argtypes = [ctypes.c_char_p]
        _LIBC.atoi.restype = ctypes.c_int
        _LIBC.atoi.argtypes = [ctypes.c_char_p]
    return _LIBC


class InputFile:
    """mqi::file_parser (moqui/base/mqi_file_handler.hpp:220-420): lines are "Key value"; blank
    lines and lines starting with '#' are skipped and a '#' ends a line; the key is the text before
    the line's first space and matches case-insensitively; the first matching line wins.  Numbers
    are read with the C library's atof / atoi, floats rounded to FP32 (get_float returns a float),
    and a missing key's default is written as std::to_string writes it first ("%f" for floats, so
    a default below 5e-7 reads back as 0).  moqui's reader throws on a line of white space only, on
    a value of white space only and on an empty item of a list; here the line is skipped, the value
    reads as "" and the item is left out."""

    def __init__(self, text: str, delimiter: str = " "):
        self.lines: List[str] = []
        self.delimiter = delimiter
        for raw in text.split("\n"):
            if not raw:
                continue
            line = raw.strip(_WS)
            if not line or line[0] == "#":
                continue
            self.lines.append(line.split("#", 1)[0])

    @classmethod
    def load(cls, path: str) -> "InputFile":
        with open(path, newline="") as f:
            return cls(f.read())

    def get_string(self, key: str, default: str) -> str:
        for line in self.lines:
            pos = line.find(self.delimiter)
            if pos >= 0 and line[:pos].strip(_WS).lower() == key.lower():
                return line[pos + 1:].strip(_WS)
        return default

    def get_string_vector(self, key: str, sep: str) -> List[str]:
        v = self.get_string(key, "")
        return [t.strip(_WS) for t in v.split(sep) if t.strip(_WS)] if v else []

    @staticmethod
    def _atof(s: str) -> float:
        return float(_libc().atof(s.encode()))

    @staticmethod
    def _atoi(s: str) -> int:
        return int(_libc().atoi(s.encode()))

    def get_float(self, key: str, default: float) -> float:
        with np.errstate(over="ignore"):   # beyond the float range: inf, as the C++ conversion gives
            return float(np.float32(self._atof(self.get_string(key, "%f" % float(np.float32(default))))))

    def get_int(self, key: str, default: int) -> int:
        return self._atoi(self.get_string(key, str(int(default))))

    def get_bool(self, key: str, default: bool) -> bool:
        """"true" (any case) or a non-zero integer; the default is written as "1" / "0"."""
        t = self.get_string(key, "1" if default else "0")
        return t.lower() == "true" or self._atoi(t) != 0


SCORERS = ("EnergyDeposition", "Dose", "LETd", "LETt", "Dij", "TrackLength")


def read_mask_mha(path: str) -> np.ndarray:
    """mask_reader::read_mha_file (moqui/base/mqi_file_handler.hpp:38-90): header lines "Key = value"
    up to `ElementDataFile = LOCAL`, then DimSize x*y*z bytes of uint8 mask."""
    with open(path, "rb") as f:
        blob = f.read()
    dims, pos = None, 0
    while pos < len(blob):
        end = blob.find(b"\n", pos)
        end = len(blob) if end < 0 else end
        line = blob[pos:end].decode("latin-1").strip()
        pos = end + 1
        key, _, value = line.partition("=")
        key, value = key.strip().lower(), value.strip()
        if key == "dimsize":
            dims = [int(InputFile._atoi(v)) for v in value.split()[:3]]
        elif key == "elementdatafile":
            if value.lower() != "local":
                raise ValueError("Mask files does not contain data.")
            break
    if dims is None:
        raise ValueError(f"{path}: no DimSize")
    n = dims[0] * dims[1] * dims[2]
    return np.frombuffer(blob[pos:pos + n], np.uint8).copy()


def mask_to_contour(mask_total: np.ndarray):
    """mask_reader::mask_to_roi (mqi_file_handler.hpp:176-218): runs of voxels, in voxel order,
    that start at a voxel whose summed mask is exactly 1 and end at the next voxel whose summed
    mask is 0 -- a CONTOUR ROI as (start, stride, accumulated stride).  A run still open at the
    end of the volume is closed there (the reference leaves its stride unset)."""
    m = np.asarray(mask_total).reshape(-1)
    start, stride = [], []
    open_run = False
    for v, x in enumerate(m):
        if x == 1 and not open_run:
            open_run = True
            start.append(v)
        if x == 0 and open_run:
            open_run = False
            stride.append(v - start[-1])
    if open_run:
        stride.append(len(m) - start[-1])
    start = np.asarray(start, np.uint32)
    stride = np.asarray(stride, np.uint32)
    return start, stride, np.cumsum(stride, dtype=np.uint64).astype(np.uint32)


def contour_voxels(start: np.ndarray, stride: np.ndarray) -> np.ndarray:
    """The voxels of a CONTOUR ROI in mask order (the order of its compact tally)."""
    if len(start) == 0:
        return np.zeros(0, np.int64)
    return np.concatenate([np.arange(int(a), int(a) + int(b), dtype=np.int64) for a, b in zip(start, stride)])


@dataclass
class TpsConfig:
    """The input keys tps_env reads (mqi_tps_env.hpp:155-330), with its defaults."""
    gpu_id: int = 0
    random_seed: int = -1
    max_histories_per_batch: int = 0
    scorers: List[str] = field(default_factory=lambda: ["Dose"])
    simulation_type: str = "perBeam"
    particles_per_history: float = -1.0
    rbe: float = 1.1
    n_fractions: int = -1
    rangeshifter_density: float = 1.19
    unit_weights: int = -1
    machine: str = ""
    calibration: str = "default"
    density_scale: float = 1.0
    shift: tuple = (0.0, 0.0, 0.0)
    output_dir: str = ""
    output_format: str = "raw"
    overwrite_results: bool = False
    stopping_statistics: bool = False
    stopping_criteria: float = -1.0      # percent
    stat_threshold: float = 0.0
    beam_numbers: List[int] = field(default_factory=list)
    scoring_mask: bool = False
    mask_files: List[str] = field(default_factory=list)
    stat_roi_mask_files: List[str] = field(default_factory=list)

    @classmethod
    def from_input(cls, p: InputFile) -> "TpsConfig":
        seed = p.get_int("RandomSeed", -1)
        if seed == -1:
            seed = int(time.time())
        scorers = p.get_string_vector("Scorer", ",")
        canon = []
        for s in scorers:
            match = [n for n in SCORERS if n.lower() == s.lower()]
            if not match:
                raise ValueError(f"Unrecognized scorer name: {s}")
            canon.append(match[0])
        sim = p.get_string("SimulationType", "perBeam")
        if "Dij" in canon:
            if len(canon) > 1:
                raise ValueError("Dij cannot be scored with the other quantities")
            sim = "perSpot"
        out = p.get_string("OutputDir", "")
        if not out:
            raise ValueError("Output directory is not provided.")
        cfg = cls(
            gpu_id=p.get_int("GPUID", 0), random_seed=seed,
            max_histories_per_batch=p.get_int("MaxHistoriesPerBatch", 0), scorers=canon, simulation_type=sim,
            particles_per_history=p.get_float("ParticlesPerHistory", -1.0), rbe=p.get_float("RBE", 1.1),
            n_fractions=p.get_int("NumberOfFraction", -1),
            rangeshifter_density=p.get_float("RangeshifterDensity", 1.19), unit_weights=p.get_int("UnitWeights", -1),
            machine=p.get_string("Machine", ""), calibration=p.get_string("Calibration", "default"),
            density_scale=p.get_float("DensityScaling", 1.0),
            shift=(p.get_float("XShift", 0.0), p.get_float("YShift", 0.0), p.get_float("ZShift", 0.0)),
            output_dir=out, output_format=p.get_string("OutputFormat", "raw"),
            overwrite_results=p.get_bool("OverwriteResults", False),
            stopping_statistics=p.get_bool("StoppingStatistics", False),
            stat_threshold=p.get_float("StatThreshold", 0.0),
            beam_numbers=[int(InputFile._atoi(v)) for v in p.get_string_vector("BeamNumbers", ",")],
            scoring_mask=p.get_bool("ScoringMask", False),
            stat_roi_mask_files=p.get_string_vector("StatROIMaskFilename", ","),
        )
        if cfg.scoring_mask:
            cfg.mask_files = p.get_string_vector("Mask", ",")
            if not cfg.mask_files:
                raise ValueError("Mask filename is missing")
        if cfg.stopping_statistics:
            cfg.stopping_criteria = p.get_float("StoppingCriteria", -1.0)
            if cfg.stopping_criteria < 0:
                raise ValueError("Statistical criteria must be positive float")
            if cfg.stat_threshold <= 0 and not cfg.stat_roi_mask_files:
                raise ValueError("If no contour or mask is selected, the statistical threshold cannot be zero")
        if cfg.calibration.lower() != "default":
            raise ValueError("Unknown calibration method")
        return cfg


@dataclass
class Beam:
    """One beam of a plan: spots as rows (nominal energy MeV, x mm, y mm, meterset) at the
    isocentre plane, the IEC angles (degrees), the isocentre (mm, CT frame), the source-to-
    isocentre distance at which histories start, and optional beamline devices (device tuples of
    beamline.children_from_devices; a range shifter's density is RangeshifterDensity).  A device
    whose angles are None is a box in the beam frame, rotated and translated with the beam (its
    translation added to the isocentre), as tps_env places its range shifters and apertures."""
    name: str
    spots: np.ndarray
    gantry: float = 0.0
    couch: float = 0.0
    collimator: float = 0.0
    isocenter: Sequence[float] = (0.0, 0.0, 0.0)
    source_to_isocenter_mm: float = 390.0
    devices: list = field(default_factory=list)


def write_volume(out_dir: str, name: str, data: np.ndarray, scale: float, fmt: str, edges) -> str:
    """save_to_bin / save_to_mhd / save_to_mha (moqui/base/mqi_io.hpp:166-183, 493-583): the FP64
    volume times scale, with the reference's header lines for .mhd (which writes `TransformMatrix`,
    `Offset` and `CenterOfRotation` without '=') and .mha (data after the header)."""
    d = (np.asarray(data, np.float64) * float(scale)).astype("<f8")
    xe, ye, ze = (np.asarray(e, np.float32) for e in edges)
    dx, dy, dz = (np.float32(e[1] - e[0]) for e in (xe, ye, ze))
    x0, y0, z0 = (np.float32(float(e[0]) + float(s) * 0.5) for e, s in ((xe, dx), (ye, dy), (ze, dz)))
    nx, ny, nz = len(xe) - 1, len(ye) - 1, len(ze) - 1
    fmt = fmt.lower()

    def g6(v):
        return f"{float(v):.6g}"

    def g9(v):
        return f"{float(v):.9g}"

    if fmt == "mhd":
        path = os.path.join(out_dir, name + ".mhd")
        with open(path, "w") as f:
            f.write("ObjectType = Image\nNDims = 3\nBinaryData = True\nBinaryDataByteOrderMSB = False\n"
                    "CompressedData = False\nTransformMatrix 1 0 0 0 1 0 0 0 1\n"
                    f"Offset {g6(x0)} {g6(y0)} {g6(z0)}\nCenterOfRotation 0 0 0\nAnatomicOrientation = RAI\n"
                    f"DimSize = {nx} {ny} {nz}\nElementType = MET_DOUBLE\n"
                    f"ElementSpacing = {g6(dx)} {g6(dy)} {g6(dz)}\nElementDataFile = {name}.raw\n")
        d.tofile(os.path.join(out_dir, name + ".raw"))
        return path
    if fmt == "mha":
        path = os.path.join(out_dir, name + ".mha")
        with open(path, "wb") as f:
            f.write(("ObjectType = Image\nNDims = 3\nBinaryData = True\nBinaryDataByteOrderMSB = False\n"
                     "CompressedData = False\nTransformMatrix = 1 0 0 0 1 0 0 0 1\n"
                     f"Origin = {g9(x0)} {g9(y0)} {g9(z0)}\nCenterOfRotation = 0 0 0\nAnatomicOrientation = RAI\n"
                     f"DimSize = {nx} {ny} {nz}\nElementType = MET_DOUBLE\nHeaderSize = -1\n"
                     f"ElementSpacing = {g9(dx)} {g9(dy)} {g9(dz)}\nElementDataFile = LOCAL\n").encode())
            f.write(d.tobytes())
        return path
    path = os.path.join(out_dir, name + ".raw")
    d.tofile(path)
    return path


class TpsEnv:
    """tps_env's per-beam run over the C ABI.  ct_hu: int16 [nz][ny][nx]; ct_edges: (xe, ye, ze) in
    mm; beams: list of Beam; machine: PBSMachine (the `Machine PBS` model); fractions: the plan's
    number of fractions, used when NumberOfFraction <= 0 (tps_env reads it from the plan then)."""

    def __init__(self, config: TpsConfig, ct_hu: np.ndarray, ct_edges, beams: List[Beam], machine: PBSMachine,
                 fractions: int = 1):
        self.cfg = config
        self.n_fractions = config.n_fractions if config.n_fractions > 0 else int(fractions)
        self.hu = np.ascontiguousarray(ct_hu, np.int16)
        self.edges = tuple(np.asarray(e, np.float32) for e in ct_edges)
        self.beams = beams
        self.machine = machine
        od = config.output_dir
        if os.path.exists(od) and not config.overwrite_results and os.listdir(od):
            raise FileExistsError("Output directory exists.")
        os.makedirs(od, exist_ok=True)

    def _plan(self, beam: Beam) -> np.ndarray:
        cfg = self.cfg
        angles = (beam.collimator, beam.gantry, beam.couch, 90.0)   # iec2dicom, mqi_tps_env.hpp:978
        if cfg.unit_weights > 0:
            plan = self.machine.plan(beam.spots, -1.0, beam.source_to_isocenter_mm, angles, beam.isocenter)
            plan["histories"] = cfg.unit_weights
        elif cfg.particles_per_history == -1:
            plan = self.machine.plan(beam.spots, -1.0, beam.source_to_isocenter_mm, angles, beam.isocenter)
        else:
            plan = self.machine.plan(beam.spots, -1.0, beam.source_to_isocenter_mm, angles, beam.isocenter,
                                     histories_from_ratio=cfg.particles_per_history)
        return plan

    def run_beam(self, k: int, beam: Beam) -> Dict[str, str]:
        cfg = self.cfg
        c = capi.Context(cfg.gpu_id)
        try:
            c.set_physics(False)
            # beamline children first (mqi_tps_env.hpp:735-758): a device given without angles
            # carries the beam's rotation, as tps_env gives its devices p_final.rotation
            rot = coordinate_rotation((beam.collimator, beam.gantry, beam.couch, 90.0))
            for d in beam.devices:
                if d[0] == "rangeshifter":
                    d = (d[0], d[1], d[2], cfg.rangeshifter_density, *d[4:])
                beam_frame = d[4] is None
                if beam_frame:
                    d = (*d[:4], (0.0, 0.0, 0.0), d[5])
                child = bl.children_from_devices([d])[0]
                if beam_frame:   # box in the beam frame, placed by the beam's transform
                    child.rot = rot
                    child.translation = (np.asarray(beam.isocenter, np.float32) +
                                         np.asarray(d[5], np.float32)).astype(np.float32)
                child.add_to(c)
            shifted = tuple(e + np.float32(s) for e, s in zip(self.edges, cfg.shift))   # X/Y/ZShift
            cid = c.add_child(*shifted)
            c.set_hu(cid, self.hu, cfg.density_scale)
            names: List[tuple] = []
            dij = None
            roi = {}
            if cfg.scoring_mask:   # the scorers' ROI: the summed masks (mqi_tps_env.hpp:775-785)
                total = sum(read_mask_mha(f).astype(np.uint16) for f in cfg.mask_files)
                st, sr, ac = mask_to_contour(total)
                roi = {"roi_method": capi.ROI_CONTOUR, "start": st, "stride": sr, "acc": ac}
            for s in cfg.scorers:
                if s == "Dose":
                    names.append((s, c.add_scorer(cid, capi.DOSE_W, **roi)))
                # EnergyDeposition and TrackLength are accepted names without a scorer in tps_env
                # (its scorer set-up, :789-933, creates none for them), so they write nothing here
                elif s == "LETd":
                    names.append(("LETd_numer", c.add_scorer(cid, capi.LETD_NUM, **roi)))
                    names.append(("LETd_denom", c.add_scorer(cid, capi.LETD_DEN, **roi)))
                elif s == "LETt":
                    names.append(("LETt_numer", c.add_scorer(cid, capi.LETT_NUM, **roi)))
                    names.append(("LETt_denom", c.add_scorer(cid, capi.LETT_DEN, **roi)))
                elif s == "Dij":
                    dij = c.add_dij_scorer(cid, capacity=1 << 28)
            stat = None
            if cfg.stopping_statistics:
                if cfg.stat_roi_mask_files:   # StatROIMaskFilename, else the whole CT
                    total = sum(read_mask_mha(f).astype(np.uint16) for f in cfg.stat_roi_mask_files)
                    st, sr, ac = mask_to_contour(total)
                    stat = c.add_stat_scorers(cid, capi.ROI_CONTOUR, st, sr, ac)
                else:
                    stat = c.add_stat_scorers(cid)
            plan = self._plan(beam)
            n = c.set_spot_plan(plan)
            seed = (cfg.random_seed + 10000 * k) & 0xFFFFFFFF
            out: Dict[str, str] = {}
            if stat is not None:
                passes, achieved = c.run_plan_until_stat(stat[0], stat[1], cfg.stopping_criteria / 100.0,
                                                         cfg.stat_threshold, 1000, seed)
                out["passes"], out["uncertainty"] = str(passes), str(achieved)
            else:
                cum = c.plan_cum
                step = cfg.max_histories_per_batch if cfg.max_histories_per_batch > 0 else n
                ranges = ([(int(cum[s]), int(cum[s + 1])) for s in range(len(plan))]
                          if cfg.simulation_type.lower() == "perspot" and dij is None else
                          [(h, min(h + step, n)) for h in range(0, n, max(step, 1))])
                for h0, h1 in ranges:
                    if h1 > h0:
                        c.transport_plan(h0, h1, seed)
            pph = 1.0 if cfg.unit_weights > 0 else cfg.particles_per_history
            # in FP32, as tps_env forms it (float particles_per_history * float rbe * int n_fractions)
            scale = float(np.float32(np.float32(pph) * np.float32(cfg.rbe)) * np.float32(self.n_fractions))
            child_index = len(beam.devices)
            for name, sid in names:
                fname = f"{beam.name}_{child_index}_{name}"
                vol = c.tally(sid)
                if roi and vol.size != self.hu.size:   # a mask-indexed tally: the CT volume is written
                    full = np.zeros(self.hu.size, np.float64)
                    full[contour_voxels(roi["start"], roi["stride"])] = vol
                    vol = full
                out[name] = write_volume(cfg.output_dir, fname, vol, scale, cfg.output_format, shifted)
            if dij is not None:
                op = c.dij_build(dij, scale=scale)
                path = os.path.join(cfg.output_dir, f"{beam.name}_{child_index}_Dij.npz")
                op.save_npz(path)
                out["Dij"] = path
            return out
        finally:
            c.close()

    def run(self) -> Dict[str, Dict[str, str]]:
        """The 1-based BeamNumbers, or every beam but those named "Setup" when BeamNumbers is
        empty or 0 (mqi_tps_env.hpp:332-360), as tps_env::initialize_and_run."""
        chosen = self.cfg.beam_numbers
        if not chosen or chosen == [0]:
            chosen = [k + 1 for k, b in enumerate(self.beams) if b.name != "Setup"]
        return {self.beams[b - 1].name: self.run_beam(i, self.beams[b - 1]) for i, b in enumerate(chosen)}
