"""Pencil-beam-scanning machine model: beam-data file -> the device spot plan (capi.SPOT_DTYPE).

moqui's generic PBS machine (moqui/base/mqi_treatment_machine_pbs.hpp) reads a beam model file
(load_beamdata, :400-520) and turns every spot of a plan into a beamlet: the energy and the spot's
phase-space widths interpolated at the nominal energy (characterize_beamlet, :199-236), the beam
started at source_to_isocenter_mm on the ray from the virtual source (beam_starting_position,
moqui/base/mqi_treatment_machine_ion.hpp:324-333), and a history count (characterize_history, :134-143, or create_beamsource's
ceil(meterset x particles per history), mqi_treatment_machine_ion.hpp:147-189).  The beamlet is
norm_1d energy x Gaussian phsp_6d (mqi_phsp6d.hpp) x the beam's coordinate_transform
(mqi_coordinate_transform.hpp): exactly what a capi.SPOT_DTYPE entry holds, so the plan is sampled
on the device (mqi_set_spot_plan) instead of on the host.

Arithmetic follows the reference's float instantiation (every step rounded to FP32).  The
reference's own class does not build here (its headers include the DICOM library), so this module
is checked against the formulas in tests/test_machine_cpu.py rather than against a reference run.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from typing import Dict, Iterable, Optional, Sequence, Tuple

import numpy as np

from . import beamline

f32 = np.float32
_SECTION = re.compile(r"(.*)\[(.*)\](.*)")


@dataclass
class SpotSpec:
    """One row of the [spot] section: nominal energy -> E, dE, x, y, x', y' (sigmas) and the
    particles-per-meterset ratio."""
    E: float
    dE: float
    x: float
    y: float
    xp: float
    yp: float
    ratio: float


@dataclass
class PBSMachine:
    beamdata: Dict[float, SpotSpec]
    sad: Tuple[float, float] = (math.inf, math.inf)
    rangeshifter: Tuple[float, float] = (0.0, 0.0)
    rangeshifter_snout_gap: float = 0.0
    aperture: Tuple[float, float] = (0.0, 0.0)
    rangeshifter_thickness: Dict[str, float] = field(default_factory=dict)
    time: Dict[str, float] = field(default_factory=dict)

    # ---------------------------------------------------------------- reading the beam model
    @classmethod
    def parse(cls, text: str) -> "PBSMachine":
        """load_beamdata: '#' starts a comment; sections [geometry] (SAD(mm), rangeshifter(mm),
        rangeshifter_snout_gap(mm), aperture(mm)), [rangeshifter_thickness] ("name" mm),
        [spot] (nominal E dE x y xp yp ratio) and [time] (key value).  A SAD of 0 means a
        parallel beam (infinite SAD), as in the pbs constructor (:104-117)."""
        geo: Dict[str, Tuple[float, float]] = {}
        rs: Dict[str, float] = {}
        spots: Dict[float, SpotSpec] = {}
        tim: Dict[str, float] = {}
        section = None
        for raw in text.splitlines():
            line = raw.split("#", 1)[0].strip()
            if not line:
                continue
            if _SECTION.fullmatch(line):
                section = line
                continue
            if section == "[geometry]":
                parts = line.split()
                vals = [float(v) for v in parts[1:3]] + [0.0, 0.0]
                geo[parts[0]] = (vals[0], vals[1])
            elif section == "[rangeshifter_thickness]":
                a, b = line.find('"'), line.rfind('"')
                rs[line[a + 1:b]] = float(line[b + 1:])
            elif section == "[spot]":
                v = [float(t) for t in line.split()]
                spots[float(f32(v[0]))] = SpotSpec(*(float(f32(x)) for x in v[1:8]))
            elif section == "[time]":
                k, val = line.split()[:2]
                tim[k] = float(val)
        sad = geo.get("SAD(mm)", (0.0, 0.0))
        return cls(
            beamdata=dict(sorted(spots.items())),
            sad=tuple(math.inf if s == 0 else float(f32(s)) for s in sad),
            rangeshifter=geo.get("rangeshifter(mm)", (0.0, 0.0)),
            rangeshifter_snout_gap=geo.get("rangeshifter_snout_gap(mm)", (0.0, 0.0))[0],
            aperture=geo.get("aperture(mm)", (0.0, 0.0)),
            rangeshifter_thickness=rs,
            time=tim,
        )

    @classmethod
    def load(cls, path: str) -> "PBSMachine":
        with open(path) as f:
            return cls.parse(f.read())

    # ---------------------------------------------------------------- characterisation
    def _bracket(self, e: float) -> Tuple[float, SpotSpec, float, SpotSpec]:
        """beamdata_.lower_bound(e) and the entry before it.  The reference prints "out-of-bound"
        and reads before the first entry when e is at or below the first nominal energy, and past
        the end above the last; both are errors here."""
        keys = list(self.beamdata)
        e = float(f32(e))
        i = int(np.searchsorted(keys, e, side="left"))
        if i == 0 or i == len(keys):
            raise ValueError(f"energy {e} MeV outside the beam model ({keys[0]}, {keys[-1]}]")
        return keys[i - 1], self.beamdata[keys[i - 1]], keys[i], self.beamdata[keys[i]]

    @staticmethod
    def _intpl(x, x0, x1, y0, y1):
        """The pbs intpl lambda in FP32: y0 + (x - x0) * (y1 - y0) / (x1 - x0), y0 when x1 == x0."""
        x, x0, x1, y0, y1 = (f32(v) for v in (x, x0, x1, y0, y1))
        return y0 if x1 == x0 else f32(y0 + (x - x0) * (y1 - y0) / (x1 - x0))

    def spot_parameters(self, e: float) -> dict:
        """Interpolated E, dE, x, y, x', y' and ratio at nominal energy e (characterize_beamlet,
        :206-214; the widths are interpolated against the bracketing rows' E, as there)."""
        k0, d, k1, u = self._bracket(e)
        mid_e = self._intpl(e, k0, k1, d.E, u.E)
        out = {"E": mid_e, "ratio": self._intpl(e, k0, k1, d.ratio, u.ratio)}
        for name in ("dE", "x", "y", "xp", "yp"):
            out[name] = self._intpl(e, d.E, u.E, getattr(d, name), getattr(u, name))
        return out

    def beam_start(self, x: float, y: float, source_to_isocenter_mm: float) -> Tuple[np.ndarray, np.ndarray]:
        """beam_starting_position (mqi_treatment_machine_ion.hpp:324-333) and the unit direction to the
        isocentre point (x, y, 0).
        An infinite SAD is a parallel beam (the reference's inf/inf would give NaN)."""
        z = f32(source_to_isocenter_mm)
        iso = np.array([x, y, 0.0], np.float32)
        beam = np.array([iso[0], iso[1], z], np.float32)
        for a in range(2):
            s = self.sad[a]
            if math.isfinite(s):
                beam[a] = f32(iso[a] * (f32(s) - z) / f32(s))
        d = iso - beam
        n = f32(math.sqrt(float(f32(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]))))
        return beam, (d / n).astype(np.float32)

    def histories(self, e: float, meterset: float, scale: float) -> int:
        """characterize_history (:134-143): meterset x ratio / scale, truncated."""
        r = self.spot_parameters(e)["ratio"]
        return int(f32(f32(meterset) * f32(r) / f32(scale)))

    def plan(self, spots: Iterable[Sequence[float]], particles_per_history: float = -1.0,
             source_to_isocenter_mm: float = 390.0, angles=(0.0, 0.0, 0.0, 0.0), isocenter=(0.0, 0.0, 0.0),
             histories_from_ratio: Optional[float] = None) -> np.ndarray:
        """A device spot plan (capi.SPOT_DTYPE) from (e, x, y, meterset) spots.  Histories per spot:
        create_beamsource's ceil(meterset x particles_per_history), or 1 when it is <= 1
        (mqi_treatment_machine_ion.hpp:163-165); with histories_from_ratio = scale, the machine's
        characterize_history instead.  angles = (collimator, gantry, couch, iec2dicom) in degrees
        and the isocentre give the beam's coordinate_transform."""
        from .capi import SPOT_DTYPE

        spots = [tuple(s) for s in spots]
        out = np.zeros(len(spots), SPOT_DTYPE)
        rot = coordinate_rotation(angles)
        for i, (e, x, y, w) in enumerate(spots):
            p = self.spot_parameters(e)
            beam, d = self.beam_start(x, y, source_to_isocenter_mm)
            out[i]["energy"] = p["E"]
            out[i]["energy_sigma"] = p["dE"]
            out[i]["mean"] = [beam[0], beam[1], beam[2], d[0], d[1]]
            out[i]["sigma"] = [p["x"], p["y"], 0.0, p["xp"], p["yp"]]
            out[i]["corr"] = [0.0, 0.0]
            out[i]["rot"] = rot
            out[i]["trans"] = np.asarray(isocenter, np.float32)
            if histories_from_ratio is not None:
                out[i]["histories"] = self.histories(e, w, histories_from_ratio)
            else:
                out[i]["histories"] = 1 if particles_per_history <= 1 else int(math.ceil(float(f32(w)) * particles_per_history))
        return out


def coordinate_rotation(angles) -> np.ndarray:
    """coordinate_transform's rotation (mqi_coordinate_transform.hpp): iec2dicom x couch x gantry x
    collimator, each a mat3x3 about one axis, from (collimator, gantry, couch, iec2dicom) degrees;
    FP32 like the reference's float instantiation.  Row-major 3x3."""
    deg2rad = f32(math.pi / 180.0)
    a = [f32(v) * deg2rad for v in angles]
    col = beamline.rotation_xyz(0.0, 0.0, float(a[0])).reshape(3, 3)
    gan = beamline.rotation_xyz(0.0, float(a[1]), 0.0).reshape(3, 3)
    cou = beamline.rotation_xyz(0.0, 0.0, float(a[2])).reshape(3, 3)
    iec = beamline.rotation_xyz(float(a[3]), 0.0, 0.0).reshape(3, 3)
    return _mul(_mul(_mul(iec, cou), gan), col).reshape(-1)


def _mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """mat3x3::operator* in FP32, each entry summed left to right."""
    r = np.empty((3, 3), np.float32)
    for i in range(3):
        for j in range(3):
            r[i, j] = f32(f32(f32(a[i, 0] * b[0, j]) + f32(a[i, 1] * b[1, j])) + f32(a[i, 2] * b[2, j]))
    return r
