#!/usr/bin/env python3
"""Generate ``mqi_tables.h``: the tabulated physics data the transport needs, as exact hex floats.

The engine's physics is driven by seven float tables that must hold exactly the same values as
moqui's for the dose to agree:

* ``cs_p_ion``   delta-ray (restricted ionisation) cross-section per unit mass density, 600 nodes
  from 0.1 MeV in 0.5 MeV steps (moqui/base/mqi_p_ionization.hpp:11)
* ``dedx``       restricted stopping power, same energy grid (mqi_p_ionization.hpp:74)
* ``range``      CSDA range in water, same energy grid (mqi_p_ionization.hpp:145)
* ``cs_pp_e``    p-p elastic cross-section, 600 nodes from 0.5 MeV in 0.5 MeV steps
  (mqi_pp_elastic.hpp:11)
* ``cs_po_e``    p-O elastic, same grid (mqi_po_elastic.hpp:12)
* ``cs_po_i``    p-O inelastic, same grid (mqi_po_inelastic.hpp:11)
* ``density_correction``  3996-entry HU->density correction factor for HU -1000..2995
  (moqui/base/materials/mqi_patient_materials.hpp:11)

The numbers are physics data (Geant4 TestEm0 tabulations and a Schneider-style calibration).  They
are parsed from the reference headers, rounded to float exactly as a C compiler rounds the decimal
literals, and written as C99 hex-float literals so that every consumer reads bit-identical values.

Usage: ``python gen_tables.py --src <reference root> [--out mqi_tables.h]``.  The generated file
is committed; rerunning on an unchanged reference reproduces it byte for byte.
"""
import argparse
import os
import re
import struct
import sys

TABLES = [
    ("cs_p_ion", "moqui/base/mqi_p_ionization.hpp", "cs_p_ion_table", 600),
    ("dedx", "moqui/base/mqi_p_ionization.hpp", "restricted_stopping_power_table", 600),
    ("range", "moqui/base/mqi_p_ionization.hpp", "range_steps", 600),
    ("cs_pp_e", "moqui/base/mqi_pp_elastic.hpp", "cs_pp_e_g4_table", 600),
    ("cs_po_e", "moqui/base/mqi_po_elastic.hpp", "cs_po_e_g4_table", 600),
    ("cs_po_i", "moqui/base/mqi_po_inelastic.hpp", "cs_po_i_g4_table", 600),
    ("density_correction", "moqui/base/materials/mqi_patient_materials.hpp", "density_correction", 3996),
]

_NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?")


def parse_table(path: str, cname: str, n: int):
    with open(path) as f:
        text = f.read()
    m = re.search(r"\b" + re.escape(cname) + r"\s*\[\s*\d+\s*\]\s*=\s*\{(.*?)\}", text, re.S)
    if not m:
        raise RuntimeError(f"table {cname} not found in {path}")
    body = re.sub(r"//[^\n]*", "", m.group(1))
    vals = [float(t) for t in _NUM.findall(body)]
    if len(vals) != n:
        raise RuntimeError(f"{cname}: expected {n} values, parsed {len(vals)}")
    # Round to binary32 the way a C compiler rounds a decimal float literal (round to nearest).
    return [struct.unpack("<f", struct.pack("<f", v))[0] for v in vals]


def hexf(v: float) -> str:
    if v == 0.0:
        return "0x0p+0f"
    return float.hex(v).replace("0x1.0000000000000p", "0x1p") + "f"


def render(tables) -> str:
    out = [
        "// Generated by gen_tables.py from the reference physics data; do not edit by hand.",
        "// Values are binary32 hex-float literals, bit-identical to the reference's float tables.",
        "#pragma once",
        "",
        "#define MQI_TABLE_N 600",
        "#define MQI_DENSITY_CORRECTION_N 3996",
        "",
        "// constexpr in C++, so a static device array can be initialised from the tables at compile time",
        "#ifdef __cplusplus",
        "#define MQI_TABLE_STORAGE static constexpr float",
        "#else",
        "#define MQI_TABLE_STORAGE static const float",
        "#endif",
        "",
    ]
    for name, vals in tables:
        out.append(f"MQI_TABLE_STORAGE mqi_tab_{name}[{len(vals)}] = {{")
        for i in range(0, len(vals), 6):
            out.append("    " + ", ".join(hexf(v) for v in vals[i:i + 6]) + ",")
        out.append("};")
        out.append("")
    return "\n".join(out)


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", required=True, help="root of the reference checkout (the directory holding moqui/)")
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "mqi_tables.h"))
    args = ap.parse_args()
    tables = [(name, parse_table(os.path.join(args.src, rel), cname, n)) for name, rel, cname, n in TABLES]
    with open(args.out, "w") as f:
        f.write(render(tables))
    print(args.out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
