#!/usr/bin/env python3
"""Stage a patched, build-ready copy of the reference engine's headers under ``oracle/_ref/src``.

This is test infrastructure: the staged copy is compiled into the reference CPU oracle
(``oracle/_ref/bin/*``) that the parity tests and the timed CPU baseline use.  Nothing in the
product library includes or links it.

The reference (moqui) is header-only C++; its CPU path builds with g++ from the headers alone.
Two problems keep it from running unmodified, and both are handled here or in the drivers:

1. ``mc::print_materials<R>`` reads material members that no longer exist
   (``moqui/kernel_functions/mqi_print_data.hpp:20-24``).  The oracle drivers declare an empty
   explicit specialisation for ``float``; no reference file is touched for this.
2. ``p_ionization_tabulated::energy_loss`` walks the range table downwards with an unsigned 16-bit
   index (``moqui/base/mqi_p_ionization.hpp:318-320``).  When the residual range falls below the
   first table entry with the index already at 0, the ``--n`` wraps to 65535 and the loop reads far
   outside the 600-entry table (a segfault on the CPU at >= 1e4 histories).  The staged copy replaces
   the loop by the guarded form "step n down while n > 0 and r < r_steps[n]", which produces the same
   index in every case where the original does not wrap.

A third file is staged beside the copy, for the input-file tests: ``mqi_file_handler.hpp`` holds
moqui's input-file reader (``mqi::file_parser``) but includes the beam-module headers, which need
the DICOM library (GDCM), absent here.  The reader itself needs none of them.
``moqui/base/mqi_file_handler_parser.hpp`` is the same file with that one include replaced by the
three DICOM-free headers the file does use (``mqi_common.hpp``, ``mqi_vec.hpp``,
``mqi_scorer.hpp``) and ``<cassert>`` added; ``oracle/ref_parser.cpp`` is compiled against it.

Usage: ``python oracle/stage_ref.py --src <reference root>`` (the directory holding ``moqui/``; the
checkout is only read).  The copy is only (re)written when the source is present, so on a machine
without the reference the previously staged copy is used as is.
"""
import argparse
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEST = os.path.join(HERE, "_ref", "src")

# The underflowing loop, matched loosely on whitespace (reference mqi_p_ionization.hpp:318-320).
_LOOP = re.compile(
    r"do\s*\{\s*if\s*\(\s*r\s*>=\s*r_steps\[n\]\s*\)\s*break;\s*\}\s*while\s*\(\s*--n\s*>\s*0\s*\);"
)
_GUARDED = "while (n > 0 && r < r_steps[n]) { --n; } /* oracle: guarded against uint16 wrap */"


_BEAM_MODULE_INCLUDE = "#include <moqui/base/mqi_beam_module_ion.hpp>"
_PARSER_INCLUDES = ("#include <cassert>\n#include <moqui/base/mqi_common.hpp>\n#include <moqui/base/mqi_vec.hpp>\n"
                    "#include <moqui/base/mqi_scorer.hpp>")


def stage_parser(src_root: str) -> str:
    """Write moqui/base/mqi_file_handler_parser.hpp (see the module docstring) into the staged
    copy; returns its path."""
    with open(os.path.join(src_root, "moqui", "base", "mqi_file_handler.hpp")) as f:
        text = f.read()
    if text.count(_BEAM_MODULE_INCLUDE) != 1:
        raise RuntimeError("expected exactly one beam-module include in mqi_file_handler.hpp")
    out = os.path.join(DEST, "moqui", "base", "mqi_file_handler_parser.hpp")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    with open(out, "w") as f:
        f.write(text.replace(_BEAM_MODULE_INCLUDE, _PARSER_INCLUDES))
    return out


def stage(src_root: str) -> str:
    src = os.path.join(src_root, "moqui")
    if not os.path.isdir(src):
        if os.path.isdir(os.path.join(DEST, "moqui")):
            return DEST
        raise FileNotFoundError(f"reference sources not found under {src_root}")
    dst = os.path.join(DEST, "moqui")
    if os.path.isdir(dst):
        shutil.rmtree(dst)
    shutil.copytree(src, dst, ignore=shutil.ignore_patterns("*.py", "*.cc", "*.hh", "*.txt", "*.md"))
    target = os.path.join(dst, "base", "mqi_p_ionization.hpp")
    with open(target) as f:
        text = f.read()
    text, n = _LOOP.subn(_GUARDED, text)
    if n != 1:
        raise RuntimeError(f"expected exactly one range-table loop to patch, found {n}")
    with open(target, "w") as f:
        f.write(text)
    stage_parser(src_root)
    return DEST


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", required=True)
    args = ap.parse_args()
    print(stage(args.src))
    return 0


if __name__ == "__main__":
    sys.exit(main())
