#!/usr/bin/env python3
"""Switch a PLUTO problem build to the GB300 AdvanceStep (or back).

PLUTO's setup tool writes the problem's ``makefile`` from
``Src/Templates/makefile``, which has an "Additional_object_files_here"
block for extra objects.  This script adds after that block

    PG_ROOT = <this repository>
    include $(PG_ROOT)/pluto_gb300/shim/Makefile.gpu

(which swaps rk_step.o / update_stage.o / ctu_step.o for gpu_step.o, links
libpluto_gb300 and compiles write_data.o / init.o with WriteData / Analysis
renamed, since gpu_step.o wraps both), or removes it again with --disable.
Either way the problem directory's write_data.o and init.o are deleted so
that make rebuilds them with the matching names.  Running it twice is
harmless; re-run it after the setup tool regenerates the makefile.

    python pluto_gb300/shim/enable.py <problem dir or makefile> [--disable]
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
MARK = "Additional_object_files_here"
BEGIN = "# >>> pluto_gb300 GPU AdvanceStep (pluto_gb300/shim/enable.py)"
END = "# <<< pluto_gb300"


def block(root: Path = ROOT) -> str:
    return f"{BEGIN}\nPG_ROOT = {root}\ninclude $(PG_ROOT)/pluto_gb300/shim/Makefile.gpu\n{END}\n"


def strip(text: str) -> str:
    """The makefile without a block this script added."""
    out, skip = [], False
    for line in text.splitlines(keepends=True):
        if line.startswith(BEGIN):
            skip = True
            continue
        if skip:
            if line.startswith(END):
                skip = False
            continue
        out.append(line)
    return "".join(out)


def enable(text: str, root: Path = ROOT) -> str:
    """Insert the block after the line that follows the marker (the dashed
    rule that closes the template's comment box)."""
    text = strip(text)
    lines = text.splitlines(keepends=True)
    for n, line in enumerate(lines):
        if MARK in line:
            at = n + 2 if n + 1 < len(lines) and lines[n + 1].lstrip().startswith("#") else n + 1
            return "".join(lines[:at]) + block(root) + "".join(lines[at:])
    raise ValueError(f"no '{MARK}' line: not a makefile written by PLUTO's setup tool")


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("target", help="problem directory or its makefile")
    ap.add_argument("--disable", action="store_true", help="remove the GPU block")
    args = ap.parse_args(argv)
    mk = Path(args.target)
    if mk.is_dir():
        mk = mk / "makefile"
    text = mk.read_text()
    new = strip(text) if args.disable else enable(text)
    if new != text:
        mk.write_text(new)
    for stale in ("write_data.o", "init.o"):  # built with the other WriteData / Analysis names
        (mk.parent / stale).unlink(missing_ok=True)
    print(f"{mk}: GPU AdvanceStep {'disabled' if args.disable else 'enabled'}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
