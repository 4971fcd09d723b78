#!/usr/bin/env python3
"""Stages a copy of WFA2-lib v2.3's C sources into baseline/_ref/WFA2-lib (git-ignored).

Test and baseline infrastructure, not part of the product. The copy is what `make -C oracle
ref` compiles into oracle/_ref/libwfa2_ref.so — on this machine and on any machine the
working tree is copied to, where the reference project itself is not present — so that the
real WFA2-lib can pin the oracle and serve as the timed CPU baseline there.

    WFA2_SRC=<path to the reference's WFA2-lib folder> python oracle/stage_wfa2.py
    python oracle/stage_wfa2.py <path to WFA2-lib>

Only the library's sources and headers (wavefront/, alignment/, system/, utils/ and
VERSION.txt) are copied, unmodified. The copy is never committed.
"""
from __future__ import annotations

import os
import shutil
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
DEST = ROOT / "baseline" / "_ref" / "WFA2-lib"
FOLDERS = ("wavefront", "alignment", "system", "utils")


def stage(src: Path, dest: Path = DEST) -> Path:
    if not (src / "wavefront" / "wavefront_align.c").exists():
        raise FileNotFoundError(f"{src} does not hold WFA2-lib's sources")
    if dest.exists():
        shutil.rmtree(dest)
    for sub in FOLDERS:
        for f in sorted((src / sub).iterdir()):
            if f.suffix in (".c", ".h"):
                (dest / sub).mkdir(parents=True, exist_ok=True)
                shutil.copy2(f, dest / sub / f.name)
    if (src / "VERSION.txt").exists():
        shutil.copy2(src / "VERSION.txt", dest / "VERSION.txt")
    return dest


def main() -> int:
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("WFA2_SRC", "")
    if not src:
        print("usage: stage_wfa2.py <WFA2-lib folder>  (or set WFA2_SRC)", file=sys.stderr)
        return 2
    print(f"staged {stage(Path(src))}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
