"""Builds the CPU oracle (TEST INFRASTRUCTURE) into oracle/_build/.

libmdzoracle.so is oracle/mdz_oracle.c compiled with -O3 -ffp-contract=off
(no FMA contraction, as the reference's double build) and, when the system
libmpfr.so.6 exists, linked against it by full path with MDZO_WITH_MPFR.
When the reference sources are present (this container), oracle/build_ref.sh
also compiles the unmodified reference into oracle/_ref/.
"""
from __future__ import annotations

import glob
import os
import platform
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "libmdzoracle.so"


def ref_root() -> Path | None:
    """The MDZ source tree the reference build and the fixture scripts read
    (MDZ_REF_ROOT, else the default oracle/build_ref.sh names), or None when
    it is not on this machine."""
    r = subprocess.run(["sh", str(HERE / "build_ref.sh"), "--root"], capture_output=True,
                       text=True)
    root = Path(r.stdout.strip()) if r.returncode == 0 and r.stdout.strip() else None
    return root if root is not None and (root / "src" / "fractal.c").exists() else None


def find_system_lib(name: str) -> str | None:
    pats = [f"/usr/lib/*-linux-gnu/{name}", f"/usr/lib64/{name}", f"/usr/lib/{name}",
            f"/lib/*-linux-gnu/{name}"]
    for p in pats:
        hits = sorted(glob.glob(p))
        if hits:
            return hits[0]
    return None


def build(reference: bool = True) -> Path:
    OUT.mkdir(exist_ok=True)
    src = HERE / "mdz_oracle.c"
    mpfr = find_system_lib("libmpfr.so.6")
    gmp = find_system_lib("libgmp.so.10")
    stamp = OUT / "variant.txt"
    variant = f"mpfr={mpfr} gmp={gmp}"
    fresh = (LIB.exists() and LIB.stat().st_mtime >= src.stat().st_mtime
             and stamp.exists() and stamp.read_text() == variant)
    if not fresh:
        cmd = ["gcc", "-std=gnu99", "-O3", "-ffp-contract=off", "-fPIC", "-shared",
               "-I", str(HERE / "shim"), str(src), "-o", str(LIB)]
        if mpfr and gmp:
            cmd[1:1] = ["-DMDZO_WITH_MPFR"]
            cmd += [mpfr, gmp]
        cmd += ["-lm", "-lpthread"]
        subprocess.run(cmd, check=True)
        stamp.write_text(variant)
    if reference and ref_root() is not None and platform.machine() == "x86_64":
        subprocess.run(["sh", str(HERE / "build_ref.sh")], check=True,
                       stdout=subprocess.DEVNULL)
    return LIB


if __name__ == "__main__":
    print(build())
