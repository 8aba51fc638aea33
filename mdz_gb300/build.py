"""Builds libmdzgpu.so (sm_103a) in-tree with nvcc.

Every translation unit under mdz_gb300/csrc is compiled in parallel into
mdz_gb300/_build/, the multi-limb kernels once per word count listed in
csrc/internal.h (MDZ_MP_WORDS_LIST, MDZ_MPW_LIST), and linked into
mdz_gb300/lib/.
Objects are rebuilt when their source or any csrc header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libmdzgpu.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def mp_word_counts() -> list[int]:
    text = (CSRC / "internal.h").read_text()
    m = re.search(r"#define MDZ_MP_WORDS_LIST\(X\)(.*)", text)
    if not m:
        raise RuntimeError("MDZ_MP_WORDS_LIST not found")
    return [int(x) for x in re.findall(r"X\((\d+)\)", m.group(1))]


def mpw_configs() -> list[tuple[int, int, int]]:
    text = (CSRC / "internal.h").read_text()
    m = re.search(r"#define MDZ_MPW_LIST\(X\)((?:.*\\\n)*.*)", text)
    if not m:
        raise RuntimeError("MDZ_MPW_LIST not found")
    return [tuple(int(v) for v in t) for t in
            re.findall(r"X\((\d+),\s*(\d+),\s*(\d+)\)", m.group(1))]


def _jobs() -> list[tuple[Path, Path, list[str]]]:
    jobs = []
    for src in sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp")):
        if src.name == "mp_kernel.cu":
            for n in mp_word_counts():
                jobs.append((src, BUILD / f"mp_kernel_w{n}.o", [f"-DMDZ_MP_WORDS={n}"]))
        elif src.name == "mpw_kernel.cu":
            for n, g, q in mpw_configs():
                jobs.append((src, BUILD / f"mpw_kernel_w{n}.o",
                             [f"-DMDZ_MPW_G={g}", f"-DMDZ_MPW_Q={q}"]))
        else:
            jobs.append((src, BUILD / (src.stem + ".o"), []))
    return jobs


def _newest_header() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(job, verbose: bool) -> str:
    src, obj, extra = job
    extra = extra + os.environ.get("MDZGPU_NVCC_FLAGS", "").split()
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-x", "cu", *extra, "-I", str(INCLUDE), "-c", str(src),
               "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj.name


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile and link libmdzgpu.so; returns its path."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    hdr = _newest_header()
    todo = []
    objs = []
    for job in _jobs():
        src, obj, _ = job
        objs.append(obj)
        if not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr):
            todo.append(job)
    if todo:
        workers = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            for name in ex.map(lambda j: _compile(j, verbose), todo):
                if verbose:
                    print("built", name, flush=True)
    newest_obj = max(o.stat().st_mtime for o in objs)
    if todo or not LIB.exists() or LIB.stat().st_mtime < newest_obj:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
