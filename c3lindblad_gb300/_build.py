"""Compile the CUDA sources into the in-tree shared library.

``nvcc -gencode arch=compute_103a,code=sm_103a`` per translation unit, in
parallel, then one ``-shared`` link.  Rebuilds only when a source or the
public header is newer than the library.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIB_DIR = PKG / "_lib"
LIB_NAME = "libc3l_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build c3lindblad_gb300")


def library_path() -> Path:
    return LIB_DIR / LIB_NAME


def _stale(out: Path, inputs) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def build(force: bool = False, verbose: bool = False) -> Path:
    LIB_DIR.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    header = INCLUDE / "c3l_gb300.h"
    out = library_path()
    if not force and not _stale(out, sources + sorted(CSRC.glob("*.h")) + [header, Path(__file__)]):
        return out
    compiler = nvcc()
    flags = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]
    objs = []
    procs = []
    for src in sources:
        obj = LIB_DIR / (src.stem + ".o")
        objs.append(obj)
        cmd = [compiler, *flags, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for cmd, p in procs:
        text, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, text))
        elif verbose and text.strip():
            print(text)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(" ".join(c) + "\n" + t for c, t in failed))
    tmp = out.with_suffix(".so.tmp")
    link = [compiler, ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n" + res.stdout)
    os.replace(tmp, out)
    for obj in objs:
        obj.unlink(missing_ok=True)
    return out


if __name__ == "__main__":
    print(build(force=True, verbose=True))
