"""Build the word-hit stage library (libhblast_gb300.so) in-tree with nvcc.

One -gencode (sm_103a), translation units compiled in parallel, objects in
h-blast_gb300/_build/.  The library is rebuilt when any source is newer than
it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # h-blast_gb300/
REPO_ROOT = PKG_ROOT.parent
LIB_PATH = PKG_ROOT / "libhblast_gb300.so"
BUILD_DIR = PKG_ROOT / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build the library")
    return cand


def sources() -> list[Path]:
    srcs = sorted((PKG_ROOT / "csrc").glob("*.cu")) + sorted((PKG_ROOT / "host").glob("*.cpp"))
    return srcs


def _deps() -> list[Path]:
    return (sources() + sorted((PKG_ROOT / "csrc").glob("*.h")) + sorted((PKG_ROOT / "csrc").glob("*.inc"))
            + sorted((PKG_ROOT / "host").glob("*.h")) + sorted((REPO_ROOT / "include").glob("*.h")))


def up_to_date() -> bool:
    if not LIB_PATH.exists():
        return False
    t = LIB_PATH.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB_PATH
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "-I", str(REPO_ROOT / "include")]

    def compile_one(src: Path) -> Path:
        obj = BUILD_DIR / (src.stem + (".cu.o" if src.suffix == ".cu" else ".cpp.o"))
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, *common, "-c", str(src), "-o", str(obj)]
        else:
            cmd = [nvcc, *common, "-x", "c++", "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
