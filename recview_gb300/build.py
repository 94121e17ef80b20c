"""Build recipes (no cmake): the CUDA library for sm_103a, the oracle's C restatement and, where
the reference checkout is present, the reference build in oracle/_ref.

    python -m recview_gb300.build            # library + oracle (+ reference build if available)

Everything is built in-tree; outputs are git-ignored.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "librecview_gb300.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "librvoracle.so"
REF_LIB = ORACLE_DIR / "_ref" / "librvref.so"
BUILD_DIR = PKG / "_build"

ARCH = os.environ.get("RV_CUDA_ARCH", "103a")
NVCC_FLAGS = [
    f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}",
    "-O3", "-lineinfo", "-std=c++17",
    # every host-side float expression follows the reference's separate roundings
    "-Xcompiler", "-fPIC,-ffp-contract=off",
    "--expt-relaxed-constexpr",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_lib(force: bool = False, verbose: bool = False) -> Path:
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.h")) + [ROOT / "include" / "recview_gb300.h"]
    if not force and not _stale(LIB, sources + headers + [Path(__file__)]):
        return LIB
    BUILD_DIR.mkdir(exist_ok=True)
    nvcc = _nvcc()
    objs = []
    cmds = []
    for src in sources:
        obj = BUILD_DIR / (src.stem + ".o")
        objs.append(obj)
        cmds.append([nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(len(cmds), os.cpu_count() or 4)) as ex:
        for f in [ex.submit(_run, c) for c in cmds]:
            f.result()
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *NVCC_FLAGS, "-shared", *map(str, objs), "-o", str(tmp)])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(force: bool = False) -> Path:
    src = ORACLE_DIR / "rv_oracle.c"
    deps = [src, ORACLE_DIR / "rv_oracle.h", ROOT / "include" / "recview_gb300.h"]
    if not force and not _stale(ORACLE_LIB, deps):
        return ORACLE_LIB
    cc = os.environ.get("CC", "gcc")
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    _run([cc, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=gnu11", "-o", str(tmp), str(src),
          "-lm", "-lpthread"])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_ref(force: bool = False) -> Path | None:
    """Reference sources compiled by oracle/build_ref.sh (the recipe locates the reference
    checkout; RECVIEW_REFERENCE overrides it); None when the checkout is absent."""
    if REF_LIB.exists() and not force:
        return REF_LIB
    r = subprocess.run(["bash", str(ORACLE_DIR / "build_ref.sh")], capture_output=True, text=True)
    if r.returncode == 3:       # the recipe found no reference checkout
        return None
    if r.returncode != 0:
        raise RuntimeError(f"oracle/build_ref.sh failed ({r.returncode})\n{r.stdout}\n{r.stderr}")
    return REF_LIB


def build_all(force: bool = False, verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f_lib = ex.submit(build_lib, force, verbose)
        f_orc = ex.submit(build_oracle, force)
        f_lib.result()
        f_orc.result()
    try:
        build_ref(force)
    except RuntimeError as e:  # the reference build is optional test infrastructure
        print(f"reference build skipped: {e}", file=sys.stderr)
    if verbose:
        print(f"platform {platform.machine()}: library, oracle"
              + (", reference" if REF_LIB.exists() else ""))


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose=True)
