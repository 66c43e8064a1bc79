"""Build libtg3.so in place with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel, then linked into one shared
library next to this file's package (../libtg3.so).  No cmake, one -gencode.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parents[1]          # thunder-refactor-expectation_gb300/
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_build"
LIB = PKG / "libtg3.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["tg3_kernels.cu", "tg3_api.cu", "tg3_tc.cu", "tg3_fused.cu", "tg3_ragged.cu",
           "tg3_cnn.cu", "tg3_conv_tc.cu", "tg3_noalloc.cu", "tg3_io.cpp", "tg3_prep.cu", "tg3_reco.cu",
           "tg3_learned.cu", "tg3_bank_gemm.cu", "tg3_local2d.cu"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found")
    return cand


def flags(debug: bool = False):
    f = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         f"-I{ROOT / 'include'}", f"-I{CSRC}", "--expt-relaxed-constexpr"] + ARCH
    if debug:
        f += ["-DTG3_DEBUG=1"]
    return f


def _needs(obj: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [ROOT / "include" / "thunder_gb300.h"]
    cc = nvcc()
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = OUT_DIR / (s.stem + ".o")
        if force or _needs(o, [s] + headers):
            jobs.append([cc, *flags(), "-c", str(s), "-o", str(o)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        list(ex.map(run, jobs))
    objs = [str(OUT_DIR / (Path(s).stem + ".o")) for s in SOURCES]
    if force or jobs or not LIB.exists():
        run([cc, *ARCH, "-shared", "-o", str(LIB), *objs, "-lcudart", "-lcufft"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
