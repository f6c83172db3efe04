"""In-tree build of the native library (nvcc, sm_103a only).

Outputs mpm_engine_gb300/_build/libgbmpm.so: one nvcc per translation unit, run in
parallel, then one link. Nothing is installed into site-packages.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PACKAGE_DIR = Path(__file__).resolve().parent
REPO = PACKAGE_DIR.parent
CSRC = PACKAGE_DIR / "csrc"
OUT_DIR = PACKAGE_DIR / "_build"
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (CUDA toolkit required to build libgbmpm.so)")


# deterministic.cu states its arithmetic operation by operation: no product may be
# contracted into an FMA there
PER_TU_FLAGS = {"deterministic.cu": ["--fmad=false"]}


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def build_native(verbose: bool = False, force: bool = False) -> Path:
    """Compiles every csrc/*.cu to an object in parallel (one nvcc per translation
    unit, sm_103a), then links them into libgbmpm.so."""
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    out = OUT_DIR / "libgbmpm.so"
    deps = sources() + sorted(CSRC.glob("*.cuh")) + [REPO / "include" / "gbmpm.h"]
    if out.exists() and not force and all(out.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return out
    nvcc = nvcc_path()
    common = [GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(REPO / "include")]
    if verbose:
        common.append("-Xptxas=-v")
    procs = []
    objs = []
    for src in sources():
        obj = OUT_DIR / (src.stem + ".o")
        objs.append(obj)
        extra = PER_TU_FLAGS.get(src.name, [])
        cmd = [nvcc] + common + extra + ["-c", "-o", str(obj), str(src)]
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    logs = []
    failed = []
    for src, pr in procs:
        text, _ = pr.communicate()
        logs.append(text)
        if pr.returncode != 0:
            failed.append(f"{src.name}:\n{text}")
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    res = subprocess.run([nvcc, GENCODE, "-shared", "-o", str(out)] + [str(o) for o in objs],
                         capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + res.stdout + res.stderr)
    if verbose:
        print("\n".join(logs) + res.stdout + res.stderr)
    return out


if __name__ == "__main__":
    import sys
    print(build_native(verbose="-v" in sys.argv, force="-f" in sys.argv))
