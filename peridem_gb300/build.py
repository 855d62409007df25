"""In-tree build of the CUDA engine (nvcc, sm_103a) into peridem_gb300/_lib/.

Translation units compile in parallel; the FP64 kernels and the engine compile with
-fmad=false so that every FP64 multiply and add rounds separately, as in the reference's
compiled CPU code. The result is one shared library exporting the C-ABI of
include/peridem_gb300.h plus the drop-in `simulate3d` executable.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIBDIR = HERE / "_lib"
LIBNAME = "libperidem_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags)
UNITS = [
    ("pd_kernels.cu", ["-fmad=false"]),
    ("pd_broadphase.cu", []),
    ("pd_fp32c.cu", []),
    ("pd_noalloc.cu", []),
    ("pd_pairs.cu", ["-fmad=false"]),
    ("pd_sell.cu", []),
    ("pd_engine.cu", ["-fmad=false"]),
    ("pd_capi.cpp", []),
    ("pd_batch.cpp", []),
    ("pd_frames.cpp", []),
    ("pd_config.cpp", []),
    ("pd_files.cpp", []),
    ("h5lite.cpp", []),
]
EXE_UNITS = [("simulate3d.cpp", [])]


def nvcc_path() -> str:
    for cand in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        p = Path(cand) / "bin" / "nvcc"
        if cand and p.exists():
            return str(p)
    p = shutil.which("nvcc")
    if not p:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build peridem_gb300")
    return p


def _flags() -> list[str]:
    return ["-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
            "-I", str(ROOT / "include"), "-I", str(CSRC)]


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _headers() -> list[Path]:
    return [*CSRC.glob("*.h"), *CSRC.glob("*.cuh"), ROOT / "include" / "peridem_gb300.h"]


def _compile(nvcc: str, src: str, extra: list[str], verbose: bool) -> Path:
    s = CSRC / src
    o = BUILD / (src + ".o")
    if _stale(o, [s, *_headers(), Path(__file__)]):
        cmd = [nvcc, *_flags(), *extra, "-c", str(s), "-o", str(o)]
        if verbose and src.endswith(".cu"):
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)
    return o


def build_engine(verbose: bool = False) -> Path:
    """Compile the engine library and the drop-in executable; return the library path."""
    nvcc = nvcc_path()
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    units = [u for u in UNITS if (CSRC / u[0]).exists()]
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda u: _compile(nvcc, u[0], u[1], verbose), units))
        exe_objs = list(ex.map(lambda u: _compile(nvcc, u[0], u[1], verbose),
                               [u for u in EXE_UNITS if (CSRC / u[0]).exists()]))
    lib = LIBDIR / LIBNAME
    if _stale(lib, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if exe_objs:
        exe = LIBDIR / "simulate3d"
        if _stale(exe, [*exe_objs, lib]):
            cmd = [nvcc, *ARCH, "-o", str(exe), *map(str, exe_objs), "-L", str(LIBDIR), "-lperidem_gb300",
                   "-Xlinker", "-rpath,$ORIGIN"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link of simulate3d failed:\n{r.stdout}\n{r.stderr}")
    return lib


def build_oracle(verbose: bool = False) -> None:
    """Compile the CPU oracle (test infrastructure) and, when the reference sources are
    present on this machine, the reference itself against the stand-in headers."""
    odir = ROOT / "oracle"
    r = subprocess.run(["make", "-C", str(odir)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    # PeriDEM's sources: PD_REFERENCE_DIR, else a checkout named `reference` beside this repository
    ref = Path(os.environ.get("PD_REFERENCE_DIR") or (ROOT.parent / "reference"))
    if (ref / "run" / "simulate3d.cpp").exists():
        r = subprocess.run(["make", "-C", str(odir), "ref", f"REF={ref}"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stdout)


if __name__ == "__main__":
    build_engine(verbose="-v" in sys.argv)
    build_oracle(verbose="-v" in sys.argv)
    print("built", LIBDIR / LIBNAME)
