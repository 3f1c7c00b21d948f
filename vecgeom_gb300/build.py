"""In-tree build of libvgnav.so for sm_103a (nvcc + g++, no cmake).

Every translation unit is compiled in parallel into ``vecgeom_gb300/_build``
and linked into ``vecgeom_gb300/lib/libvgnav.so``.  The FP64 kernel set is
compiled with ``-fmad=false`` so that no multiply-add is contracted: its
results are bit-identical to the reference's scalar CPU navigator.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libvgnav.so"
PEAK_LIB = LIBDIR / "libvgpeak.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, object name, extra nvcc flags); the navigation kernels are compiled three times:
# with the phi/theta section code (namespace `sections`), without it (`full_ranges`) and with
# the boolean-solid code but not the section code (`booleans`, one launch shape per kernel
# family: with the section code as well this unit compiled for seven minutes)
UNITS = [
    ("kernels_nav.cu", "kernels_nav_sections", ["-fmad=false", "-DVGN_SECTIONS=1"]),
    ("kernels_nav.cu", "kernels_nav_full_ranges", ["-fmad=false", "-DVGN_SECTIONS=0"]),
    ("kernels_nav.cu", "kernels_nav_booleans", ["-fmad=false", "-DVGN_SECTIONS=0", "-DVGN_BOOLEANS=1"]),
    ("kernels_sort.cu", "kernels_sort", []),
    ("host_geometry.cpp", "host_geometry", []),
    ("host_shapes.cpp", "host_shapes", []),
    ("vgnav_api.cpp", "vgnav_api", []),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvgnav")


def _compile(nvcc: str, src: str, name: str, extra: list[str]) -> Path:
    out = BUILD / (name + ".o")
    srcp = CSRC / src
    deps = [srcp] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.inc"))
    deps += [INCLUDE / "vgnav.h"]
    if out.exists() and out.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return out
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE), "-I", str(CSRC)]
    common += os.environ.get("VGN_NVCC_FLAGS", "").split()  # extra defines for build experiments
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, "-lineinfo", "-Xptxas", "-v", *common, *extra, "-c", str(srcp), "-o", str(out)]
    else:
        cmd = [nvcc, "-x", "c++", *common, "-Xcompiler", "-ffp-contract=off", *extra, "-c", str(srcp), "-o", str(out)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    (BUILD / (name + ".ptxas.txt")).write_text(res.stderr)
    return out


def build(verbose: bool = False) -> Path:
    """Compile (incrementally) and link libvgnav.so; returns its path."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(lambda u: _compile(nvcc, *u), UNITS))
    if not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-cudart", "static", "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    # FMA throughput probe used by bench.py for the compute roofline (not part of libvgnav)
    peak_src = CSRC / "peak_fp.cu"
    if not PEAK_LIB.exists() or PEAK_LIB.stat().st_mtime < peak_src.stat().st_mtime:
        cmd = [nvcc, *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", str(peak_src), "-o", str(PEAK_LIB),
               "-cudart", "static"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
