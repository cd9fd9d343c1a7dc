"""Build libfalcon_dsp_gb300.so in-tree with nvcc for sm_103a.

Every CUDA/C++ translation unit under csrc/ (kernels + C ABI) and cpp/ (the
reference-compatible C++ class API) is compiled in parallel and linked into
libfalcon_dsp_gb300/_lib/libfalcon_dsp_gb300.so.  The CUDA runtime is linked
statically so the library loads next to any PyTorch build.

    python -m libfalcon_dsp_gb300.build        # or build() from Python
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CPP = os.path.join(PKG, "cpp")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libfalcon_dsp_gb300.so")
INCLUDE = os.path.join(ROOT, "include")
GEN = os.path.join(OBJ, "gen")  # generated sources (the predefined filter table)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                     "-I", INCLUDE, "-I", CSRC, "-I", os.path.join(CPP, "include"), "-I", GEN]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfalcon_dsp_gb300")
    return cand


def sources() -> list[str]:
    out = []
    for d, exts in ((CSRC, (".cu",)), (CPP, (".cc", ".cu"))):
        if not os.path.isdir(d):
            continue
        for f in sorted(os.listdir(d)):
            if f.endswith(exts):
                out.append(os.path.join(d, f))
    return out


def _headers() -> list[str]:
    hs = []
    for d in (CSRC, INCLUDE, os.path.join(CPP, "include"), GEN):
        for r, _, fs in os.walk(d):
            hs += [os.path.join(r, f) for f in fs if f.endswith((".h", ".cuh", ".hpp", ".inc"))]
    return hs


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    cmd = [nvcc()] + NVCC_FLAGS + extra + lang + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _gen_filter_table() -> None:
    """The predefined resampling filters (filter_design.py, scipy at build
    time) as a C++ include, regenerated when the generator changes."""
    out = os.path.join(GEN, "fdsp_filter_table.inc")
    gen = os.path.join(PKG, "filter_design.py")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(gen):
        return
    from . import filter_design
    filter_design.write_table_inc(out)


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    _gen_filter_table()
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra or []), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
