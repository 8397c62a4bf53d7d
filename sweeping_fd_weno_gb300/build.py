"""In-tree build of the CUDA library libswfd.so (sm_103a only).

Each translation unit is compiled by its own nvcc process in parallel, then
linked into ``sweeping_fd_weno_gb300/_lib/libswfd.so``.  The library is built
with ``-fmad=false``: the reference's x86-64 build forms no fused multiply-add,
and the FP64 path must round every product and sum the way it does.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
BUILD = PKG / "_build"
SOURCES = ["swfd_api.cu", "swfd_kernels.cu", "swfd_sweep.cu", "swfd_ubar.cu", "swfd_control.cu",
           "swfd_static.cu", "swfd_batch.cu", "swfd_matlab1d.cu", "swfd_ex7.cu", "swfd_solve1d.cu"]
# measurement and test probes (include/swfd_probe.h): a library of their own
PROBE_SOURCES = ["swfd_probe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libswfd")


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src, *CSRC.glob("*.h"), *CSRC.glob("*.cuh"), *(PKG.parent / "include").glob("*.h"),
            Path(__file__)]
    return any(d.stat().st_mtime > obj.stat().st_mtime for d in deps if d.exists())


def build(verbose: bool = False, force: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile every .cu translation unit and link libswfd.so; return its path."""
    BUILD.mkdir(exist_ok=True)
    OUT.mkdir(exist_ok=True)
    cc = nvcc()
    flags = NVCC_FLAGS + list(extra_flags or [])
    jobs = []
    for name in SOURCES + PROBE_SOURCES:
        src = CSRC / name
        obj = BUILD / (Path(name).stem + ".o")
        if force or _stale(obj, src):
            jobs.append([cc, *ARCH, *flags, "-I", str(PKG.parent / "include"), "-c", str(src),
                         "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        results = list(ex.map(lambda cmd: subprocess.run(cmd, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if verbose or r.returncode != 0:
            print(" ".join(cmd))
            print(r.stdout, r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    lib = OUT / "libswfd.so"
    objs = [str(BUILD / (Path(n).stem + ".o")) for n in SOURCES]
    if force or jobs or not lib.exists():
        cmd = [cc, *ARCH, "-shared", "-o", str(lib), *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            print(" ".join(cmd))
            print(r.stdout, r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc link of libswfd.so failed")
    probe = OUT / "libswfd_probe.so"
    pobjs = [str(BUILD / (Path(n).stem + ".o")) for n in PROBE_SOURCES]
    if force or jobs or not probe.exists():
        cmd = [cc, *ARCH, "-shared", "-o", str(probe), *pobjs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            print(" ".join(cmd))
            print(r.stdout, r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc link of libswfd_probe.so failed")
    # the C host request loop over the batch API (host/swfd_serve.c)
    serve, src = OUT / "swfd_serve", PKG / "host" / "swfd_serve.c"
    if force or not serve.exists() or serve.stat().st_mtime < max(src.stat().st_mtime,
                                                                  lib.stat().st_mtime):
        cuda_lib = Path(cc).resolve().parent.parent / "lib64"
        cmd = ["gcc", "-O2", "-std=c11", "-Wall", "-I", str(PKG.parent / "include"), str(src),
               "-L", str(OUT), "-lswfd", "-L", str(cuda_lib), "-lcudart", "-lpthread", "-lm",
               "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + str(cuda_lib), "-o", str(serve)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            print(" ".join(cmd))
            print(r.stdout, r.stderr)
        if r.returncode != 0:
            raise RuntimeError("gcc build of swfd_serve failed")
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
