"""In-tree build of libmfx.so: CUDA engine (sm_103a) + C++ host library.

Compiles ``csrc/*.cu`` with nvcc for ``sm_103a`` only and ``host/*.cc`` with
g++, in parallel, and links ``monofonic_gb300/_build/libmfx.so`` against
cuFFT.  Objects are rebuilt when a source or any header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
BUILD = PKG / "_build"
LIB = BUILD / "libmfx.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> pathlib.Path:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and pathlib.Path(c, "bin", "nvcc").exists():
            return pathlib.Path(c)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return pathlib.Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: the mfx engine needs the CUDA toolkit")


def _sources():
    cu = sorted((PKG / "csrc").glob("*.cu"))
    cc = sorted((PKG / "host").glob("*.cc"))
    return cu, cc


def _headers():
    hs = list((PKG / "csrc").glob("*.cuh")) + list((PKG / "csrc").glob("*.h"))
    hs += list((PKG / "host").glob("*.h")) + list((ROOT / "include").glob("*.h"))
    return hs


def _stale(obj: pathlib.Path, src: pathlib.Path, hdr_mtime: float) -> bool:
    if not obj.exists():
        return True
    m = obj.stat().st_mtime
    return m < src.stat().st_mtime or m < hdr_mtime


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    (BUILD / "obj").mkdir(parents=True, exist_ok=True)
    cu, cc = _sources()
    hdr_mtime = max((h.stat().st_mtime for h in _headers()), default=0.0)
    inc = ["-I", str(ROOT / "include"), "-I", str(PKG / "csrc"), "-I", str(PKG / "host")]
    jobs = []
    objs = []
    for s in cu:
        o = BUILD / "obj" / (s.stem + ".cu.o")
        objs.append(o)
        if force or _stale(o, s, hdr_mtime):
            jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "--expt-relaxed-constexpr", *inc, "-c", str(s), "-o", str(o)])
    for s in cc:
        o = BUILD / "obj" / (s.stem + ".cc.o")
        objs.append(o)
        if force or _stale(o, s, hdr_mtime):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-I", str(cuda / "include"), *inc,
                         "-c", str(s), "-o", str(o)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp%d" % os.getpid())
        run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcufft", "-lpthread",
             "-Xlinker", "-rpath," + str(cuda / "lib64")])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
