"""Build recipe of the CUDA library (nvcc only; no cmake, no torch extension).

Compiles every csrc/*.cu for sm_103a in parallel and links
_build/libletkf_gpu.so in the package directory.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shlex
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libletkf_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def nvcc() -> str:
    p = os.path.join(CUDA_HOME, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src: str, extra: list[str], out: str = OUT, force: bool = False) -> str:
    obj = os.path.join(out, os.path.basename(src)[:-3] + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(REPO, "include", "letkf_gpu.h"))
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", os.path.join(REPO, "include"), "-I", CSRC, "-c", src, "-o", obj, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None, out_dir: str | None = None) -> str:
    """Compile and link the library; returns its path.  `extra` adds nvcc flags
    (e.g. -DLG_PHASE_CLOCKS) and `out_dir` builds into another directory."""
    out = out_dir or OUT
    lib = os.path.join(out, "libletkf_gpu.so")
    os.makedirs(out, exist_ok=True)
    # LETKF_NVCC_FLAGS adds flags to every build (e.g. a kernel variant for
    # a timing comparison, kept through the builds that scripts run first)
    extra = list(extra or []) + shlex.split(os.environ.get("LETKF_NVCC_FLAGS", ""))
    srcs = sources()
    # objects built with other flags are rebuilt (the flags of the last build
    # are kept beside the library)
    stamp = os.path.join(out, "build_flags.txt")
    flags = " ".join(extra)
    force = not os.path.exists(stamp) or open(stamp).read() != flags
    if force and os.path.exists(stamp):
        # a build with new flags that fails part way leaves no stamp, so the
        # next build recompiles every object instead of reusing some by mtime
        os.remove(stamp)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, out, force), srcs))
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-cudart", "shared",
               "-Xlinker", f"-rpath,{os.path.join(CUDA_HOME, 'lib64')}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as f:
        f.write(flags)
    if verbose:
        print(lib)
    return lib


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
