"""Build the engine's shared library in-tree (no CMake, no torch extension).

CUDA sources are compiled by nvcc for sm_103a only; host C++ by g++.  Objects
compile in parallel and link into ``rebop_gb300/_build/librebop_gb300.so``
with the CUDA runtime linked statically, so the library's only run-time
dependency is the NVIDIA driver.  ``python -m rebop_gb300.build`` runs it.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "librebop_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["ssa_thread.cu", "ssa_fast.cu", "ssa_spec.cu", "ssa_warp.cu", "fp64_peak.cu", "mdn.cu"]
CXX_SOURCES = ["network.cpp", "engine.cpp", "capi.cpp", "ssa_jit.cpp", "batch.cpp", "tune.cpp"]
# Device headers embedded in the library for run-time network compilation.
JIT_HEADERS = ["rtc_types.hpp", "ssa_args.hpp", "b64.cuh", "rng.cuh", "ssa_exact.cuh", "ssa_spec_body.cuh"]
JIT_SOURCES_CPP = "jit_headers.cpp"


def cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _sources() -> list[Path]:
    return ([CSRC / s for s in CUDA_SOURCES + CXX_SOURCES] + sorted(CSRC.glob("*.hpp"))
            + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "rebop_gb300.h"])


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources() if p.exists())


def _write_jit_headers() -> Path:
    """C++ file holding the device headers as string literals."""
    out = ["// generated by rebop_gb300/build.py from csrc/ -- do not edit", "namespace rbg {",
           "extern const char *const kJitHeaderNames[] = {"]
    out += [f'    "{h}",' for h in JIT_HEADERS]
    out += ["};", "extern const char *const kJitHeaderSources[] = {"]
    for h in JIT_HEADERS:
        text = (CSRC / h).read_text()
        if ')RBGJIT"' in text:
            raise RuntimeError(f"{h} holds the raw-string delimiter")
        out.append('    R"RBGJIT(' + text + ')RBGJIT",')
    out += ["};", f"extern const int kJitHeaderCount = {len(JIT_HEADERS)};", "}  // namespace rbg", ""]
    path = BUILD / JIT_SOURCES_CPP
    path.write_text("\n".join(out))
    return path


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    jit_cpp = _write_jit_headers()
    cuda = cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    jobs = []
    for s in CUDA_SOURCES:
        obj = BUILD / (s + ".o")
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", *inc, "-c", str(CSRC / s), "-o", str(obj)])
    for s in CXX_SOURCES:
        obj = BUILD / (s + ".o")
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                     "-Wall", "-Wno-unused-function", *inc, "-I", str(cuda / "include"), "-c", str(CSRC / s),
                     "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-c", str(jit_cpp), "-o", str(BUILD / (JIT_SOURCES_CPP + ".o"))])

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err)
    objs = [str(BUILD / (s + ".o")) for s in CUDA_SOURCES + CXX_SOURCES + [JIT_SOURCES_CPP]]
    tmp = BUILD / f"librebop_gb300.{os.getpid()}.so"
    run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *objs, "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
