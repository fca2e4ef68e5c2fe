"""In-tree build of the sm_103a backend library and of the oracle checker.

`build_backend()` compiles every `csrc/*.cu` to an object in parallel with nvcc
(`-gencode arch=compute_103a,code=sm_103a`) and links `libstwo_gb300.so` next to this file.
`build_oracle()` compiles the CPU oracle (test infrastructure) with g++ into `oracle/_build/`.
Both skip work when outputs are newer than their sources. No cmake; a couple of minutes at most.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libstwo_gb300.so")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE, "_build", "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _write_codegen_headers() -> None:
    """The two headers that generated constraint kernels compile against (NVRTC has no file
    system view of the package), as C++ raw strings in _build/codegen_headers.inc; rewritten only
    when they change."""
    out = os.path.join(BUILD, "codegen_headers.inc")
    parts = []
    for var, name in (("kFieldCuh", "field.cuh"), ("kCodegenRtCuh", "codegen_rt.cuh")):
        with open(os.path.join(CSRC, name)) as f:
            text = f.read()
        assert ")STWORT" not in text
        parts.append(f'static const char {var}[] = R"STWORT({text})STWORT";\n')
    body = "// Generated by stwo_gb300/build.py from csrc/field.cuh and csrc/codegen_rt.cuh.\n" + "".join(parts)
    if not os.path.exists(out) or open(out).read() != body:
        with open(out, "w") as f:
            f.write(body)


def build_backend(force: bool = False, verbose: bool = False) -> str:
    """Compile and link libstwo_gb300.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    # The Poseidon252 round-constant table is generated from the hash's published constant
    # derivation (rewritten only when it differs).
    _run([sys.executable, os.path.join(CSRC, "gen_poseidon252_constants.py")])
    _write_codegen_headers()
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    nvcc = _nvcc()
    hdr_time = _newest(headers)
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            jobs.append([nvcc, *NVCC_FLAGS, "-I", BUILD, "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for r in ex.map(_run, jobs):
                if verbose and (r.stdout or r.stderr):
                    sys.stderr.write(r.stdout + r.stderr)
    if force or jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        tmp = LIB + ".tmp"
        _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lnvrtc"])
        os.replace(tmp, LIB)
    return LIB


def build_oracle(force: bool = False) -> str:
    """Compile the oracle (C++ restatement of the reference; the checker) into oracle/_build."""
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    srcs = glob.glob(os.path.join(ORACLE, "*.cpp"))
    deps = srcs + glob.glob(os.path.join(ORACLE, "*.h"))
    if force or not os.path.exists(ORACLE_LIB) or os.path.getmtime(ORACLE_LIB) < _newest(deps):
        tmp = ORACLE_LIB + ".tmp"
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", *sorted(srcs), "-o", tmp])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


if __name__ == "__main__":
    print(build_backend(force="--force" in sys.argv, verbose=True))
    print(build_oracle(force="--force" in sys.argv))
