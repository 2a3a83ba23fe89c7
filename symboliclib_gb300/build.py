"""In-tree build of the engine's native libraries (no CMake, no setuptools).

    python -m symboliclib_gb300.build            # build what is out of date
    python -m symboliclib_gb300.build --force    # rebuild everything

Produces
    symboliclib_gb300/lib/libsymgb.so            front end + device engine (C ABI: include/symgb.h)
    symboliclib_gb300/lib/libsymgb_workloads.so  synthetic workloads (tests, benchmark)
    oracle/_build/liboracle.so                   CPU oracle (test infrastructure only)

CUDA code is compiled for sm_103a only.  Host code is portable C/C++ (the
same sources build on x86-64 and aarch64).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIB = PKG / "lib"
OBJ = PKG / "_build"
ORACLE_BUILD = ROOT / "oracle" / "_build"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
CXX = os.environ.get("CXX", "g++")
CC = os.environ.get("CC", "gcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-pthread", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
            f"-I{INCLUDE}"]
NVCCFLAGS = ARCH + ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INCLUDE}",
                    "-Xptxas", "-warn-spills"]

FRONTEND = sorted((CSRC / "frontend").glob("*.cpp"))
ENGINE_CPP = [CSRC / "engine" / "program.cpp", CSRC / "engine" / "codegen.cpp"]
PRELUDE = CSRC / "engine" / "jit_prelude.cuh"
ENGINE_CU = sorted((CSRC / "engine").glob("*.cu"))
WORKLOADS = [CSRC / "workloads" / "workloads_capi.cpp"]
ORACLE_SRC = [ROOT / "oracle" / "evaluate.c"]


def _headers() -> list[Path]:
    return (list(INCLUDE.rglob("*.h")) + list(INCLUDE.rglob("*.hpp")) + list(CSRC.rglob("*.hpp"))
            + list(CSRC.rglob("*.cuh")) + [Path(__file__)])


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _compile(src: Path, force: bool, hdrs: list[Path]) -> Path:
    out = OBJ / (src.parent.name + "_" + src.name + ".o")
    if force or _stale(out, [src] + hdrs):
        if src.suffix == ".cu":
            _run([NVCC] + NVCCFLAGS + ["-c", str(src), "-o", str(out)])
        elif src.suffix == ".c":
            _run([CC, "-std=c99", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", f"-I{INCLUDE}",
                  "-c", str(src), "-o", str(out)])
        else:
            _run([CXX] + CXXFLAGS + [f"-I{CSRC / 'engine'}", "-c", str(src), "-o", str(out)])
    return out


def _prelude_source() -> Path:
    """The compiled executor's device prelude (jit_prelude.cuh) as a C++ string
    constant, handed to NVRTC at the head of every generated module."""
    out = OBJ / "jit_prelude_text.cpp"
    text = PRELUDE.read_text()
    body = ("namespace symgb {\nnamespace engine {\nextern const char* const kJitPrelude;\n"
            f'const char* const kJitPrelude = R"SYMGB_PRELUDE({text})SYMGB_PRELUDE";\n}}\n}}\n')
    if not out.exists() or out.read_text() != body:
        out.write_text(body)
    return out


def build(force: bool = False, verbose: bool = False) -> dict[str, Path]:
    if not Path(NVCC).exists():
        raise RuntimeError(f"nvcc not found at {NVCC}")
    for d in (LIB, OBJ, ORACLE_BUILD):
        d.mkdir(parents=True, exist_ok=True)
    hdrs = _headers()
    prelude = _prelude_source()
    srcs = FRONTEND + ENGINE_CPP + [prelude] + ENGINE_CU + WORKLOADS + ORACLE_SRC
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = dict(zip(srcs, ex.map(lambda s: _compile(s, force, hdrs), srcs)))

    cudalib = str(CUDA_HOME / "lib64")
    libsymgb = LIB / "libsymgb.so"
    core = [objs[s] for s in FRONTEND + ENGINE_CPP + [prelude] + ENGINE_CU]
    if force or _stale(libsymgb, core):
        _run([NVCC] + ARCH + ["-shared", "-o", str(libsymgb)] + [str(o) for o in core]
             + ["-lcudart", "-lnvrtc", "-lpthread", f"-L{cudalib}", "-Xlinker", f"-rpath={cudalib}"])
    libw = LIB / "libsymgb_workloads.so"
    wobjs = [objs[s] for s in WORKLOADS]
    if force or _stale(libw, wobjs + [libsymgb]):
        _run([CXX, "-shared", "-o", str(libw)] + [str(o) for o in wobjs]
             + [f"-L{LIB}", "-lsymgb", "-lpthread", "-Wl,-rpath,$ORIGIN"])
    liboracle = ORACLE_BUILD / "liboracle.so"
    oobjs = [objs[s] for s in ORACLE_SRC]
    if force or _stale(liboracle, oobjs):
        _run([CC, "-shared", "-o", str(liboracle)] + [str(o) for o in oobjs] + ["-lm"])
    out = {"symgb": libsymgb, "workloads": libw, "oracle": liboracle}
    if verbose:
        for k, v in out.items():
            print(f"{k}: {v}")
    return out


def clean() -> None:
    for d in (LIB, OBJ, ORACLE_BUILD):
        if d.exists():
            shutil.rmtree(d)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    build(force="--force" in sys.argv, verbose=True)
