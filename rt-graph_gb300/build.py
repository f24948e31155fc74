"""Build librtg.so (CUDA kernels for sm_103a + C++ host code), the drop-in CLIs and the
CPU oracle. Plain nvcc / g++ invocations compiled in parallel; objects are reused when
they are newer than every source and header they could depend on.

Usage: python rt-graph_gb300/build.py [--clean] [--no-cli] [--no-oracle]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
INCLUDE = REPO / "include"
CSRC = PKG / "csrc"
HOST = PKG / "host"
CLI = PKG / "cli"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
BINDIR = PKG / "bin"
LIB = LIBDIR / "librtg.so"
ORACLE = REPO / "oracle"

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
CC = os.environ.get("CC", "gcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))

NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp",
    "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}",
]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall",
             f"-I{INCLUDE}", f"-I{CSRC}", f"-I{CUDA_HOME / 'include'}"]

# the drop-in command-line tools: name -> source (the SI tools share one source that
# selects its kernel family from argv[0])
CLI_TOOLS = {
    "bs_tc": "bs_tc_main.cpp",
    "rt_tc": "rt_tc_main.cpp",
    "bs": "si_main.cpp",
    "hi": "si_main.cpp",
    "ip": "si_main.cpp",
    "bi_naive": "si_main.cpp",
    "bi_dynamic": "si_main.cpp",
    "rt_intersection": "si_main.cpp",
    "convertor": "convertor_main.cpp",
    "s_generator": "s_generator_main.cpp",
    "m_generator": "m_generator_main.cpp",
}


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return sorted(list(INCLUDE.glob("*.h")) + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh"))
                  + list(HOST.glob("*.h")) + list(CLI.glob("*.h")))


def _compile(src: Path, obj: Path, extra: tuple[str, ...] = ()) -> Path:
    obj.parent.mkdir(parents=True, exist_ok=True)
    if src.suffix == ".cu":
        cmd = [NVCC, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [CXX, *CXX_FLAGS, *extra, f"-I{HOST}", "-c", str(src), "-o", str(obj)]
    _run(cmd)
    return obj


# the library variants: the product, and the checked build (every CSR and counting form
# validated on the device before a count, kernel indexes checked; see include/rtg.h)
LIB_VARIANTS = {
    "librtg.so": ("obj", ()),
    "librtg_checked.so": ("obj_checked", ("-DRTG_CHECKED",)),
}


def build_lib(jobs: int | None = None, variants: tuple[str, ...] = tuple(LIB_VARIANTS)) -> Path:
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    hdrs = _headers()
    todo = []
    links = []
    for name in variants:
        objdir, extra = LIB_VARIANTS[name]
        objs = []
        stale = False
        for s in srcs:
            o = BUILD / objdir / (s.name + ".o")
            objs.append(o)
            if _stale(o, [s, *hdrs]):
                todo.append((s, o, extra))
                stale = True
        links.append((LIBDIR / name, objs, stale))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda t: _compile(*t), todo))
    LIBDIR.mkdir(parents=True, exist_ok=True)
    for lib, objs, stale in links:
        if stale or _stale(lib, objs):
            tmp = lib.with_suffix(".so.tmp")
            _run([NVCC, *ARCH, "-shared", "-o", str(tmp), *map(str, objs),
                  "-Xcompiler", "-fopenmp", "-lgomp", "-lcudart"])
            os.replace(tmp, lib)
    return LIB


def build_cli(jobs: int | None = None) -> list[Path]:
    """Host mirror of the reference interface (host/*.cpp) + one executable per tool."""
    if not CLI.exists():
        return []
    hdrs = _headers()
    host_srcs = sorted(HOST.glob("*.cpp"))
    host_objs = []
    todo = []
    for s in host_srcs:
        o = BUILD / "host" / (s.name + ".o")
        host_objs.append(o)
        if _stale(o, [s, *hdrs]):
            todo.append((s, o))
    mains = sorted(set(CLI_TOOLS.values()))
    main_objs = {}
    for m in mains:
        s = CLI / m
        if not s.exists():
            continue
        o = BUILD / "cli" / (m + ".o")
        main_objs[m] = o
        if _stale(o, [s, *hdrs]):
            todo.append((s, o))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda so: _compile(*so), todo))
    BINDIR.mkdir(parents=True, exist_ok=True)
    out = []
    for tool, m in CLI_TOOLS.items():
        if m not in main_objs:
            continue
        exe = BINDIR / tool
        deps = [main_objs[m], *host_objs, LIB]
        if _stale(exe, deps):
            _run([CXX, "-o", str(exe), str(main_objs[m]), *map(str, host_objs),
                  f"-L{LIBDIR}", "-lrtg", f"-Wl,-rpath,{LIBDIR}", f"-L{CUDA_HOME / 'lib64'}",
                  "-lcudart", f"-Wl,-rpath,{CUDA_HOME / 'lib64'}", "-fopenmp"])
        out.append(exe)
    return out


def build_oracle() -> Path | None:
    """The CPU oracle (test infrastructure; never linked into librtg)."""
    src = ORACLE / "rtg_oracle.c"
    if not src.exists():
        return None
    out = ORACLE / "_build" / "liboracle.so"
    out.parent.mkdir(parents=True, exist_ok=True)
    if _stale(out, [src, ORACLE / "rtg_oracle.h"]):
        _run([CC, "-O3", "-fPIC", "-shared", "-fopenmp", "-std=c11", "-Wall",
              str(src), "-o", str(out), "-lm"])
    return out


def build_all(cli: bool = True, oracle: bool = True) -> None:
    build_lib()
    if cli:
        build_cli()
    if oracle:
        build_oracle()


def clean() -> None:
    for d in (BUILD, LIBDIR, BINDIR, ORACLE / "_build"):
        if d.exists():
            shutil.rmtree(d)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    build_all(cli="--no-cli" not in sys.argv, oracle="--no-oracle" not in sys.argv)
    print("built", LIB)
