"""In-tree build of the native parts: the CUDA engine (sm_103a), the
scene generator, the legacy ``pbig.h`` archive and the CPU oracle.

Everything is compiled with plain ``nvcc``/``gcc``/``g++`` command lines into
``pbig_gb300/_build`` (and ``oracle/_build``), a few translation units in
parallel. A stamp records the host architecture so that binaries copied from
another machine are rebuilt rather than loaded.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pbig_gb300")
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "_build")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("PBIG_NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
CUDA_HOME = os.path.dirname(os.path.dirname(os.path.realpath(NVCC)))

ENGINE_SOURCES = ["engine.cu", "kernels.cu", "noalloc.cu", "update.cu", "serve_batch.cu"]
ENGINE_HEADERS = ["kernels.cuh", "engine.h"]

LIB_ENGINE = os.path.join(BUILD, "libpbig_gb300.so")
LIB_GEN = os.path.join(BUILD, "libpbig_gen.so")
LIB_LEGACY = os.path.join(BUILD, "libpbig.a")
LIB_ORACLE = os.path.join(ORACLE_BUILD, "liborc.so")


def _stamp_ok(out_dir: str) -> bool:
    p = os.path.join(out_dir, ".arch")
    try:
        with open(p) as f:
            return f.read().strip() == platform.machine()
    except OSError:
        return False


def _write_stamp(out_dir: str) -> None:
    with open(os.path.join(out_dir, ".arch"), "w") as f:
        f.write(platform.machine())


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}):\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)


def _engine_cmds(extra: list[str]) -> tuple[list[list[str]], list[str]]:
    objs, cmds = [], []
    for src in ENGINE_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        # -ffp-contract=off: the host autotuner rounds like its device twin
        cmds.append([NVCC, *ARCH_FLAGS, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fvisibility=hidden", "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
                     *extra, "-c", os.path.join(CSRC, src), "-o", obj])
    return cmds, objs


def build(verbose: bool = False, force: bool = False, with_oracle: bool = True) -> dict:
    """Compile every native component; returns the paths of the outputs."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    if not _stamp_ok(BUILD):
        force = True
    if with_oracle and not _stamp_ok(ORACLE_BUILD):
        for f in os.listdir(ORACLE_BUILD):
            os.remove(os.path.join(ORACLE_BUILD, f))

    extra = os.environ.get("PBIG_NVCC_EXTRA", "").split()
    engine_deps = [os.path.join(CSRC, f) for f in ENGINE_SOURCES + ENGINE_HEADERS] + \
        [os.path.join(INCLUDE, "pbig2.h")]
    jobs = []

    # 1. CUDA engine: compile objects in parallel, then link the shared lib
    cmds, objs = _engine_cmds(extra)
    need_engine = force or _stale(LIB_ENGINE, engine_deps)

    # 2. generator (host C; no fp contraction so x86 and arm64 agree)
    gen_src = os.path.join(CSRC, "gen.c")
    gen_cmd = ["gcc", "-O2", "-shared", "-fPIC", "-std=c11", "-ffp-contract=off", "-fno-fast-math",
               "-pthread", gen_src, "-o", LIB_GEN, "-lm"]
    need_gen = force or _stale(LIB_GEN, [gen_src])

    # 3. legacy archive (pbig_init / pbig_check / pbig_finalize) built against
    #    include/report.h; clients with their own report.h compile the same
    #    source with their header first on the include path.
    legacy_src = os.path.join(CSRC, "legacy_pbig.cc")
    legacy_obj = os.path.join(BUILD, "legacy_pbig.o")
    legacy_cmd = ["g++", "-O2", "-fPIC", "-std=c++17", "-DDIMS=3", "-I", INCLUDE, "-c", legacy_src,
                  "-o", legacy_obj]
    need_legacy = force or _stale(LIB_LEGACY, [legacy_src, os.path.join(INCLUDE, "pbig2.h"),
                                              os.path.join(INCLUDE, "report.h"),
                                              os.path.join(INCLUDE, "rect.h")])

    # 4. oracle (test infrastructure)
    orc_src = os.path.join(ORACLE, "oracle.c")
    orc_cmd = ["gcc", "-O2", "-shared", "-fPIC", "-std=gnu11", "-pthread", orc_src, "-o", LIB_ORACLE, "-lm"]
    need_orc = with_oracle and (force or _stale(LIB_ORACLE, [orc_src]))

    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        futs = []
        if need_engine:
            futs += [ex.submit(_run, c, verbose) for c in cmds]
        if need_gen:
            futs.append(ex.submit(_run, gen_cmd, verbose))
        if need_legacy:
            futs.append(ex.submit(_run, legacy_cmd, verbose))
        if need_orc:
            futs.append(ex.submit(_run, orc_cmd, verbose))
        for f in futs:
            f.result()
    if need_engine:
        _run([NVCC, *ARCH_FLAGS, "-shared", "-o", LIB_ENGINE, *objs], verbose)
    if need_legacy:
        if os.path.exists(LIB_LEGACY):
            os.remove(LIB_LEGACY)
        _run(["ar", "rcs", LIB_LEGACY, legacy_obj], verbose)
    _write_stamp(BUILD)
    if with_oracle:
        _write_stamp(ORACLE_BUILD)
    return {"engine": LIB_ENGINE, "gen": LIB_GEN, "legacy": LIB_LEGACY,
            "oracle": LIB_ORACLE if with_oracle else None}


def compile_client(sources: list[str], out: str, include_first: list[str] | None = None, std: str = "-std=gnu++14",
                   dims: int = 3, verbose: bool = False, extra: list[str] | None = None) -> str:
    """Build a program that uses the legacy ``pbig.h`` API: the client's own
    sources plus the legacy shim compiled against the client's ``report.h``
    (``include_first`` directories come before ours on the include path, as
    the shim inlines the client's ``report::operator()``)."""
    build(verbose=verbose, with_oracle=False)
    inc = []
    for d in include_first or []:
        inc += ["-I", d]
    shim = os.path.join(os.path.dirname(out) or ".", "legacy_pbig_shim.o")
    _run(["g++", "-O2", "-std=c++17", f"-DDIMS={dims}", *inc, "-I", INCLUDE, "-c",
          os.path.join(CSRC, "legacy_pbig.cc"), "-o", shim], verbose)
    cmd = ["g++", "-O2", std, f"-DDIMS={dims}", *(extra or []), *inc, "-I", INCLUDE, *sources, shim, "-o", out,
           "-L", BUILD, "-lpbig_gb300", f"-Wl,-rpath,{BUILD}"]
    _run(cmd, verbose)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
