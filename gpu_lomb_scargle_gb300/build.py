"""Build recipe of the native libraries (no cmake; nvcc + the host compiler).

Outputs, in ``gpu_lomb_scargle_gb300/lib/``:

* ``liblsgb.so``                -- the engine and its ``lsgb_*`` C ABI (include/lsgb.h);
* ``libpyls{noerror,error}{float,double}.so`` -- the four drop-in libraries exporting
  ``LombScarglePy`` (include/lombscargle_py.h), the file names
  source/lombscarglegpu.py:279-287 loads;
* ``lsgb_main`` -- the command-line front end (the reference's paper and release CLIs).

Device code is compiled once, for sm_103a only, and linked into every library.
Objects are rebuilt only when a source or header is newer than them.
Usage: ``python -m gpu_lomb_scargle_gb300.build [--force] [--jobs N]``.
"""
from __future__ import annotations

import argparse
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
OBJ = LIB / "obj"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
               "-fvisibility=hidden", "-I", str(INCLUDE)]
HOST_FLAGS = ["-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fopenmp"]

VARIANTS = {
    "libpylsnoerrorfloat.so": ("0", "float"),
    "libpylsnoerrordouble.so": ("0", "double"),
    "libpylserrorfloat.so": ("1", "float"),
    "libpylserrordouble.so": ("1", "double"),
}

HEADERS = [CSRC / "lsgb_internal.h", CSRC / "lsgb_device.h", CSRC / "lsgb_cpu.h", INCLUDE / "lsgb.h",
           INCLUDE / "lombscargle_py.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the engine has no CPU build, CUDA is required")


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd, force: bool, out: Path, deps):
    if not force and not _stale(out, deps):
        return out, "cached"
    out.parent.mkdir(parents=True, exist_ok=True)
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return out, (p.stdout + p.stderr).strip()


def build(force: bool = False, jobs: int = 0, verbose: bool = False) -> Path:
    nv = nvcc()
    OBJ.mkdir(parents=True, exist_ok=True)
    jobs = jobs or min(8, os.cpu_count() or 4)
    compile_steps = []
    k_obj = OBJ / "lsgb_kernels.o"
    compile_steps.append(([nv, *ARCH, *NVCC_COMMON, "-Xptxas", "-v", "-c",
                           str(CSRC / "lsgb_kernels.cu"), "-o", str(k_obj)],
                          k_obj, [CSRC / "lsgb_kernels.cu", *HEADERS]))
    t_obj = OBJ / "lsgb_tensor.o"
    compile_steps.append(([nv, *ARCH, *NVCC_COMMON, "-Xptxas", "-v", "-c",
                           str(CSRC / "lsgb_tensor.cu"), "-o", str(t_obj)],
                          t_obj, [CSRC / "lsgb_tensor.cu", *HEADERS]))
    n_obj = OBJ / "lsgb_noalloc.o"
    compile_steps.append(([nv, *ARCH, *NVCC_COMMON, "-c", str(CSRC / "lsgb_noalloc.cu"), "-o",
                           str(n_obj)], n_obj, [CSRC / "lsgb_noalloc.cu", *HEADERS]))
    s_obj = OBJ / "lsgb_server.o"
    compile_steps.append(([nv, *NVCC_COMMON, *HOST_FLAGS, "-c", str(CSRC / "lsgb_server.cpp"),
                           "-o", str(s_obj)], s_obj, [CSRC / "lsgb_server.cpp", *HEADERS]))
    e_obj = OBJ / "lsgb_engine.o"
    compile_steps.append(([nv, *NVCC_COMMON, *HOST_FLAGS, "-c", str(CSRC / "lsgb_engine.cpp"),
                           "-o", str(e_obj)], e_obj, [CSRC / "lsgb_engine.cpp", *HEADERS]))
    v_objs = {}
    for lib, (err, dt) in VARIANTS.items():
        o = OBJ / (lib.replace(".so", "") + "_pyabi.o")
        v_objs[lib] = o
        compile_steps.append(([nv, *NVCC_COMMON, *HOST_FLAGS, f"-DLS_ERROR={err}",
                               f"-DLS_DTYPE={dt}", "-c", str(CSRC / "lsgb_pyabi.cpp"), "-o", str(o)],
                              o, [CSRC / "lsgb_pyabi.cpp", *HEADERS]))
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(_run, c, force, o, d) for c, o, d in compile_steps]
        for f in futs:
            out, log = f.result()
            if verbose and log and log != "cached":
                print(f"[{out.name}]\n{log}")
    link = [nv, *ARCH, "-shared", "-cudart", "shared", "-Xcompiler", "-fopenmp"]
    link_steps = [(link + [str(k_obj), str(t_obj), str(e_obj), str(n_obj), str(s_obj), "-o",
                           str(LIB / "liblsgb.so"), "-lpthread"],
                   LIB / "liblsgb.so", [k_obj, t_obj, e_obj, n_obj, s_obj])]
    for lib, o in v_objs.items():
        link_steps.append((link + [str(o), str(k_obj), str(t_obj), str(e_obj), "-o", str(LIB / lib)],
                           LIB / lib, [o, k_obj, t_obj, e_obj]))
    cli = LIB / "lsgb_main"
    link_steps.append(([nv, *NVCC_COMMON, *HOST_FLAGS, "-O2", str(CSRC / "lsgb_cli.cpp"), "-o",
                        str(cli), "-ldl"],
                       cli, [CSRC / "lsgb_cli.cpp", CSRC / "lsgb_cpu.h", INCLUDE / "lsgb.h"]))
    with cf.ThreadPoolExecutor(jobs) as ex:
        for f in [ex.submit(_run, c, force, o, d) for c, o, d in link_steps]:
            f.result()
    return LIB


def build_oracle(force: bool = False) -> Path:
    """Compile the test-only C oracle (oracle/_build/liblsoracle.so)."""
    out = ROOT / "oracle" / "_build" / "liblsoracle.so"
    src = ROOT / "oracle" / "ls_oracle.c"
    if force or _stale(out, [src]):
        out.parent.mkdir(parents=True, exist_ok=True)
        cc = os.environ.get("CC", "gcc")
        subprocess.run([cc, "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                        "-fvisibility=hidden", str(src), "-o", str(out), "-lm"], check=True)
    return out


def build_reference_cpu() -> bool:
    """Compile the reference's own sources into oracle/_ref/ when they are present (the
    recipe, oracle/Makefile, finds the checkout: LSGB_REFERENCE_DIR); machines that only
    run the tests have no checkout, and the recipe then builds nothing."""
    p = subprocess.run(["make", "-C", str(ROOT / "oracle"), "ref-if-present", "-j4"],
                       capture_output=True, text=True)
    if p.returncode != 0:
        print(p.stdout[-2000:], p.stderr[-2000:], file=sys.stderr)
        return False
    return (ROOT / "oracle" / "_ref" / "libpylsnoerrordouble.so").exists()


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=0)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    lib = build(force=a.force, jobs=a.jobs, verbose=a.verbose)
    build_oracle(force=a.force)
    print(lib)


if __name__ == "__main__":
    main()
