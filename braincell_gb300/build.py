"""In-tree build of the native library ``braincell_gb300/_native/libbraincell_gb300.so``.

Every translation unit is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked with the
static CUDA runtime.  Host code is plain C++17 (no x86 intrinsics), so the same
recipe builds on x86_64 and aarch64.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys

__all__ = ["build_native", "NATIVE_DIR", "SOURCES"]

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
NATIVE_DIR = os.path.join(HERE, "_native")
LIB = os.path.join(NATIVE_DIR, "libbraincell_gb300.so")
SOURCES = ["bc_kernels.cu", "bc_gru.cu", "bc_plan.cpp", "bc_lower.cpp"]
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the GB300 library cannot be built without the CUDA toolkit.")


def _flags(debug: bool) -> list[str]:
    f = [
        GENCODE,
        "-std=c++17",
        "-O3" if not debug else "-O0",
        "-lineinfo",
        "-Xcompiler",
        "-fPIC",
        "-Xcompiler",
        "-Wall",
        "-Xcompiler",
        "-pthread",
        "--expt-relaxed-constexpr",
        "-I" + os.path.join(HERE, "..", "include"),
    ]
    return f


def build_native(force: bool = False, verbose: bool = False, debug: bool = False, ptxas_info: bool = False,
                 defines: tuple = (), out: str | None = None) -> str:
    """Compile (if stale) and return the path of the shared library.

    ``defines`` adds ``-D`` macros (e.g. ``("BC_PHASE_TIMERS",)`` for the cycle
    counters); ``out`` writes the library elsewhere than the in-tree default.
    """
    lib_path = out or LIB
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    inc = os.path.join(HERE, "..", "include")
    deps += [os.path.join(inc, h) for h in os.listdir(inc) if h.endswith(".h")]
    if not force and os.path.exists(lib_path):
        lib_m = os.path.getmtime(lib_path)
        if all(os.path.getmtime(d) <= lib_m for d in deps if os.path.exists(d)):
            return lib_path
    os.makedirs(NATIVE_DIR, exist_ok=True)
    nvcc = _nvcc()
    objs = []
    procs = []
    for s in srcs:
        obj = os.path.join(NATIVE_DIR, os.path.basename(s) + ".o")
        objs.append(obj)
        cmd = [nvcc, "-x", "cu", "-c", s, "-o", obj] + _flags(debug) + ["-D" + d for d in defines]
        if ptxas_info and s.endswith(".cu"):
            cmd += ["-Xptxas", "-v"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((s, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    errors = []
    for s, pr in procs:
        log, _ = pr.communicate()
        if pr.returncode != 0:
            errors.append(f"--- {os.path.basename(s)} ---\n{log}")
        elif (verbose or ptxas_info) and log:
            print(log, file=sys.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    os.makedirs(os.path.dirname(os.path.abspath(lib_path)), exist_ok=True)
    tmp = lib_path + ".tmp"
    link = [nvcc, "-shared", GENCODE, "-o", tmp] + objs + ["-cudart", "static", "-lpthread"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout)
    os.replace(tmp, lib_path)
    for o in objs:
        try:
            os.remove(o)
        except OSError:
            pass
    return lib_path


if __name__ == "__main__":
    print(build_native(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
