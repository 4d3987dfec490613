"""Builds the in-tree CUDA library ``hyperdeal_gb300/_lib/libhyperdeal_gb300.so``.

Every translation unit under ``csrc/`` is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and linked with
the shared CUDA runtime.  The kernel templates are instantiated one
(dimension, nodes per direction) pair per generated unit (``_build/gen/``,
see ``csrc/hd_dispatch.cu``) so that the heavy instantiations compile in
parallel.  Objects are rebuilt when a source or header changes.
"""
from __future__ import annotations

import glob
import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
BUILD_DIR = os.path.join(PKG, "_build")
LIB_NAME = "libhyperdeal_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)
# the bounds-checked variant (-DHD_CHECK): every global load and store of the ECL kernels checks
# its index and records a violation in the operator's device status instead of accessing memory
CHECK_LIB_PATH = os.path.join(OUT_DIR, "libhyperdeal_gb300_check.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _deps_hash(extra: str = "") -> str:
    h = hashlib.sha1(extra.encode())
    for p in sorted(glob.glob(os.path.join(CSRC, "*")) + [os.path.join(ROOT, "include", "hyperdeal_gb300.h")]):
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    return h.hexdigest()


# (family, header, factory) of the generated instantiation units and their (D, N) pairs; the
# generic kernels' ghost-region variants (family ecl_gh) compile in units of their own
GEN_UNITS = ([("ecl", "hd_ecl.cuh", "EclLaunchers", "make_launchers", D, N) for D in range(2, 7) for N in range(2, 7)]
             + [("ecl_gh", "hd_ecl.cuh", None, None, D, N) for D in range(2, 7) for N in range(2, 7)]
             + [("batch", "hd_batch.cuh", "BatchLaunchers", "make_batch_launchers", D, N)
                for D in (4, 5) for N in range(3, 7)]
             + [("gauss", "hd_gauss.cuh", "GaussLaunchers", "make_gauss_launchers", D, N)
                for D in range(2, 7) for N in range(2, 6)])


def _unit_text(fam: str, header: str, ret, factory, D: int, N: int) -> str:
    if fam == "ecl_gh":
        return '#include "%s"\nnamespace hd {\nHD_ECL_GH_INSTANCES(, %d, %d)\n}\n' % (header, D, N)
    extern = "HD_ECL_GH_INSTANCES(extern, %d, %d)\n" % (D, N) if fam == "ecl" else ""
    return ('#include "%s"\nnamespace hd {\n%s%s %s_launchers_%d_%d() { return %s<%d, %d>(); }\n}\n'
            % (header, extern, ret, fam, D, N, factory, D, N))


def _generate_units(build_dir: str = BUILD_DIR) -> list:
    gen = os.path.join(build_dir, "gen")
    os.makedirs(gen, exist_ok=True)
    out = []
    for fam, header, ret, factory, D, N in GEN_UNITS:
        path = os.path.join(gen, "%s_%d_%d.cu" % (fam, D, N))
        text = _unit_text(fam, header, ret, factory, D, N)
        if not os.path.exists(path) or open(path).read() != text:
            with open(path, "w") as f:
                f.write(text)
        out.append(path)
    return out


def build(force: bool = False, verbose: bool = False, jobs: int | None = None, check: bool = False) -> str:
    """Compile and link the library (check=True: the bounds-checked variant); returns its path."""
    build_dir = BUILD_DIR + ("_check" if check else "")
    lib_path = CHECK_LIB_PATH if check else LIB_PATH
    os.makedirs(build_dir, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu"))) + _generate_units(build_dir)
    flags = ARCH + NVCC_FLAGS + ["-I", CSRC] + (["-DHD_CHECK"] if check else [])
    stamp = os.path.join(OUT_DIR, ".stamp_check" if check else ".stamp")
    digest = _deps_hash(" ".join(flags))
    if not force and os.path.exists(lib_path) and os.path.exists(stamp) and open(stamp).read() == digest:
        return lib_path
    os.makedirs(OUT_DIR, exist_ok=True)

    def compile_one(src: str) -> str:
        obj = os.path.join(build_dir, os.path.basename(src) + ".o")
        key = os.path.join(build_dir, os.path.basename(src) + ".key")
        if not force and os.path.exists(obj) and os.path.exists(key) and open(key).read() == digest:
            return obj
        cmd = [nvcc()] + flags + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        with open(key, "w") as f:
            f.write(digest)
        return obj

    jobs = jobs or min(len(sources), max(2, os.cpu_count() or 2))
    # the slowest units first, so that they do not start last
    order = sorted(sources, key=lambda p: (0 if os.path.basename(p).startswith(("ecl_5", "ecl_6", "batch_5"))
                                           else 1 if os.path.basename(p).startswith(("ecl_4", "batch_4")) else 2))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, order))
    tmp = lib_path + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib_path)
    with open(stamp, "w") as f:
        f.write(digest)
    return lib_path


def build_cpp_app(name: str = "advection_hyperrectangle") -> str:
    """Compile a C++ host program of cpp/ against include/hyperdeal_gb300.hpp and the library (g++)."""
    lib = build()
    src = os.path.join(PKG, "cpp", name + ".cc")
    exe = os.path.join(OUT_DIR, name)
    if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(src), os.path.getmtime(lib),
                                                             os.path.getmtime(os.path.join(ROOT, "include",
                                                                                           "hyperdeal_gb300.hpp"))):
        return exe
    cuda_home = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda_home, "include"),
           src, "-o", exe, "-L", OUT_DIR, "-lhyperdeal_gb300", "-Wl,-rpath," + OUT_DIR,
           "-L", os.path.join(cuda_home, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(cuda_home, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed:\n%s\n%s" % (r.stdout, r.stderr))
    return exe


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True, check="--check" in sys.argv))
