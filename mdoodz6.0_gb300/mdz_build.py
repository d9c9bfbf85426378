"""Build of the native parts: the CUDA library (sm_103a only) and the CPU
oracle.  Compiles in-tree; outputs are git-ignored.

    libmdoodz_gb300.so   mdoodz6.0_gb300/lib/   product: CUDA kernels + C ABI
    libmdoodz_refshim.so mdoodz6.0_gb300/lib/   product: reference-signature drop-ins over that ABI
    libmdz_oracle.so     oracle/_build/         checker only (tests, smoke, bench's CPU leg)
    libmdoodz_ref.so     oracle/_ref/           reference compiled in place (only where its sources exist)
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libmdoodz_gb300.so")
REFSHIM_LIB = os.path.join(LIBDIR, "libmdoodz_refshim.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "libmdz_oracle.so")
# the reference's SOURCE directory (for the oracle's in-place build and the
# layout check): MDZ_REF_SRC, else the location it has in this container
REF_SRC = os.environ.get("MDZ_REF_SRC", "/root/reference/SOURCE")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code without fused multiply-adds (the box and grid lines of
# PureShearALE are formed on the host and must round as the reference's C)
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "-I" + INCLUDE, "-I" + CSRC, "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def _nvcc():
    for c in ("nvcc", "/usr/local/cuda/bin/nvcc"):
        try:
            subprocess.run([c, "--version"], capture_output=True, check=True)
            return c
        except Exception:
            continue
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build_cuda(verbose=False, extra_flags=()):
    """Compile every csrc/*.cu for sm_103a in parallel and link the C-ABI library."""
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    newest_header = max([os.path.getmtime(h) for h in headers] + [0])
    jobs = []
    for s in sources:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        if (not os.path.exists(o) or os.path.getmtime(o) < os.path.getmtime(s)
                or os.path.getmtime(o) < newest_header or extra_flags):
            jobs.append((s, o))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        futs = [ex.submit(_run, [nvcc] + NVCC_FLAGS + list(extra_flags) + ["-c", s, "-o", o]) for s, o in jobs]
        for f in futs:
            logs.append(f.result())
    objs = [os.path.join(OBJ, os.path.basename(s)[:-3] + ".o") for s in sources]
    if jobs or not os.path.exists(LIB):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    build_refshim()
    if verbose:
        print("".join(logs))
    return LIB


def build_refshim():
    """The reference-signature drop-ins (refshim/mdz_refshim.c) against the
    generated layout view of the reference's structures, linked to the CUDA
    library: lib/libmdoodz_refshim.so."""
    src = os.path.join(PKG, "refshim", "mdz_refshim.c")
    deps = [src, LIB] + glob.glob(os.path.join(INCLUDE, "*.h"))
    if os.path.exists(REFSHIM_LIB) and all(os.path.getmtime(REFSHIM_LIB) >= os.path.getmtime(d) for d in deps):
        return REFSHIM_LIB
    _run(["gcc", "-std=gnu99", "-O2", "-fPIC", "-shared", "-Wall", "-I" + INCLUDE, src, "-o", REFSHIM_LIB,
          "-L" + LIBDIR, "-lmdoodz_gb300", "-Wl,-rpath,$ORIGIN", "-lm"])
    return REFSHIM_LIB


def build_oracle():
    """The oracle: the CPU restatement the tests compare with (plain gcc; builds on x86 and Arm)."""
    _run(["make", "-s", "-C", ORACLE_DIR, "port"])
    return ORACLE_LIB


def build_reference():
    """The reference's own hot-path C files compiled in place (this container only)."""
    if not os.path.isdir(REF_SRC):
        return None
    _run(["make", "-s", "-j8", "-C", ORACLE_DIR, "ref", "REF_SRC=" + REF_SRC])
    return os.path.join(ORACLE_DIR, "_ref", "libmdoodz_ref.so")


def build_all(verbose=False):
    lib = build_cuda(verbose=verbose)
    orc = build_oracle()
    ref = build_reference()
    return lib, orc, ref


if __name__ == "__main__":
    print(build_all(verbose="-v" in sys.argv))
