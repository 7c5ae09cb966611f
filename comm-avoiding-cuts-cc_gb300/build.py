"""Build recipe for libcac (sm_103a), the drop-in command lines, and the oracle.

    python comm-avoiding-cuts-cc_gb300/build.py            # library + CLIs + oracle
    python comm-avoiding-cuts-cc_gb300/build.py --no-oracle

Every CUDA translation unit is compiled by nvcc for exactly one target,
`-gencode arch=compute_103a,code=sm_103a`, in parallel, then linked into lib/libcac.so.
The command lines are plain C++ linked against it with an $ORIGIN rpath. Objects are rebuilt
when a source or header is newer. No cmake, no x86-only flags: the same recipe runs on the
x86-64 build container and on the aarch64 GPU host.
"""
import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
OBJDIR = os.path.join(LIBDIR, "obj")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
CUDA_HOME = os.path.dirname(os.path.dirname(os.path.realpath(NVCC)))
CXX = os.environ.get("CXX", "g++")
NVFLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                  "-I" + os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build_lib(verbose=False, extra_flags=()):
    os.makedirs(OBJDIR, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    jobs = []
    for src in sources:
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        if _newer(obj, [src] + headers) or extra_flags:
            jobs.append((src, obj))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        futs = {ex.submit(_run, [NVCC] + NVFLAGS + list(extra_flags) + ["-c", s, "-o", o]): s for s, o in jobs}
        for f in cf.as_completed(futs):
            logs.append((futs[f], f.result()))
    lib = os.path.join(LIBDIR, "libcac.so")
    objs = [os.path.join(OBJDIR, os.path.basename(s) + ".o") for s in sources]
    if jobs or _newer(lib, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart", "-lpthread"])
    if verbose:
        for s, log in logs:
            if log.strip():
                print("==", os.path.basename(s), "\n", log)
    return lib


def build_cli():
    os.makedirs(BINDIR, exist_ok=True)
    lib = os.path.join(LIBDIR, "libcac.so")
    out = []
    for src in sorted(glob.glob(os.path.join(CLI, "*.cpp"))):
        exe = os.path.join(BINDIR, os.path.splitext(os.path.basename(src))[0])
        if _newer(exe, [src, lib, os.path.join(ROOT, "include", "cac.h")]):
            _run([CXX, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), src, "-o", exe,
                  "-L" + LIBDIR, "-lcac", "-Wl,-rpath,$ORIGIN/../lib", "-Wl,-rpath," + LIBDIR])
        out.append(exe)
    return out


# Where the reference's source tree is mounted: CAC_REFERENCE_ROOT, else the build container's
# mount point. The reference checker under oracle/_ref is built only where that tree exists.
DEFAULT_REFERENCE_ROOT = "/root/reference"


def reference_root():
    return os.environ.get("CAC_REFERENCE_ROOT", DEFAULT_REFERENCE_ROOT)


def build_oracle(ref=None):
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    ref = ref or reference_root()
    if os.path.isdir(ref):
        _run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle", "refbuild"), "REF=" + ref])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--no-oracle", action="store_true")
    ap.add_argument("--reference", default=None,
                    help="reference source tree for oracle/_ref (default: $CAC_REFERENCE_ROOT or %s)"
                    % DEFAULT_REFERENCE_ROOT)
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true", help="print registers / spills / smem per kernel")
    a = ap.parse_args()
    extra = ("-Xptxas", "-v") if a.ptxas_info else ()
    build_lib(verbose=a.verbose or a.ptxas_info, extra_flags=extra)
    build_cli()
    if not a.no_oracle:
        build_oracle(a.reference)
    print("built", os.path.join(LIBDIR, "libcac.so"))


if __name__ == "__main__":
    sys.exit(main())
