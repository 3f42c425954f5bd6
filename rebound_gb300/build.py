"""Build librebound_gb300.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into
rebound_gb300/librebound_gb300.so.  Kernels whose results must round exactly
like the reference's -ffp-contract=off build (integrators, tree, collisions,
WHFast) are compiled with --fmad=false; the direct-sum force kernels keep FMA.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "librebound_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
          "-diag-suppress", "1444", "-I" + os.path.join(os.path.dirname(HERE), "include")]
# Units whose arithmetic must not be contracted into FMAs.
NO_FMAD = {"sim.cu", "tree.cu", "collide.cu", "whfast.cu", "whfast_prog.cu", "ensemble_exact.cu", "ensemble_dh.cu"}


def elf_matches_host(path):
    """True if `path` is an ELF object for this machine (x86_64 and aarch64 trees differ)."""
    import platform
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if head[:4] != b"\x7fELF" or want is None:
        return False
    return int.from_bytes(head[18:20], "little") == want


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build rebound_gb300")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src, objdir):
    obj = os.path.join(objdir, src + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "rebound_gb300.h"))
    if elf_matches_host(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    flags = list(COMMON)
    if src in NO_FMAD:
        # no contraction in device code, nor in the host code that restates the
        # reference's arithmetic (hardsphere, SEI coefficients, ghost boxes)
        flags += ["--fmad=false", "-Xcompiler", "-ffp-contract=off"]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "cu"] + ARCH + flags + ["-c", path, "-o", obj]
    else:
        cmd = [nvcc()] + ARCH + flags + ["-c", path, "-o", obj]
    subprocess.check_call(cmd)
    return obj


def build(force=False, verbose=True):
    import platform
    objdir = os.path.join(HERE, "_build", platform.machine())
    os.makedirs(objdir, exist_ok=True)
    srcs = sources()
    if not force and elf_matches_host(OUT):
        newest = max(os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC))
        newest = max(newest, os.path.getmtime(os.path.join(os.path.dirname(HERE), "include", "rebound_gb300.h")))
        if os.path.getmtime(OUT) >= newest:
            return OUT
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, objdir), srcs))
    tmp = OUT + ".tmp"
    subprocess.check_call([nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs +
                          ["-lcudart", "-lpthread"])
    os.replace(tmp, OUT)
    if verbose:
        print("built", OUT, file=sys.stderr)
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv)
