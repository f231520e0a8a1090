"""Build recipe of libcupic_gpu.so (sm_103a), in-tree under cupic_gb300/_build.

Translation units are compiled in parallel with nvcc, one -gencode, then
linked into one shared library.  -fmad=false keeps every float/double
operation separately rounded (fused multiply-adds are written out
explicitly), which is what lets the CPU oracle match results bit for bit;
-ffp-contract=off does the same for the host compiler.
"""
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcupic_gpu.so")
EXE = os.path.join(OUT, "cupic_run")
REF_LIB = os.path.join(OUT, "libcupic_ref.so")
SOURCES = ["capi.cu", "particles.cu", "jacobi.cu", "io.cu", "noalloc.cu", "refine.cu", "batch.cu",
           "files.cpp"]
MAIN = "cupic_main.cpp"
REF_API = "ref_api.cpp"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build cupic_gb300")
    return cand


def common_flags():
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
        "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
        "-I", os.path.join(HERE, "..", "include"),
    ]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _arch_changed(out_dir):
    """True when out_dir was built on another host architecture (objects
    built on x86_64 do not run on the aarch64 GPU hosts and vice versa)."""
    stamp = os.path.join(out_dir, ".arch")
    cur = platform.machine()
    old = open(stamp).read().strip() if os.path.exists(stamp) else ""
    if old != cur:
        with open(stamp, "w") as f:
            f.write(cur)
        return True
    return False


def build(force=False, verbose=False):
    """Compile (if stale) and return the path of libcupic_gpu.so."""
    os.makedirs(OUT, exist_ok=True)
    force = _arch_changed(OUT) or force
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "cupic_gpu.h"))
    cc = nvcc()
    procs, objs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [cc] + common_flags() + ["-c", s, "-o", o]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode:
            failed.append(src)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    if force or procs or _stale(LIB, objs):
        cmd = [cc] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
        subprocess.run(cmd, check=True)
    gxx = [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-I", os.path.join(HERE, "..", "include")]
    link = ["-L", OUT, "-lcupic_gpu", "-Wl,-rpath,$ORIGIN"]
    headers.append(os.path.join(HERE, "..", "include", "cupic_ref.h"))
    main = os.path.join(CSRC, MAIN)
    if force or _stale(EXE, [main, LIB] + headers):
        # the drop-in program: host code only, linked against the library
        subprocess.run(gxx + [main, "-o", EXE] + link, check=True)
    ref = os.path.join(CSRC, REF_API)
    if force or _stale(REF_LIB, [ref, LIB] + headers):
        # the reference's C++ host functions over the C-ABI
        subprocess.run(gxx + ["-shared", "-fPIC", ref, "-o", REF_LIB] + link, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
