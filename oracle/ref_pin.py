"""Build and run the reference's own input_data getters (src/init.cu:424-789)
and, in a second program, its particle-file reader and snapshot writers
(src/init.cu:348-420, src/diagnostic.cu:48-215); and compile the device
code of its mesh and particle kernels (src/mesh.cu, src/particles.cu) into
cubins that oracle/ref_kernels.py runs on a GPU.

TEST INFRASTRUCTURE ONLY.  The reference's sources are compiled where they
lie (REF_SRC below) with nvcc into oracle/_ref/ -- never copied -- together with:
- a project-written GSL API shim (ref_pin/gsl*, written from the math);
- a forced include that renames mesh.cu's own double atomicAdd, which sm_60+
  already defines (defect D1);
- a harness (ref_pin/pin_main.cpp) that calls the getters and prints every
  derived parameter as exact hex doubles.
The getters and file programs need no GPU: only host functions run.
"""
import json
import os
import shutil
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
PIN = os.path.join(HERE, "ref_pin")
OUT = os.path.join(HERE, "_ref")
BIN = os.path.join(OUT, "ref_pin")
# where the reference's sources lie; this recipe is the one place that names
# it, and CUPIC_REFERENCE_SRC overrides it
REF_SRC = os.environ.get("CUPIC_REFERENCE_SRC", "/root/reference/src")
UNITS = ["init", "cc", "particles", "diagnostic", "cuda", "mesh"]


def available():
    return os.path.isdir(REF_SRC) and shutil.which("nvcc") is not None


def build(force=False):
    """Compile oracle/_ref/ref_pin when the reference sources are present."""
    if not available():
        return None
    if os.path.exists(BIN) and not force:
        return BIN
    obj = os.path.join(OUT, "obj")
    os.makedirs(obj, exist_ok=True)
    flags = ["-gencode", "arch=compute_103a,code=sm_103a", "-dc", "-I", PIN, "-w"]
    procs = []
    for u in UNITS:
        extra = ["-include", os.path.join(PIN, "d1_guard.h")] if u == "mesh" else []
        procs.append(subprocess.Popen(["nvcc"] + flags + extra +
                                      [os.path.join(REF_SRC, u + ".cu"), "-o", os.path.join(obj, u + ".o")]))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("nvcc failed on a reference source")
    subprocess.run(["g++", "-O0", "-c", os.path.join(PIN, "gsl_shim.cpp"), "-I", PIN, "-o",
                    os.path.join(obj, "gsl_shim.o")], check=True)
    subprocess.run(["g++", "-O0", "-c", os.path.join(PIN, "pin_main.cpp"), "-o",
                    os.path.join(obj, "pin_main.o")], check=True)
    objs = [os.path.join(obj, u + ".o") for u in UNITS + ["gsl_shim", "pin_main"]]
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a"] + objs + ["-o", BIN],
                   check=True)
    return BIN


def run(input_text):
    """Derived parameters of one input_data text, from the reference's code."""
    exe = build()
    if exe is None:
        raise RuntimeError("reference sources not available")
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "input"))
        os.makedirs(os.path.join(d, "run"))
        with open(os.path.join(d, "input", "input_data"), "w") as f:
            f.write(input_text)
        out = subprocess.run([exe, d], capture_output=True, text=True, check=True).stdout
    return json.loads(out)


FILES_BIN = os.path.join(OUT, "ref_files")


def build_files(force=False):
    """Compile oracle/_ref/ref_files: the reference's particle-file reader and
    snapshot writers (init.cu, diagnostic.cu) with their cudaMalloc/cudaMemcpy
    on host memory (ref_pin/host_mem.h), driven by ref_pin/files_main.cpp."""
    if not available():
        return None
    if os.path.exists(FILES_BIN) and not force:
        return FILES_BIN
    build()
    obj = os.path.join(OUT, "obj")
    flags = ["-gencode", "arch=compute_103a,code=sm_103a", "-dc", "-I", PIN, "-w",
             "-include", os.path.join(PIN, "host_mem.h")]
    procs = [subprocess.Popen(["nvcc"] + flags + [os.path.join(REF_SRC, u + ".cu"), "-o",
                                                  os.path.join(obj, u + "_host.o")])
             for u in ("init", "diagnostic")]
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("nvcc failed on a reference source")
    subprocess.run(["g++", "-O0", "-c", os.path.join(PIN, "files_main.cpp"), "-o",
                    os.path.join(obj, "files_main.o")], check=True)
    objs = [os.path.join(obj, n + ".o") for n in
            ("init_host", "diagnostic_host", "cc", "particles", "cuda", "mesh", "gsl_shim",
             "files_main")]
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a"] + objs +
                   ["-o", FILES_BIN], check=True)
    return FILES_BIN


def run_files(workdir):
    """Runs ref_files in workdir (input/ prepared by the caller); the
    reference's files appear in workdir/output."""
    exe = build_files()
    if exe is None:
        raise RuntimeError("reference sources not available")
    os.makedirs(os.path.join(workdir, "run"), exist_ok=True)
    os.makedirs(os.path.join(workdir, "output"), exist_ok=True)
    subprocess.run([exe, workdir], check=True)


# Device code of the reference's kernels, for tests/test_gpu_ref_kernels.py:
# one cubin per source file, sm_103a, compiled with nvcc's default arithmetic
# flags as the reference's own makefile does (src/makefile:6).  A cubin holds
# GPU code only, so it runs on any host architecture through the driver API.
KERNEL_CUBINS = {u: os.path.join(OUT, f"ref_{u}.cubin") for u in ("mesh", "particles")}


def build_kernels(force=False):
    """Compile oracle/_ref/ref_{mesh,particles}.cubin from the reference's
    src/mesh.cu and src/particles.cu where they lie (mesh.cu with the D1
    rename of its own double atomicAdd).  Returns the paths, or None when
    the sources are absent."""
    if not available():
        return None
    if all(os.path.exists(c) for c in KERNEL_CUBINS.values()) and not force:
        return KERNEL_CUBINS
    os.makedirs(OUT, exist_ok=True)
    procs = []
    for u, out in KERNEL_CUBINS.items():
        extra = ["-include", os.path.join(PIN, "d1_guard.h")] if u == "mesh" else []
        procs.append(subprocess.Popen(["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
                                       "-I", PIN, "-w"] + extra +
                                      [os.path.join(REF_SRC, u + ".cu"), "-o", out]))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("nvcc failed on a reference source")
    return KERNEL_CUBINS
