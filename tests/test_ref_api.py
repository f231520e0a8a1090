"""The reference-named C++ surface (include/cupic_ref.h, libcupic_ref.so).

libcupic_ref.so must define every function cupic_ref.h declares, under the
reference's own C++ signatures, so that the reference's unchanged
src/main.cu links against it.  Where the reference sources are present, its
main.cu is compiled and linked against the library (no GPU needed).
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "cupic_gb300", "_build")


@pytest.fixture(scope="module")
def ref_lib():
    from cupic_gb300 import build
    build.build()
    return os.path.join(BUILD, "libcupic_ref.so")


def declared():
    text = open(os.path.join(ROOT, "include", "cupic_ref.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"^(?:void|int|double)\s+(\w+)\s*\(", text, flags=re.M))


def test_library_defines_every_declared_function(ref_lib):
    out = subprocess.run(["nm", "-DC", "--defined-only", ref_lib], capture_output=True, text=True,
                         check=True).stdout
    defined = set(re.findall(r" T (\w+)\(", out))
    names = declared()
    assert len(names) == 36
    assert names <= defined, sorted(names - defined)


def test_signatures_are_the_references(ref_lib):
    out = subprocess.run(["nm", "-DC", "--defined-only", ref_lib], capture_output=True, text=True,
                         check=True).stdout
    for sig in ("charge_deposition(double*, particle*, int*, particle*, int*)",
                "poisson_solver(double, double*, double*)",
                "field_solver(double*, double*, double*)",
                "particle_mover(particle*, int*, particle*, int*, double*, double*)",
                "cc(double, int*, particle**, int*, particle**, double*, double*)",
                "init_sim(double**, double**, double**, double**, particle**, particle**, int**, "
                "int**, double*)"):
        assert sig in out, sig


def test_reference_main_links_against_the_library(ref_lib, tmp_path):
    from oracle.ref_pin import REF_SRC
    if not (os.path.isdir(REF_SRC) and shutil.which("nvcc")):
        pytest.skip("reference sources not present")
    obj = tmp_path / "main.o"
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-w", "-c",
                    "-I", os.path.join(ROOT, "oracle", "ref_pin"), os.path.join(REF_SRC, "main.cu"),
                    "-o", str(obj)], check=True)
    exe = tmp_path / "cupic_main"
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", str(obj), "-o", str(exe),
                    "-L", BUILD, "-lcupic_ref", "-lcupic_gpu", f"-Xlinker=-rpath,{BUILD}"],
                   check=True)
    und = subprocess.run(["nm", "-uC", str(obj)], capture_output=True, text=True).stdout
    needed = {m for m in re.findall(r" U (\w+)\(", und) if not m.startswith(("std", "__", "cuda", "operator"))}
    assert needed <= declared(), sorted(needed - declared())
    assert {"charge_deposition", "poisson_solver", "field_solver", "particle_mover", "cc",
            "init_sim"} <= needed
