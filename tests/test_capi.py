"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/cupic_gpu.h declares.  No compute calls: this runs without a GPU."""
import ctypes
import os
import re
import subprocess

import pytest

import cupic_gb300 as cg
from cupic_gb300.params import Params, StepStats

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if not name.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", name)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        syms.update(re.findall(r"\b(cupic_\w+)\s*\(", text))
    return syms


@pytest.fixture(scope="module")
def lib():
    from cupic_gb300 import build
    build.build()
    return cg.load_library()


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in sorted(syms) if not hasattr(lib, s)]
    assert not missing, f"declared but not exported: {missing}"
    assert sorted(syms) == sorted(cg.EXPORTED)


def test_exported_symbols_have_c_linkage(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", cg.library_path()], capture_output=True,
                         text=True, check=True).stdout
    names = {line.split()[-1] for line in out.splitlines() if line.strip()}
    for s in declared_symbols():
        assert s in names, f"{s} missing or mangled"


def test_library_is_built_for_sm_103a(lib):
    out = subprocess.run(["cuobjdump", "--list-elf", cg.library_path()], capture_output=True,
                         text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    assert "sm_103a" in out.stdout


def test_struct_layouts_match_header():
    assert ctypes.sizeof(StepStats) == 8 + 8 + 4 * 16 + 4 + 4 + 4 + 4  # padded to 8
    p = Params()
    assert ctypes.sizeof(p) % 8 == 0


def test_params_default_matches_python_mirror(lib):
    p = Params()
    assert lib.cupic_params_default(ctypes.byref(p)) == 0
    q = cg.workload_params("small")
    for k in ("ncx", "ncy", "ds", "dt", "n", "eps0", "phi_p", "mi", "kti", "ppr", "tol",
              "max_sweeps"):
        assert getattr(p, k) == getattr(q, k), k
    assert p.ppr == 1280


def test_create_without_gpu_fails_cleanly(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    p = cg.workload_params("tiny")
    h = ctypes.c_void_p()
    rc = lib.cupic_create(ctypes.byref(p), 0, ctypes.byref(h))
    assert rc == 10 and not h.value  # CUPIC_ERR_NODEVICE, no exit()
    with pytest.raises(cg.CupicError):
        cg.Sim(p)


def test_invalid_params_rejected_before_device(lib):
    p = cg.workload_params("tiny")
    p.ncx = 1
    h = ctypes.c_void_p()
    assert lib.cupic_create(ctypes.byref(p), 0, ctypes.byref(h)) == 1  # CUPIC_ERR_ARG
    assert lib.cupic_destroy(None) == 1
    assert lib.cupic_step(None, 1) == 1


def test_strerror_names_every_status(lib):
    for s in range(11):
        assert lib.cupic_strerror(s) and lib.cupic_strerror(s) != b"unknown status"


def test_input_data_parser_matches_oracle(lib, tmp_path):
    from oracle import oracle
    path = tmp_path / "input_data"
    path.write_text("#execution configuration\n n_ini = 0;\nn_prev = 0;\nn_save = 100;\n"
                    "n_fin = 200000;\nne = 1.0e14;\nTe = 1.0e3;\nbeta = 1.0e-1;\n"
                    "gamma = 1.0e3;\nphi_p = -5.0e0;\nncx = 127;\nncy = 1021;\nds = 1.0e-1;\n"
                    "dt = 1.0e-3;\n")
    a = cg.params_from_input_data(str(path))
    b = oracle.params_from_input_data(str(path))
    for k, _ in Params._fields_:
        assert getattr(a, k) == getattr(b, k), k
    assert a.ncx == 127 and a.ncy == 1021 and a.mi == 1000.0 and a.kti == 0.1
    assert a.min_sweeps == 1023  # max(nnx, nny) + 1 (mesh.cu:67,94)


def test_missing_input_data_is_an_error(lib, tmp_path):
    with pytest.raises(cg.CupicError) as e:
        cg.params_from_input_data(str(tmp_path / "nope"))
    assert e.value.status == 4
