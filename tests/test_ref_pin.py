"""Pins the oracle (and the product's parser) to the reference's own code.

tests/golden/ref_getters.json holds, for 8 input_data files, every parameter
the reference's own init_* getters derive (src/init.cu:424-789), printed as
exact hex doubles. The getters are compiled from the reference's sources by
oracle/ref_pin.py and the file is made by tests/golden/make_ref_getters.py.
The oracle's restatement and the C-ABI's parser must reproduce them bit for
bit. No GPU is needed.
"""
import json
import math
import os

import pytest

import cupic_gb300 as cg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_getters.json")
PI = 3.1415926535897932  # stdh.h


def cases():
    with open(GOLDEN) as f:
        return json.load(f)


def h(x):
    return float.fromhex(x)


def check(p, ref):
    assert p.n == h(ref["n"]), "n = ne * Dl^3 (init.cu:542-556)"
    assert p.eps0 == h(ref["eps0"]), "epsilon0 (init.cu:612-630)"
    assert p.phi_p == h(ref["phi_p"]), "phi_p (init.cu:523-538)"
    assert p.mi == h(ref["mi"]) and p.kti == h(ref["kti"])
    assert p.me == h(ref["me"]) and p.kte == h(ref["kte"])
    assert p.qe == h(ref["qe"]) and p.qi == h(ref["qi"])
    assert p.ds == h(ref["ds"]) and p.dt == h(ref["dt"])
    assert (p.ncx, p.ncy) == (ref["ncx"], ref["ncy"])
    assert (p.nnx, p.nny) == (ref["nnx"], ref["nny"])
    assert (p.n_ini, p.n_prev, p.n_save, p.n_fin) == (ref["n_ini"], ref["n_prev"], ref["n_save"],
                                                      ref["n_fin"])
    lx, ly = p.ds * p.ncx, p.ds * p.ncy
    assert lx == h(ref["Lx"]) and ly == h(ref["Ly"])
    # init.cu:686-714, as the oracle and the kernels compute them
    assert math.sqrt(2.0 * PI * p.me / p.kte) / (p.n * lx * p.ds) == h(ref["dtin_e"])
    assert math.sqrt(2.0 * PI * p.mi / p.kti) / (p.n * lx * p.ds) == h(ref["dtin_i"])
    # particles per species, int(n*Lx*ds*ds)*ncy in 32-bit int (init.cu:136).
    # The reference's product wraps past 2^31 (defect D16); the library keeps
    # the exact product, whose low 32 bits must match.
    exact = p.ppr * p.ncy
    wrapped = (exact + 2 ** 31) % 2 ** 32 - 2 ** 31
    assert wrapped == ref["N"], "particles per species (init.cu:136)"


@pytest.mark.parametrize("k", range(8))
def test_oracle_parser_matches_reference_getters(oracle_mod, tmp_path, k):
    c = cases()[k]
    path = tmp_path / "input_data"
    path.write_text(c["input_data"])
    check(oracle_mod.params_from_input_data(str(path)), c["reference"])


@pytest.mark.parametrize("k", range(8))
def test_library_parser_matches_reference_getters(tmp_path, k):
    from cupic_gb300 import build
    build.build()
    c = cases()[k]
    path = tmp_path / "input_data"
    path.write_text(c["input_data"])
    check(cg.params_from_input_data(str(path)), c["reference"])


def test_golden_file_regenerates_from_the_reference():
    """Where the reference sources are present, its getters still give the
    committed values."""
    from oracle import ref_pin
    if not ref_pin.available():
        pytest.skip("reference sources not present")
    for c in cases()[:3]:
        assert ref_pin.run(c["input_data"]) == c["reference"]
