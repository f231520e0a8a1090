"""The reference's text files, pinned to the reference's own code.

tests/golden/ref_files.json holds the files that the reference's writers
(src/diagnostic.cu:48-215) and its particle reader (src/init.cu:348-420)
produced for a small seeded case, compiled from its sources by
oracle/ref_pin.py (tests/golden/make_ref_files.py).  The library's writers
must reproduce them byte for byte, and its reader must return the written
values bit for bit.  No GPU is needed.
"""
import json
import os

import numpy as np
import pytest

import cupic_gb300 as cg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_files.json")


@pytest.fixture(scope="module")
def gold():
    from cupic_gb300 import build
    build.build()
    with open(GOLDEN) as f:
        g = json.load(f)
    g["p"] = np.array([[float.fromhex(v) for v in r] for r in g["particles"]])
    g["m"] = np.array([float.fromhex(v) for v in g["mesh"]]).reshape(g["ncy"] + 1, g["ncx"] + 1)
    return g


def bookmarks(p, ncy, ds):
    """[first, last] index per row of row-sorted particles, -1 when empty."""
    bm = np.full(2 * ncy, -1, dtype=np.int32)
    rows = (p[:, 1] / ds).astype(int)
    for r in range(ncy):
        idx = np.nonzero(rows == r)[0]
        if idx.size:
            bm[2 * r], bm[2 * r + 1] = idx[0], idx[-1]
    return bm


def test_particle_snapshot_matches_reference(gold, tmp_path):
    path = tmp_path / "p.dat"
    cg.write_particles_file(path, gold["p"])
    assert path.read_text() == gold["files"]["particles_snap.dat"]


def test_mesh_snapshot_matches_reference(gold, tmp_path):
    path = tmp_path / "m.dat"
    cg.write_mesh_file(path, gold["m"])
    assert path.read_text() == gold["files"]["mesh.dat"]


def test_bookmarks_and_bins_match_reference(gold, tmp_path):
    bm = bookmarks(gold["p"], gold["ncy"], gold["ds"])
    cg.write_bookmarks_file(tmp_path / "bm.dat", bm)
    assert (tmp_path / "bm.dat").read_text() == gold["files"]["bm.dat"]
    cg.write_bins_file(tmp_path / "bins.dat", gold["p"], gold["ds"])
    assert (tmp_path / "bins.dat").read_text() == gold["files"]["bins.dat"]


def test_reader_round_trips_bit_for_bit(gold, tmp_path):
    path = tmp_path / "p.dat"
    cg.write_particles_file(path, gold["p"], header=gold["header"])
    got = cg.read_particles_file(path)
    assert got.shape == gold["p"].shape
    assert got.view(np.int64).tolist() == gold["p"].view(np.int64).tolist()  # -0.0 included


def test_header_line_is_what_the_reference_reader_skips(gold, tmp_path):
    """With a header line the reference's loader keeps every particle: its
    snapshot of the headered input is the whole input."""
    path = tmp_path / "p.dat"
    cg.write_particles_file(path, gold["p"], header=gold["header"])
    lines = path.read_text().splitlines(keepends=True)
    assert lines[0] == "# " + gold["header"] + "\n"
    assert "".join(lines[1:]) == gold["files"]["particles_snap.dat"]


def test_headerless_file_keeps_first_particle(gold, tmp_path):
    """Defect D12: the reference's loader takes line 1 of a header-less
    snapshot for a header and loses that particle; this reader keeps it."""
    ref = gold["files"]["noheader_snap.dat"].splitlines(keepends=True)
    assert len(ref) == len(gold["p"]) - 1
    assert "".join(ref) == "".join(gold["files"]["particles_snap.dat"].splitlines(keepends=True)[1:])
    path = tmp_path / "p.dat"
    cg.write_particles_file(path, gold["p"])
    got = cg.read_particles_file(path)
    assert got.view(np.int64).tolist() == gold["p"].view(np.int64).tolist()


def test_reader_skips_non_particle_lines_and_checks_capacity(tmp_path):
    path = tmp_path / "p.dat"
    path.write_text("# header\n\n 1 2 3 4 \nbad line\n 5 6 7 8\n 9 10 11\n")
    got = cg.read_particles_file(path)
    assert got.tolist() == [[1, 2, 3, 4], [5, 6, 7, 8]]
    import ctypes
    L = cg.load_library()
    out = np.empty((1, 4))
    n = ctypes.c_int64()
    rc = L.cupic_read_particles_file(os.fsencode(path), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     1, ctypes.byref(n))
    assert rc == 5  # CUPIC_ERR_CAPACITY
    assert L.cupic_read_particles_file(os.fsencode(tmp_path / "missing"), None, 0, ctypes.byref(n)) == 4


def test_input_data_rewrite(gold, tmp_path):
    """main.cu:98-113: the header is kept, line 1 becomes n_ini = n_fin, the
    other lines are kept, and the parameters still parse the same."""
    path = tmp_path / "input_data"
    path.write_text(gold["input_data"])
    before = cg.params_from_input_data(path)
    cg.rewrite_input_data(path, 12345)
    old, new = gold["input_data"].splitlines(), path.read_text().splitlines()
    assert new[0] == old[0] and new[1] == "n_ini = 12345;" and new[2:] == old[2:]
    after = cg.params_from_input_data(path)
    assert after.n_ini == 12345
    for f in ("ncx", "ncy", "ds", "dt", "n", "eps0", "phi_p", "mi", "kti", "n_fin", "n_save"):
        assert getattr(after, f) == getattr(before, f), f
    # a last line without a newline is kept
    path.write_text(gold["input_data"].rstrip("\n"))
    cg.rewrite_input_data(path, 7)
    assert path.read_text().splitlines()[-1] == old[-1]
    assert not os.path.exists(str(path) + "_new")


def test_reference_file_pin_regenerates(gold):
    """Where the reference sources are present, its writers still give the
    committed files."""
    import subprocess
    import sys
    from oracle import ref_pin
    if not ref_pin.available():
        pytest.skip("reference sources not present")
    before = open(GOLDEN).read()
    subprocess.run([sys.executable, os.path.join(ROOT, "tests", "golden", "make_ref_files.py")],
                   check=True, capture_output=True)
    assert open(GOLDEN).read() == before
