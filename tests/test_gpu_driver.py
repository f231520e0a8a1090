"""The drop-in program (cupic_run, the reference's main.cu:26-117) and the
restart path, on the GPU.

A run from n_ini = 0 writes the reference's particle files every n_save
steps and rewrites n_ini in input_data; a second run restarts from the last
files (init.cu:84-93, with the loader keeping every particle: defect D12
fixed).  Both runs are held bit-exact against the FP32 oracle driven through
the same sequence, and the graph loop against the stage-by-stage loop.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import cupic_gb300 as cg
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

INPUT = ("#execution configuration\nn_ini = 0;\nn_prev = 0;\nn_save = 10;\nn_fin = 20;\n"
         "ne = 4.2246e15;\nTe = 1.0e3;\nbeta = 1.0;\ngamma = 100.0;\nphi_p = -0.43102;\n"
         "ncx = 16;\nncy = 64;\nds = 0.5;\ndt = 0.05;\n")


def run(tmp, name):
    d = tmp / name
    for sub in ("input", "output/particles", "restart"):
        (d / sub).mkdir(parents=True, exist_ok=True)
    return d


def drive(d, *extra):
    r = subprocess.run([cg.driver_path(), *extra, str(d / "input" / "input_data"), str(d / "output"),
                        str(d / "restart")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout.splitlines()


def snap(d, species, i):
    return cg.read_particles_file(d / "output" / "particles" / f"{species}_t_{i}.dat")


def linear_phi(p):
    j = np.arange(p.nny, dtype=np.float64)[:, None]
    return np.broadcast_to((1.0 - j / p.ncy) * p.phi_p, (p.nny, p.nnx)).copy()


@pytest.fixture(scope="module")
def first_run(tmp_path_factory, gpu_lib):
    tmp = tmp_path_factory.mktemp("driver")
    d = run(tmp, "graph")
    (d / "input" / "input_data").write_text(INPUT)
    out = drive(d)
    return d, out


def test_run_from_initial_condition(first_run):
    d, out = first_run
    assert out[0].startswith("Simulation initialized with ")
    ts = [l for l in out if l.startswith("t = ")]
    assert len(ts) == 21 and ts[0] == "t = 0" and ts[-1] == "t = 1"
    assert out[-1] == "Simulation finished!"
    for i in (0, 10, 20):
        for s in ("electrons", "ions"):
            assert (d / "output" / "particles" / f"{s}_t_{i}.dat").exists()
    lines = (d / "input" / "input_data").read_text().splitlines()
    assert lines[1] == "n_ini = 20;" and lines[2:] == INPUT.splitlines()[2:]


def test_run_matches_oracle(first_run):
    d, _ = first_run
    path = d.parent / "orig_input"
    path.write_text(INPUT)
    p = cg.params_from_input_data(path)
    ora = Oracle(p, fp64=False)
    ora.init_plasma()
    for i in (0, 10, 20):
        if i:
            ora.step(10)
        for sp, s in enumerate(("electrons", "ions")):
            np.testing.assert_array_equal(snap(d, s, i), ora.particles(sp), err_msg=f"{s} t={i}")


def test_stage_loop_matches_graph_loop(first_run, tmp_path):
    d, out = first_run
    e = run(tmp_path, "stages")
    (e / "input" / "input_data").write_text(INPUT)
    out2 = drive(e, "--stages")
    assert out2 == out
    for i in (0, 10, 20):
        for s in ("electrons", "ions"):
            a = (d / "output" / "particles" / f"{s}_t_{i}.dat").read_text()
            b = (e / "output" / "particles" / f"{s}_t_{i}.dat").read_text()
            assert a == b, f"{s} t={i}"


def test_restart_matches_oracle(first_run, tmp_path):
    d, _ = first_run
    r = run(tmp_path, "restart")
    text = (d / "input" / "input_data").read_text().replace("n_fin = 20;", "n_fin = 30;")
    (r / "input" / "input_data").write_text(text)
    (r / "input_at_start").write_text(text)
    for s in ("electrons", "ions"):
        shutil.copy(d / "output" / "particles" / f"{s}_t_20.dat", r / "restart" / f"{s}.dat")
    out = drive(r)
    assert out[0] == "Simulation state loaded from time t = 1"
    ts = [l for l in out if l.startswith("t = ")]
    assert ts[0] == "t = 1" and ts[-1] == "t = 1.5" and len(ts) == 11
    # every particle of the restart files is loaded (D12 fixed)
    for s in ("electrons", "ions"):
        np.testing.assert_array_equal(snap(r, s, 20), snap(d, s, 20))
    p = cg.params_from_input_data(r / "input_at_start")
    assert p.n_ini == 20
    ora = Oracle(p, fp64=False)
    ora.load(0, snap(d, "electrons", 20))
    ora.load(1, snap(d, "ions", 20))
    ora.set_phi(linear_phi(p))
    ora.deposit()
    ora.solve(p.init_tol, p.init_min_sweeps, p.init_max_sweeps, p.check_every)
    ora.field()
    ora.set_time(p.n_ini + 1, p.n_ini * p.dt + p.dt)
    ora.step(10)
    for sp, s in enumerate(("electrons", "ions")):
        np.testing.assert_array_equal(snap(r, s, 30), ora.particles(sp), err_msg=s)
    assert (r / "input" / "input_data").read_text().splitlines()[1] == "n_ini = 30;"


def test_snapshots_from_context(gpu_lib, tmp_path):
    """mesh_snapshot / save_bm / save_bins straight from a context match the
    library's arrays written by the file writers."""
    p = cg.workload_params("tiny")
    with cg.Sim(p) as sim:
        sim.init_plasma()
        sim.step(3)
        for what, arr in (("rho_last", sim.rho(1)), ("phi", sim.phi()), ("ex", sim.efield()[0]),
                          ("ey", sim.efield()[1])):
            sim.mesh_snapshot(what, tmp_path / f"{what}.dat")
            cg.write_mesh_file(tmp_path / f"{what}_ref.dat", np.asarray(arr, dtype=np.float64))
            assert (tmp_path / f"{what}.dat").read_text() == (tmp_path / f"{what}_ref.dat").read_text()
        sim.save_bm(0, tmp_path / "bm.dat")
        cg.write_bookmarks_file(tmp_path / "bm_ref.dat", sim.bookmarks(0))
        assert (tmp_path / "bm.dat").read_text() == (tmp_path / "bm_ref.dat").read_text()
        sim.save_bins(1, tmp_path / "bins.dat")
        cg.write_bins_file(tmp_path / "bins_ref.dat", sim.particles(1), p.ds)
        assert (tmp_path / "bins.dat").read_text() == (tmp_path / "bins_ref.dat").read_text()
        sim.particles_snapshot(0, tmp_path / "e.dat")
        np.testing.assert_array_equal(cg.read_particles_file(tmp_path / "e.dat"), sim.particles(0))


def test_reference_shaped_main_matches_program(first_run, tmp_path):
    """A main in the shape of main.cu, calling the reference-named functions
    of libcupic_ref.so from a bin/ directory with ../input and ../output,
    writes the same particle files as cupic_run."""
    d, out = first_run
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    build = os.path.join(root, "cupic_gb300", "_build")
    exe = tmp_path / "ref_shape_main"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(root, "include"),
                    os.path.join(root, "tests", "ref_shape_main.cpp"), "-o", str(exe), "-L", build,
                    "-lcupic_ref", "-lcupic_gpu", f"-Wl,-rpath,{build}"], check=True)
    w = tmp_path / "case"
    for sub in ("bin", "input", "output/particles"):
        (w / sub).mkdir(parents=True)
    (w / "input" / "input_data").write_text(INPUT)
    r = subprocess.run([str(exe)], cwd=w / "bin", capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == out[0] and [l for l in lines if l.startswith("t = ")] == \
        [l for l in out if l.startswith("t = ")]
    for i in (0, 10, 20):
        for s in ("electrons", "ions"):
            a = (d / "output" / "particles" / f"{s}_t_{i}.dat").read_text()
            b = (w / "output" / "particles" / f"{s}_t_{i}.dat").read_text()
            assert a == b, f"{s} t={i}"
    for i in (10, 20):
        for f in (f"charge_t_{i - 1}.dat", f"potential_t_{i - 1}.dat", f"bm_electrons_t_{i}.dat",
                  f"bins_electrons_t_{i}.dat"):
            assert (w / "output" / f).stat().st_size > 0, f
