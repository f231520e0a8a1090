"""Parity at the benchmarked shape: the 512x2048-cell workload with 100
particles per cell per species (2.1e8 particles), 200 fixed Jacobi sweeps
per step, seed 1 -- the configuration bench.py times.

Its rows are 512 cells wide (513-node field rows in the push's shared
memory), the solve takes the tuned many-CTA layout with temporal blocking,
and each push unit streams about 51,000 particles.  The GPU must give the
FP32 oracle's bits for the particles (order included), row counts, charge,
potential, field and every per-step counter after set-up and after two
steps.  The reference path it stands for is particles.cu:110-231,
mesh.cu:162-472 and cc.cu:73-296 of AntonioTejero/cupic.
"""
import pytest

import cupic_gb300 as cg
from oracle.oracle import Oracle
from parity import check_state, check_stats

pytestmark = pytest.mark.gpu


def test_large_workload_matches_oracle(gpu_lib):
    p = cg.workload_params("large")
    ora = Oracle(p, fp64=False)
    with cg.Sim(p) as sim:
        plan = sim.solver_plan()
        assert plan[0] > 1, f"expected a many-CTA solve, got {plan}"
        sim.init_plasma()
        ora.init_plasma()
        check_state(sim, ora)
        for _ in range(2):
            sim.step(1)
            ora.step(1)
            g = sim.stats(1)[0]
            check_stats(g, ora.stats())
            assert g["flags"] == 0
        check_state(sim, ora)
    ora.close()
