"""The 64x256 workload's 1000 steps against the FP64 oracle: the
time-averaged probe current and density profile within 2%.

The workload as configured (Jacobi to max |dphi| < 1e-6, at most 2000
sweeps a step) hits its sweep cap every step; the potential then lags the
plasma and the run goes unstable near step 690, in the GPU and in both
oracles alike.  The reference's own stop rule converges further: max |dphi|
< 1e-4 (main.cu:64) after at least max(nnx, nny) sweeps (mesh.cu:67).  The
precision form states it as an FP64 residual below 4e-4 (a Jacobi sweep
changes a node by a quarter of its residual), checked every 32 sweeps, after
at least 288 sweeps (the multiple of 32 above max(nnx, nny) = 257) and at
most 6016.  With that rule the workload's 1000 steps run bounded; near step
1100 the 6016-sweep cap no longer brings the residual below the tolerance,
and by step 1155 electrons cross two rows a step -- in the FP64 oracle too,
so 2000 steps of this shape are not run (the 2000-step check runs on a
256x64 slab in test_gpu_precision.py).

The GPU runs the precision form: FP32 sweeps on a correction, an FP64
residual and update every 32 sweeps.  The oracle runs all-FP64 Jacobi with
the same stop rule, in the reference's arithmetic.  Both start from the
same seed.  Compared over the last 1000 steps:
- the net charge the probe absorbs per step (ions minus electrons), mean;
- each species' row occupancy sampled every 10 steps, mean (the density
  profile), normwise.
"""
import numpy as np
import pytest

import cupic_gb300 as cg
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

STEPS = 1000
TOL = 0.02


def params():
    return cg.workload_params("small", refine_every=32, tol=4e-4, min_sweeps=288, max_sweeps=6016,
                              check_every=32, init_tol=4e-3, init_min_sweeps=288,
                              init_max_sweeps=20000)


def run_gpu(p):
    cur, dens, sweeps = [], [], []
    with cg.Sim(p) as sim:
        sim.init_plasma()
        for k in range(0, STEPS, 10):
            try:
                sim.step(10)
            except cg.CupicError:
                print("\nstats of the last steps:", *sim.stats(10), sep="\n")
                raise
            for s in sim.stats(10):
                cur.append(p.qe * s["absorbed"][0] + p.qi * s["absorbed"][1])
                sweeps.append(s["sweeps"])
            if k + 10 > STEPS // 2:
                dens.append([sim.row_counts(sp) for sp in (0, 1)])
        flags = sim.flags()
    return np.array(cur), np.mean(np.array(dens, dtype=float), axis=0), np.array(sweeps), flags


def run_oracle(p):
    o = Oracle(p, fp64=True)
    o.init_plasma()
    cur, dens = [], []
    for k in range(STEPS):
        o.step(1)
        s = o.stats()
        cur.append(p.qe * s["absorbed"][0] + p.qi * s["absorbed"][1])
        if k >= STEPS // 2 and (k + 1) % 10 == 0:
            dens.append([o.row_counts(sp) for sp in (0, 1)])
    flags = o.flags()
    o.close()
    return np.array(cur), np.mean(np.array(dens, dtype=float), axis=0), flags


def test_precision_form_1000_steps_against_fp64_oracle(gpu_lib):
    p = params()
    g_cur, g_dens, g_sweeps, g_flags = run_gpu(p)
    o_cur, o_dens, o_flags = run_oracle(p)
    assert g_flags == 0 and o_flags == 0
    half = STEPS // 2
    gi, oi = g_cur[half:].mean(), o_cur[half:].mean()
    err_i = abs(gi - oi) / abs(oi)
    err_n = [float(np.abs(g_dens[sp] - o_dens[sp]).max() / o_dens[sp].max()) for sp in (0, 1)]
    print(f"\nprobe current over steps {half + 1}-{STEPS}: GPU {gi:.4f}, FP64 oracle {oi:.4f} "
          f"({err_i:.2e}); density profile e {err_n[0]:.2e}, i {err_n[1]:.2e}; "
          f"sweeps per step {g_sweeps.mean():.0f} (max {g_sweeps.max()})")
    assert err_i <= TOL
    assert max(err_n) <= TOL
