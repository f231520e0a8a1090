"""Long runs of a probe-bias instance on the oracle (CPU).

A fixed number of Jacobi sweeps per step does not converge the potential
of these meshes, and the lag lets a global oscillation of the potential
grow until particles cross two rows in a step.  The GPU path stops there
with a device flag.  These runs show the growth on the oracle itself, so
it belongs to the algorithm with that solve, and show that a longer solve
keeps the same instance bounded.
"""
import numpy as np

from cupic_gb300.params import bias_instances
from oracle.oracle import Oracle


def phi_range(sweeps, steps):
    p = bias_instances(32, seed=3, sweeps=sweeps)[2]  # 32x128 cells, phi_p = -4.80
    o = Oracle(p, fp64=False)
    try:
        o.init_plasma()
        o.step(steps)
        phi = o.phi()
        return float(phi.min()), float(phi.max())
    finally:
        o.close()


def test_fixed_200_sweeps_let_the_potential_oscillation_grow():
    lo, hi = phi_range(200, 460)
    assert hi > 20.0, (lo, hi)   # 40.7 Te/e at step 460; the probe holds -4.8


def test_2000_sweeps_keep_the_same_instance_bounded():
    lo, hi = phi_range(2000, 460)
    assert -5.0 < lo and hi < 6.0, (lo, hi)
