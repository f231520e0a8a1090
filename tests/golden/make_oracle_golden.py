"""Generate tests/golden/oracle_small.json: the FP32 oracle on the 64x256
workload (20 particles per cell per species, seed 0) after set-up and after
steps 1 and 10, as SHA-256 digests of the exact arrays plus the per-step
counters.  The GPU must reproduce the digests bit for bit
(tests/test_gpu_parity.py), and the oracle must keep reproducing them
(tests/test_oracle_golden.py).  Run from the repository root:
    python tests/golden/make_oracle_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden", "oracle_small.json")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def snapshot(particles, row_counts, rho_fixed, phi, ex, ey):
    """Digests of one state; particles as float32 (the device layout), mesh
    arrays as int64 / float32 node arrays."""
    out = {}
    for sp in (0, 1):
        p = np.asarray(particles(sp), dtype=np.float64).astype(np.float32)
        out[f"particles{sp}"] = digest(p)
        out[f"rows{sp}"] = digest(np.asarray(row_counts(sp), dtype=np.int32))
        out[f"first{sp}"] = [float(v) for v in p[:4].ravel()]
    out["rho_fixed"] = digest(np.asarray(rho_fixed(), dtype=np.int64))
    out["phi"] = digest(np.asarray(phi(), dtype=np.float64).astype(np.float32))
    out["ex"] = digest(np.asarray(ex, dtype=np.float64).astype(np.float32))
    out["ey"] = digest(np.asarray(ey, dtype=np.float64).astype(np.float32))
    return out


def oracle_run():
    import cupic_gb300 as cg
    from oracle.oracle import Oracle
    o = Oracle(cg.workload_params("small"), fp64=False)
    o.init_plasma()
    res = {"workload": "small (64x256, 20 ppc, seed 0)", "states": {}, "stats": []}

    def snap(tag):
        ex, ey = o.efield()
        res["states"][tag] = snapshot(o.particles, o.row_counts, o.rho_fixed, o.phi, ex, ey)

    snap("init")
    for k in range(1, 11):
        o.step(1)
        st = o.stats()
        res["stats"].append({key: st[key] for key in ("step", "absorbed", "removed", "injected",
                                                       "live", "sweeps")})
        if k in (1, 10):
            snap(f"step{k}")
    return res


if __name__ == "__main__":
    with open(GOLDEN, "w") as f:
        json.dump(oracle_run(), f, indent=1)
    print(f"wrote {GOLDEN}")
