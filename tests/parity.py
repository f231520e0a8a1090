"""Comparison helpers shared by the GPU-vs-oracle parity tests.

The kernels round every float operation where the FP32 oracle does, so the
results are expected to be identical; the contract they are held to is
  bit-exact : row (bin) indices, absorbed/removed/injected counts, order
  <= 1e-5   : relative error of rho, phi, E, x, y, vx, vy (FP32)
Relative errors are normwise: max |got - ref| / max |ref| over the array.
"""
import numpy as np

RTOL = 1e-5  # contract tolerance for FP32 quantities


def rel_err(g, o):
    g = np.asarray(g, dtype=np.float64)
    o = np.asarray(o, dtype=np.float64)
    scale = max(np.abs(o).max(), 1e-30) if o.size else 1.0
    return float(np.abs(g - o).max() / scale) if g.size else 0.0


def check_fp32(g, o, what):
    assert g.shape == o.shape, f"{what}: shape {g.shape} vs {o.shape}"
    err = rel_err(g, o)
    assert err <= RTOL, f"{what}: relative error {err:.3e} > {RTOL}"
    return err


def check_stats(g, o, keys=("step", "absorbed", "removed", "injected", "live", "sweeps")):
    for k in keys:
        assert g[k] == o[k], f"{k}: gpu {g[k]} oracle {o[k]} at step {o['step']}"


def check_state(sim, ora, exact=True):
    """Row counts, particles (order included), fixed-point charge, phi and E
    of a GPU context against an FP32 oracle instance."""
    for sp in (0, 1):
        rg, ro = sim.row_counts(sp), ora.row_counts(sp)
        np.testing.assert_array_equal(rg, ro, err_msg=f"row counts of species {sp}")
        g, o = sim.particles(sp), ora.particles(sp)
        check_fp32(g, o, f"particles of species {sp}")
        if exact:
            np.testing.assert_array_equal(g, o, err_msg=f"particles of species {sp} (bitwise)")
        del g, o
    np.testing.assert_array_equal(sim.rho_fixed(0), ora.rho_fixed(), err_msg="fixed-point charge")
    check_fp32(sim.phi(), ora.phi(), "phi")
    exg, eyg = sim.efield()
    exo, eyo = ora.efield()
    check_fp32(exg, exo, "Ex")
    check_fp32(eyg, eyo, "Ey")
    if exact:
        np.testing.assert_array_equal(sim.phi().astype(np.float64), ora.phi(), err_msg="phi bitwise")
        np.testing.assert_array_equal(exg.astype(np.float64), exo, err_msg="Ex bitwise")
        np.testing.assert_array_equal(eyg.astype(np.float64), eyo, err_msg="Ey bitwise")


def split_rows(parts, counts):
    ends = np.cumsum(np.asarray(counts, dtype=np.int64))
    return np.split(parts, ends[:-1])


def pair_rows(g, g_counts, o, o_counts, rows=None, close=1e-4, most_lost=4):
    """Pairs up the particles of two runs of the same push whose values
    differ only by rounding.  Both arrays are in row order (the counts say
    how many each row holds).  A particle within rounding of a row boundary
    can be binned one row up or down in the other run, which also shifts
    the order, so every particle of row r of `o` is paired with its nearest
    neighbour in (x, y, vx, vy), scaled by each column's largest value,
    among rows r-1..r+1 of `g`.  rows: the rows of `o` to pair (all by
    default).  A particle with no counterpart within `close` -- one within
    rounding of y = 0 or y = Ly that left the domain in one run only -- is
    dropped; at most `most_lost` may be.  Returns the paired arrays."""
    from scipy.spatial import cKDTree
    scale = np.maximum(np.abs(o).max(axis=0), 1e-30)
    gr, orow = split_rows(g, g_counts), split_rows(o, o_counts)
    ncy = len(orow)
    rows = range(ncy) if rows is None else rows
    G, O, lost = [], [], 0
    for r in rows:
        if not len(orow[r]):
            continue
        cand = np.concatenate([gr[k] for k in (r - 1, r, r + 1) if 0 <= k < ncy])
        d, idx = cKDTree(cand / scale).query(orow[r] / scale)
        keep = d <= close
        lost += int((~keep).sum())
        idx = idx[keep]
        assert len(np.unique(idx)) == len(idx), f"row {r}: pairing is not one to one"
        G.append(cand[idx])
        O.append(orow[r][keep])
    assert lost <= most_lost, f"{lost} particles without a counterpart"
    return np.concatenate(G), np.concatenate(O)
