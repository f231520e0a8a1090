"""Host-format particle transfers through the C-ABI: a page-locked (mapped)
host array is read in place by the upload kernel, a pageable one is staged
through device scratch; downloads go through the scratch to either kind.
Both paths must give the same bits."""
import ctypes

import numpy as np
import pytest

import cupic_gb300 as cg

pytestmark = pytest.mark.gpu


def pinned(shape, dtype):
    torch = pytest.importorskip("torch")
    tdt = {np.float64: torch.float64, np.float32: torch.float32}[dtype]
    return torch.empty(shape, dtype=tdt, pin_memory=True).numpy()


def test_pinned_and_pageable_transfers_agree(gpu_lib):
    p = cg.workload_params("tiny")
    sims = [cg.Sim(p) for _ in range(3)]
    try:
        src = sims[0]
        src.init_plasma()
        src.step(3)
        for sp in (0, 1):
            ref = src.particles(sp)  # pageable destination: staged copy
            n = ref.shape[0]
            assert n > 0
            # mapped destination, at an offset inside its allocation
            big = pinned((n + 5, 4), np.float64)
            dst = big[3:3 + n]
            got = ctypes.c_int64()
            rc = src.L.cupic_store_particles(src.h, sp, dst.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                             n, ctypes.byref(got))
            assert rc == 0 and got.value == n
            np.testing.assert_array_equal(dst, ref)
            f32 = pinned((n, 4), np.float32)
            rc = src.L.cupic_store_particles_f32(src.h, sp, f32.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                 n, ctypes.byref(got))
            assert rc == 0
            np.testing.assert_array_equal(f32, src.particles(sp, f32=True))
            # the same particles uploaded from a pageable and from a mapped array
            sims[1].load(sp, ref)
            sims[2].load(sp, dst)
        for sp in (0, 1):
            np.testing.assert_array_equal(sims[1].row_counts(sp), sims[2].row_counts(sp))
            np.testing.assert_array_equal(sims[1].particles(sp), sims[2].particles(sp))
            np.testing.assert_array_equal(sims[1].row_counts(sp), src.row_counts(sp))
    finally:
        for s in sims:
            s.close()


def test_repeated_transfers_reuse_scratch(gpu_lib):
    """Uploads and downloads of growing sizes through one context."""
    p = cg.workload_params("tiny")
    sim = cg.Sim(p)
    try:
        sim.init_plasma()
        full = sim.particles(0)
        for frac in (0.25, 1.0, 0.5):
            part = full[: int(len(full) * frac)]
            sim.load(0, part)
            back = sim.particles(0)
            assert back.shape == part.shape
            np.testing.assert_array_equal(np.sort(back, axis=0), np.sort(part.astype(np.float32).astype(np.float64), axis=0))
    finally:
        sim.close()


def test_nowait_init_matches_waiting_init(gpu_lib):
    """init_plasma enqueued without waiting (a server's admission) leaves
    the same state as the waiting call once the context is synchronised."""
    p = cg.workload_params("tiny")
    a, b = cg.Sim(p), cg.Sim(p)
    try:
        a.init_plasma()
        b.init_plasma(wait=False)
        b.sync()
        assert a.get_time() == b.get_time()
        for sp in (0, 1):
            np.testing.assert_array_equal(a.particles(sp), b.particles(sp))
        np.testing.assert_array_equal(a.phi(), b.phi())
        a.step(3)
        b.step(3)
        for sp in (0, 1):
            np.testing.assert_array_equal(a.particles(sp), b.particles(sp))
        assert a.stats(1)[0]["live"] == b.stats(1)[0]["live"]
    finally:
        a.close()
        b.close()


def test_reused_streams_and_pool_give_identical_runs(gpu_lib):
    """Contexts created after others were destroyed reuse their streams and
    pooled memory; every run still gives the same bits."""
    cg.reserve(1 << 28, contexts=4)
    p = cg.workload_params("tiny")
    ref = None
    for k in range(6):
        sim = cg.Sim(p)
        try:
            sim.init_plasma(wait=(k % 2 == 0))
            sim.step(4)
            got = [sim.particles(sp) for sp in (0, 1)] + [sim.phi()]
        finally:
            sim.close()
        if ref is None:
            ref = got
        else:
            for a, b in zip(ref, got):
                np.testing.assert_array_equal(a, b)
