"""Runs kernels of the reference's own CUDA sources on a GPU.

TEST INFRASTRUCTURE ONLY: tests/test_gpu_ref_kernels.py uses it to pin the
FP64 oracle's hot-path arithmetic to the reference's code.  The product
never imports it.

The kernels come from oracle/_ref/ref_mesh.cubin and ref_particles.cubin,
which oracle/ref_pin.py compiles from the reference's src/mesh.cu and
src/particles.cu where they lie.  They are loaded with the CUDA driver API
(libcuda) into the context torch holds, looked up by their C++ names, and
launched on the legacy default stream, where torch also runs its copies.
Device memory is torch tensors.

Each launcher documents the buffer sizes its launch reads and writes, so
that every index stays inside the tensors it is given.
"""
import ctypes
import os

from oracle.ref_pin import KERNEL_CUBINS

# C++ names of the kernels (Itanium mangling of the reference's signatures)
KERNELS = {
    # mesh.cu:297  jacobi_iteration(dim3, double, double, double*, double*, double*)
    "jacobi_iteration": ("mesh", b"_Z16jacobi_iteration4dim3ddPdS0_S0_"),
    # mesh.cu:385  field_derivation(double, double*, double*, double*)
    "field_derivation": ("mesh", b"_Z16field_derivationdPdS_S_"),
    # particles.cu:110  fast_grid_to_particle(int, int, double, particle*, int*,
    #                                        double*, double*, double*, double*)
    "fast_grid_to_particle": ("particles", b"_Z21fast_grid_to_particleiidP8particlePiPdS2_S2_S2_"),
    # particles.cu:189  leap_frog_step(double, double, particle*, int*, double*, double*)
    "leap_frog_step": ("particles", b"_Z14leap_frog_stepddP8particlePiPdS2_"),
}


class Dim3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint), ("y", ctypes.c_uint), ("z", ctypes.c_uint)]


def available():
    return all(os.path.exists(p) for p in KERNEL_CUBINS.values())


class RefKernels:
    def __init__(self):
        import torch
        self.torch = torch
        torch.zeros(1, device="cuda")  # the primary context, current on this thread
        torch.cuda.synchronize()
        cu = ctypes.CDLL("libcuda.so.1")
        self.cu = cu
        ctx = ctypes.c_void_p()
        self._ok(cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self.mods = {}
        for unit, path in KERNEL_CUBINS.items():
            m = ctypes.c_void_p()
            self._ok(cu.cuModuleLoad(ctypes.byref(m), os.fsencode(path)), f"cuModuleLoad {path}")
            self.mods[unit] = m
        self.fn = {}
        for name, (unit, sym) in KERNELS.items():
            f = ctypes.c_void_p()
            self._ok(cu.cuModuleGetFunction(ctypes.byref(f), self.mods[unit], sym), name)
            self.fn[name] = f
        cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 6 + [
            ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]

    @staticmethod
    def _ok(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUDA driver error {rc}")

    def close(self):
        for m in self.mods.values():
            self.cu.cuModuleUnload(m)
        self.mods = {}

    def launch(self, name, grid, block, smem, args):
        """args: ctypes scalars / Dim3 / c_void_p, in the kernel's order."""
        params = (ctypes.c_void_p * len(args))(
            *[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        gx, gy, gz = (tuple(grid) + (1, 1))[:3]
        bx, by, bz = (tuple(block) + (1, 1))[:3]
        self._ok(self.cu.cuLaunchKernel(self.fn[name], gx, gy, gz, bx, by, bz, smem, None,
                                        params, None), f"launch {name}")

    def sync(self):
        self._ok(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    @staticmethod
    def ptr(t):
        return ctypes.c_void_p(t.data_ptr())

    # ---- launchers ----------------------------------------------------------
    def jacobi_window(self, rho_win, phi_win, err, nnx, ds, eps0):
        """One jacobi_iteration block (mesh.cu:297-381) on a window of 6 node
        rows: halo row, the block's 512/nnx = 4 rows (nnx = 128), halo row.
        The launch reads rho_win and phi_win at indices < 6 nnx, writes
        phi_win rows 1..4 and err[0]; both windows hold 6 nnx doubles."""
        by = 512 // nnx
        assert by == 4 and rho_win.numel() >= (by + 2) * nnx and phi_win.numel() >= (by + 2) * nnx
        bd = Dim3(nnx, by, 1)
        smem = (2 * nnx * (by + 1) + by) * 8  # mesh.cu:84
        self.launch("jacobi_iteration", (1,), (nnx, by), smem,
                    [bd, ctypes.c_double(ds), ctypes.c_double(eps0), self.ptr(rho_win),
                     self.ptr(phi_win), self.ptr(err)])

    def field(self, phi, ex, ey, nnx, nny, ds):
        """field_derivation over the whole mesh as field_solver launches it
        (mesh.cu:124-154): blocks (nnx, 512/nnx), (nny-2)/(512/nnx) of them.
        Requires (nny-2) divisible by 512/nnx and 512/nnx > 1; reads phi at
        every node, writes ex and ey at every node (nnx*nny doubles each)."""
        by = 512 // nnx
        assert by > 1 and (nny - 2) % by == 0
        for t in (phi, ex, ey):
            assert t.numel() == nnx * nny
        self.launch("field_derivation", ((nny - 2) // by,), (nnx, by), nnx * (by + 2) * 8,
                    [ctypes.c_double(ds), self.ptr(phi), self.ptr(ex), self.ptr(ey)])

    def gather_row(self, j, q, parts, bm, ex, ey, fx, fy, nnx, ds):
        """fast_grid_to_particle (particles.cu:110-185) for cell row j alone.
        The kernel takes its row for the vertical weight from blockDim.x
        (defect D4); one block of j threads, given the field and bookmarks
        from row j on, makes that the particle's own row.  Needs 2 <= j <=
        1024.  Reads ex, ey at node rows j and j+1 (so j+1 < nny), bm[2j],
        bm[2j+1], and the particles between them; writes fx, fy there."""
        assert 2 <= j <= 1024 and (j + 2) * nnx <= ex.numel() and 2 * j + 1 < bm.numel()
        smem = 2 * 2 * nnx * 8 + 2 * 4  # particles.cu:45
        off = j * nnx * 8
        self.launch("fast_grid_to_particle", (1,), (j,), smem,
                    [ctypes.c_int(nnx), ctypes.c_int(q), ctypes.c_double(ds), self.ptr(parts),
                     ctypes.c_void_p(bm.data_ptr() + 8 * j),
                     ctypes.c_void_p(ex.data_ptr() + off), ctypes.c_void_p(ey.data_ptr() + off),
                     self.ptr(fx), self.ptr(fy)])

    def leap_frog(self, dt, m, parts, bm, fx, fy, ncy):
        """leap_frog_step as particle_mover launches it (particles.cu:60-65):
        ncy blocks of 512 threads; reads bm[0 .. 2 ncy) and, for every row,
        the particles and forces between its bookmarks."""
        assert bm.numel() == 2 * ncy
        self.launch("leap_frog_step", (ncy,), (512,), 0,
                    [ctypes.c_double(dt), ctypes.c_double(m), self.ptr(parts), self.ptr(bm),
                     self.ptr(fx), self.ptr(fy)])
