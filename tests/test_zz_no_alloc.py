"""GPU test of the allocation-free entry point sgld_kbyu_dot_noalloc.

Callers that cannot allocate device memory when they apply the operator (a
loop with a device-memory budget fixed at start-up, a process whose memory
belongs to another allocator) use this variant of the K*u kernel; its
per-CTA scratch is a static device array instead of context memory.  This
test calls it through the C ABI twice in a row (the shared scratch keeps the
previous call's contents) and checks y and u.y against the existing entry
point sgld_kbyu, with the tolerance of the other K*u parity tests (1e-13
relative for y, 1e-12 for the dot product), and that it refuses to run while
the device holds another context's element matrix; that an eager call leaves
the device's free memory unchanged; and that the call captured into a CUDA
graph and replayed with new inputs meets the same references.  It is collected
last so that a run that stops at the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_kbyu_dot_noalloc_matches_kbyu(built_lib):
    import torch

    from sgldbench_gb300 import VoxelSolver, _lib
    from sgldbench_gb300 import domains as D

    rng = np.random.default_rng(5)
    vox = rng.random((16, 32, 16)) < 0.8
    s = VoxelSolver(vox, non_dyadic=0, omega=0.6)
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    nfull = 3 * (s.resY + 1) * (s.resX + 1) * (s.resZ + 1)
    u_full = torch.zeros(nfull, dtype=torch.float64, device=dev)
    y_full = torch.full((nfull,), float("nan"), dtype=torch.float64, device=dev)
    dot = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    # before the moduli are set the call is refused without touching the device
    rc = lib.sgld_kbyu_dot_noalloc(s.ctx, ctypes.c_void_p(u_full.data_ptr()), ctypes.c_void_p(y_full.data_ptr()),
                                   ctypes.c_void_p(dot.data_ptr()), ctypes.c_void_p(s.stream))
    assert rc == _lib.SGLD_OK + 3
    F, fixed = D.cantilever3(s.voxels, s.nodMapBack(1))
    s.set_fixed_dofs(fixed)
    s.set_modulus(rng.uniform(0.1, 1.0, s.numElements))
    nodes = s.nodMapBack(1) - 1
    idx = torch.from_numpy((3 * nodes[:, None] + np.arange(3)[None, :]).reshape(-1)).to(dev)
    for _ in range(2):
        u = rng.standard_normal(s.numDOFs)
        y_ref = s.Solving_KbyU_MatrixFree(u)
        u_full.zero_()
        u_full[idx] = torch.from_numpy(u).to(dev)
        y_full.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = lib.sgld_kbyu_dot_noalloc(s.ctx, ctypes.c_void_p(u_full.data_ptr()), ctypes.c_void_p(y_full.data_ptr()),
                                       ctypes.c_void_p(dot.data_ptr()), ctypes.c_void_p(s.stream))
        assert rc == _lib.SGLD_OK, lib.sgld_last_error(s.ctx)
        torch.cuda.synchronize()
        y = y_full[idx].cpu().numpy()
        assert _rel(y, y_ref) <= 1e-13
        assert not torch.isnan(y_full).any()     # inactive nodes are written too (zeros)
        d_ref = float(u @ y_ref)
        assert abs(dot.item() - d_ref) <= 1e-12 * abs(d_ref)
    # another material's context takes the device's constant-memory element
    # matrix; the allocation-free call uploads nothing, so it refuses until a
    # regular call on its own context binds the matrix again
    other = VoxelSolver(vox, non_dyadic=0, omega=0.6, poisson_ratio=0.45)
    other.set_fixed_dofs(fixed)
    other.set_modulus(np.ones(other.numElements))
    other.Solving_KbyU_MatrixFree(np.ones(other.numDOFs))

    def call():
        return lib.sgld_kbyu_dot_noalloc(s.ctx, ctypes.c_void_p(u_full.data_ptr()),
                                         ctypes.c_void_p(y_full.data_ptr()), ctypes.c_void_p(dot.data_ptr()),
                                         ctypes.c_void_p(s.stream))

    assert call() == _lib.SGLD_OK + 3
    y_ref = s.Solving_KbyU_MatrixFree(u)
    assert call() == _lib.SGLD_OK, lib.sgld_last_error(s.ctx)
    torch.cuda.synchronize()
    assert _rel(y_full[idx].cpu().numpy(), y_ref) <= 1e-13
    other.close()

    # the eager call takes no device memory; then the use the entry point
    # exists for: the call captured into a CUDA graph and replayed with new
    # inputs (graph instantiation itself may take memory, so that is not checked)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(dev)[0]
    assert call() == _lib.SGLD_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == free0
    side = torch.cuda.Stream(dev)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        rc = lib.sgld_kbyu_dot_noalloc(s.ctx, ctypes.c_void_p(u_full.data_ptr()), ctypes.c_void_p(y_full.data_ptr()),
                                       ctypes.c_void_p(dot.data_ptr()), ctypes.c_void_p(side.cuda_stream))
    assert rc == _lib.SGLD_OK, lib.sgld_last_error(s.ctx)
    for _ in range(2):
        u = rng.standard_normal(s.numDOFs)
        y_ref = s.Solving_KbyU_MatrixFree(u)
        u_full[idx] = torch.from_numpy(u).to(dev)
        y_full.fill_(float("nan"))
        dot.fill_(float("nan"))
        torch.cuda.synchronize()
        graph.replay()
        torch.cuda.synchronize()
        assert _rel(y_full[idx].cpu().numpy(), y_ref) <= 1e-13
        d_ref = float(u @ y_ref)
        assert abs(dot.item() - d_ref) <= 1e-12 * abs(d_ref)
    del graph
    s.close()
