"""CPU tests of the boundary: the CUDA library builds for sm_103a, loads
without a GPU and exports every entry point that include/sgld_gpu.h declares;
the host-side logic that needs no device agrees with the oracle."""
import ctypes
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sgld_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sgld_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_header(built_lib):
    lib = ctypes.CDLL(built_lib)
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from sgldbench_gb300 import _lib

    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_reference_level_rule_matches_oracle(built_lib):
    from oracle import glue as G
    from sgldbench_gb300 import _lib

    lib = _lib.load(built_lib)
    for shape in [(32, 64, 32), (128, 256, 128), (16, 24, 16), (8, 16, 8), (40, 70, 30)]:
        vox = np.ones(shape, bool)
        _, nlev, _, _ = G.voxel_discretization(vox)
        assert lib.sgld_reference_num_levels(int(vox.sum()), 50000) == nlev
    assert lib.sgld_reference_num_levels(4194304, 5000) == 5


def test_create_without_gpu_fails_cleanly(built_lib):
    """No device here: sgld_create must return an error code, not crash."""
    import torch

    if torch.cuda.is_available():
        return
    from sgldbench_gb300 import VoxelSolver, _lib

    try:
        VoxelSolver(np.ones((8, 16, 8), bool))
    except _lib.SgldError as e:
        assert e.code in (2, 5)
    else:
        raise AssertionError("expected an error without a GPU")


def test_domain_bc_matches_oracle_cantilever():
    from oracle import glue as G
    from sgldbench_gb300 import domains as D

    vox = np.ones((8, 16, 8), bool)
    m = G.build_model(vox, omega=0.6)
    F, fixed = D.cantilever3(vox, m.levels[0].nodMapBack)
    assert np.array_equal(F, m.F)
    assert np.array_equal(fixed, m.levels[0].fixedDOFs)
    rng = np.random.default_rng(2)
    vox = rng.random((16, 24, 16)) < 0.8
    m = G.build_model(vox, omega=0.6)
    padded = G.voxel_discretization(vox)[2]
    F, fixed = D.cantilever3(padded, m.levels[0].nodMapBack, nelx=m.nelx)
    assert np.array_equal(F, m.F)
    assert np.array_equal(fixed, m.levels[0].fixedDOFs)


def test_create_rejects_device_ordinal_out_of_range(built_lib):
    """The per-device tables hold 64 devices; other ordinals are an argument
    error, reported before any CUDA call (so it needs no GPU)."""
    from sgldbench_gb300 import VoxelSolver, _lib

    for dev in (-1, 64):
        try:
            VoxelSolver(np.ones((8, 16, 8), bool), device=dev)
        except _lib.SgldError as e:
            assert e.code == 1 and "device" in str(e)
        else:
            raise AssertionError(f"device {dev} accepted")
