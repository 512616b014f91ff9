"""GPU: the learned start for a sequence of load cases (sgld_cases_*, the
protocol of the ~250M-DOF stress analysis: train on solves of perturbed load
cases, then start held-out cases from what was learned).

* Every start converges to the same answer: held-out cases solved from the
  basis start and from the network's start agree with the oracle's FP64 solve
  to 1e-10 within 1e-6 in compliance and 1e-5 in displacement (relative L2),
  and meet 1e-6 on the true residual.
* The basis start is the energy-optimal combination of the training
  solutions: a training load solved again starts at its own solution (below
  1e-3 of the zero start in sqrt(r'Mr), one outer iteration at most), and
  held-out cases need fewer inner iterations than from zero.
* The network trains (each case's Adam steps lower the loss on its own
  sample) and is judged against the basis start
  alone: a correction is kept only when it lowers r'Mr, so a kept correction
  always starts closer (start_ratio < basis_ratio); the test prints the inner
  iterations of the three starts, which is what the network gains or loses.
"""
import numpy as np
import pytest

from oracle import glue as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model(built_lib):
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import domains as D

    vox = D.gaussian_blobs(64, 32, 32, seed=1, n_blobs=24, fill=0.35)
    s = VoxelSolver(vox, num_levels=4, non_dyadic=0, omega=0.6, pad=False)
    nodes = s.nodMapBack(1)
    fixed = D.fix_bottom_layers(vox, nodes, layers=2)
    s.set_fixed_dofs(fixed)
    s.set_modulus(np.ones(s.numElements))
    s.Solving_AssembleFEAstencil()
    Ftr = D.perturbed_patch_loads(vox, nodes, 8, seed=1, radius=4.0, shift=4.0, exclude_below=2)
    Fho = D.perturbed_patch_loads(vox, nodes, 3, seed=2, radius=4.0, shift=4.0, exclude_below=2)
    m = G.build_model_fixed(vox, fixed, non_dyadic=0, omega=0.6, num_levels=4)
    G.set_modulus(m, np.ones(s.numElements))
    G.assemble_stencil(m)
    yield s, m, Ftr, Fho
    s.close()


def _check_against_oracle(m, F, U, info):
    m.F = F
    U_o, _ = G.solve(m, tol=1e-10, maxIT=5000)
    c_o = G.compliance(m, U_o)
    assert info["converged"] and info["true_relres"] <= 1e-6, info
    assert abs(F @ U - c_o) <= 1e-6 * abs(c_o)
    assert np.linalg.norm(U - U_o) <= 1e-5 * np.linalg.norm(U_o)


def test_basis_start(model):
    from sgldbench_gb300 import LoadCases

    s, m, Ftr, Fho = model
    lc = LoadCases(s, max_basis=8, net_level=-1)
    for F in Ftr:
        lc.solve(F, mode="basis", train=True)
    assert lc.basis_size == 8
    # a training load starts at its own solution (to its solve's tolerance)
    _, iz, _ = lc.solve(Ftr[3], mode="zero")
    _, info, st = lc.solve(Ftr[3], mode="basis", diagnostics=True)
    assert st["basis"] == 8 and st["basis_ratio"] < 1e-3, (info, st)
    assert info["its"] <= 1 and info["inner_its"] < iz["inner_its"], (iz, info)
    for F in Fho:
        U0, i0, _ = lc.solve(F, mode="zero")
        U1, i1, st1 = lc.solve(F, mode="basis", diagnostics=True)
        assert st1["basis_ratio"] < 1.0
        assert i1["inner_its"] < i0["inner_its"], (i0, i1, st1)
        _check_against_oracle(m, F, U1, i1)
    lc.close()


def test_network_start(model):
    from sgldbench_gb300 import LoadCases

    s, m, Ftr, Fho = model
    lc = LoadCases(s, max_basis=8, net_level=0, train_steps=30)
    losses = []
    for F in Ftr:
        _, _, st = lc.solve(F, mode="learned", train=True)
        losses.append((st["net_loss_before"], st["net_loss"]))
    assert lc.basis_size == 8
    # each case's training lowers the loss on its own sample
    assert sum(a > b for a, b in losses) >= 0.75 * len(losses), losses
    assert sum(b for _, b in losses) < sum(a for a, _ in losses), losses
    rows = []
    for F in Fho:
        _, ib, stb = lc.solve(F, mode="basis", diagnostics=True)
        U, il, stl = lc.solve(F, mode="learned", diagnostics=True)
        assert stl["net_used"] == 1
        if stl["net_accepted"]:
            assert stl["start_ratio"] < stl["basis_ratio"]
        else:
            assert stl["start_ratio"] == stl["basis_ratio"]
        _check_against_oracle(m, F, U, il)
        rows.append((ib["inner_its"], il["inner_its"], stl["net_accepted"], stl["net_ratio"]))
    print("held-out inner iterations (basis start, basis + network start, kept, r'Mr ratio):", rows)
    lc.close()
