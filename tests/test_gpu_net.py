"""GPU: the learned warm start's U-Net (forward, gradients, Adam) against the
oracle restatement (oracle/net.py, itself pinned to finite differences on
the CPU).

The oracle reproduces the device's rounding points (BF16 activations and
weights, BF16-rounded gradient operands) in float64, so the two differ only
by FP32 accumulation order and the rare BF16 rounding flip that it causes.
Tolerances: output and gradient relative L2 error <= 2e-2 (one BF16 ulp is
2^-8 = 3.9e-3); loss within 1e-2 relative; parameters after one Adam step
within 1e-5 of the learning rate per entry where the gradient is not tiny.
"""
import numpy as np
import pytest

from oracle.net import UNet as OracleNet
from oracle.net import adam_step

pytestmark = pytest.mark.gpu


def _rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, float) - b) / max(np.linalg.norm(b), 1e-300))


CASES = [((9, 7, 6), 8, 3, 3, [8, 16, 16]), ((13, 9, 8), 8, 3, 4, [16, 32, 48, 64]), ((6, 5, 5), 4, 3, 1, [8])]


@pytest.fixture(params=CASES, ids=["L3", "L4_default_widths", "L1"])
def case(request, built_lib):
    from sgldbench_gb300.net import UNet

    dims, cin, cout, L, w = request.param
    net = UNet(dims, cin, cout, L, w, seed=7)
    orc = OracleNet(dims, cin, cout, L, w, emulate=True)
    yield net, orc, dims, cin, cout
    net.close()


def _inputs(dims, cin, cout, seed):
    rng = np.random.default_rng(seed)
    V = int(np.prod(dims))
    x = rng.standard_normal((V, cin)).astype(np.float32)
    t = rng.standard_normal((V, cout)).astype(np.float32)
    m = (rng.random(V) > 0.25).astype(np.float32)
    return x, t, m


def test_param_count_and_layout(case):
    net, orc, *_ = case
    assert net.num_params == orc.nparam
    p = net.get_params()
    # biases start at zero, weights are He-uniform
    for ci, co, taps, _, wo, bo in orc.conv:
        assert np.all(p[bo:bo + co] == 0)
        assert np.abs(p[wo:bo]).max() <= np.sqrt(6.0 / (taps * ci)) * 1.0001


def test_forward_matches_oracle(case):
    net, orc, dims, cin, cout = case
    x, _, _ = _inputs(dims, cin, cout, 1)
    p = net.get_params()
    p[orc.conv[-1][4]:] *= 10.0   # a head of ordinary size
    net.set_params(p)
    y = net.forward(x)
    y_ref, _ = orc.forward(p.astype(np.float64), x)
    assert y.shape == y_ref.shape
    assert _rel_l2(y, y_ref) <= 2e-2


def test_gradient_matches_oracle(case):
    net, orc, dims, cin, cout = case
    x, t, m = _inputs(dims, cin, cout, 2)
    p = net.get_params()
    p[orc.conv[-1][4]:] *= 10.0
    net.set_params(p)
    loss, g = net.grad(x, t, m)
    loss_ref, g_ref, _ = orc.value_and_grad(p.astype(np.float64), x, t, m)
    assert abs(loss - loss_ref) <= 1e-2 * loss_ref
    assert _rel_l2(g, g_ref) <= 2e-2
    # per convolution, so that no layer hides behind a large neighbour
    for ci, co, taps, _, wo, bo in orc.conv:
        assert _rel_l2(g[wo:bo + co], g_ref[wo:bo + co]) <= 5e-2


def test_adam_step_matches_oracle(case):
    net, orc, dims, cin, cout = case
    x, t, m = _inputs(dims, cin, cout, 3)
    p0 = net.get_params().astype(np.float64)
    net.set_params(p0)
    _, g = net.grad(x, t, m)
    lr = 1e-3
    net.set_params(p0)
    net.train_step(x, t, m, lr=lr)
    p1 = net.get_params().astype(np.float64)
    w_ref, _, _ = adam_step(p0, np.zeros_like(p0), np.zeros_like(p0), g.astype(np.float64), 1, lr)
    big = np.abs(g) > 1e-3 * np.abs(g).max()
    # first step of Adam moves each parameter by lr * sign(g) (up to eps)
    assert np.abs(p1 - w_ref)[big].max() <= 1e-5 * lr + 1e-6 * np.abs(p0[big]).max()


def test_training_reduces_loss(built_lib):
    """A few hundred Adam steps fit a smooth target field (the network can learn)."""
    from sgldbench_gb300.net import UNet

    dims = (17, 9, 9)
    V = int(np.prod(dims))
    yy, xx, zz = np.meshgrid(np.arange(dims[0]), np.arange(dims[1]), np.arange(dims[2]), indexing="ij")
    coords = np.stack([a.transpose(2, 1, 0).ravel() for a in (yy, xx, zz)], axis=1) / 8.0
    x = np.concatenate([coords, np.ones((V, 1)), np.zeros((V, 4))], axis=1).astype(np.float32)
    t = np.stack([np.sin(coords[:, 0]), np.cos(coords[:, 1]), coords[:, 2] ** 2], axis=1).astype(np.float32)
    net = UNet(dims, 8, 3, 3, [16, 16, 16], seed=1)
    first = net.train_step(x, t, lr=3e-3)
    for _ in range(300):
        last = net.train_step(x, t, lr=3e-3)
    net.close()
    assert last < 0.05 * first


def test_learned_warm_start_in_simp_loop(built_lib):
    """SIMP loop with the reference's warm start (the previous displacement),
    with the previous change as an extra search direction, and with the
    network's correction added to that subspace.  The solves run to the same
    tolerance, so the designs agree to that tolerance; the starts change only
    the iteration counts, which the test reports.  Every accepted start lowered
    the preconditioned residual norm (the acceptance rule), and neither
    variant may cost iterations."""
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import domains as D

    nx, ny, nz = 64, 32, 32
    vox = D.cuboid(nx, ny, nz)
    s = VoxelSolver(vox, num_levels=4, non_dyadic=0, omega=0.6, pad=False)
    F, fixed = D.cantilever3(vox, s.nodMapBack(1))
    s.set_fixed_dofs(fixed)
    kw = dict(volfrac=0.3, rMin=1.5, nLoop=30, tol=1e-6, maxIT=500, precision="mixed_df")
    runs = {mode: s.TopOpti_GlobalVolumeConstraint(F, learned=mode, net_level=3, **kw)[1] for mode in (0, 2, 1)}
    s.close()
    n = min(len(h) for h in runs.values())
    inner = {mode: sum(h["inner_iterations"] for h in hist[:n]) for mode, hist in runs.items()}
    h1 = runs[1]
    print(f"\nwarm starts over {n} SIMP iterations, inner CG iterations: previous displacement {inner[0]}, "
          f"+ previous change {inner[2]}, + network {inner[1]}; network guesses used "
          f"{sum(h['net_used'] for h in h1)}, starts accepted {sum(h['net_accepted'] for h in h1)}, "
          f"network device time {sum(h['t_net'] for h in h1):.3f} s")
    assert sum(h["net_used"] for h in h1) >= n - 3
    for hist in (runs[1], runs[2]):
        for h in hist:
            if h["net_accepted"]:
                assert 0.0 < h["net_r0_ratio"] < 1.0
    for mode in (1, 2):
        assert inner[mode] <= 1.02 * inner[0]
        c0, c1 = runs[0][n - 1]["compliance"], runs[mode][n - 1]["compliance"]
        assert abs(c1 - c0) <= 1e-3 * abs(c0)
