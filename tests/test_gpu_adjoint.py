"""The hand-written SPH adjoint on the GPU against the FP64 CPU adjoint of the oracle and
against central finite differences of the FP64 forward, plus checkpointing exactness and
the torch.autograd harness.

Loss: per instance, the mean over particles of |x_final - target|^2, summed over
instances; targets are the initial positions plus seeded noise.
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from tay_gb300 import workloads as W
from tay_gb300.adjoint import SphRollout, make_function

from parity import normwise

pytestmark = pytest.mark.gpu

STEPS = 40
TANK_MIN = (0.0, 0.0, 0.0)
TANK_MAX = (0.12, 0.07, 0.08)
PARAMS = [(0.05, 20.0), (0.08, 22.0)]
TOL = 1e-3  # relative, gradients


def _instances():
    s = W.sph_dam(6, 6, 5)
    return [(s.points, a, c, TANK_MIN, TANK_MAX) for a, c in PARAMS]


def _targets(roll):
    rng = np.random.default_rng(5)
    x0 = np.concatenate([ps.p[:, :3] for ps, *_ in roll.instances]).astype(np.float64)
    return x0 + 1e-3 * rng.standard_normal(x0.shape)


def _dl_dx(x, target, roll):
    g = np.zeros_like(x, dtype=np.float64)
    for k in range(len(roll.instances)):
        a, b = roll.offsets[k], roll.offsets[k + 1]
        g[a:b] = 2.0 * (x[a:b] - target[a:b]) / (b - a)
    return g


def _ctx64(alpha, c0):
    return O.sph_context(np.float64, alpha=alpha, c0=c0, tank_min=TANK_MIN, tank_max=TANK_MAX)


def _loss64(x0, v0, alpha, c0, target):
    r = O.sph_adjoint_f64(x0, v0, _ctx64(alpha, c0), STEPS)
    return float(np.mean(np.sum((r["x_final"] - target) ** 2, axis=1)))


@pytest.fixture(scope="module")
def gpu_grads(gpu):
    roll = SphRollout(_instances(), STEPS, checkpoint_every=0)
    x, _ = roll.forward()
    target = _targets(roll)
    dx0, dv0, dp = roll.backward(_dl_dx(x, target, roll))
    roll.close()
    return {"x": x, "target": target, "dx0": dx0, "dv0": dv0, "dp": dp}


def test_adjoint_matches_fp64_cpu_adjoint(gpu_grads):
    roll = SphRollout(_instances(), STEPS)
    for k, (ps, alpha, c0, *_) in enumerate(roll.instances):
        a, b = roll.offsets[k], roll.offsets[k + 1]
        x0 = ps.p[:, :3].astype(np.float64)
        v0 = np.zeros_like(x0)
        tgt = gpu_grads["target"][a:b]
        fwd = O.sph_adjoint_f64(x0, v0, _ctx64(alpha, c0), STEPS)
        # FP32 GPU and FP64 CPU trajectories: same positions to well within the tolerance
        assert normwise(gpu_grads["x"][a:b] - x0, fwd["x_final"] - x0) < 1e-3
        g = 2.0 * (fwd["x_final"] - tgt) / (b - a)
        ref = O.sph_adjoint_f64(x0, v0, _ctx64(alpha, c0), STEPS, dl_dx=g)
        dp = gpu_grads["dp"][k]
        assert abs(dp[0] - ref["dalpha"]) <= TOL * abs(ref["dalpha"]), (k, dp[0], ref["dalpha"])
        assert abs(dp[1] - ref["dc0"]) <= TOL * abs(ref["dc0"]), (k, dp[1], ref["dc0"])
        assert normwise(gpu_grads["dx0"][a:b], ref["dx0"]) < TOL
        assert normwise(gpu_grads["dv0"][a:b], ref["dv0"]) < TOL


def test_adjoint_matches_finite_differences(gpu_grads):
    """Central differences of the FP64 forward: alpha with relative eps 1e-3; c0 with
    relative eps 1e-5 (the loss is not smooth in c0 over a 1e-3 step: pairs cross the
    viscosity switch v.x = 0; the eps-1e-3 value is reported, not asserted)."""
    roll = SphRollout(_instances(), STEPS)
    ps, alpha, c0, *_ = roll.instances[0]
    n = ps.n
    x0 = ps.p[:, :3].astype(np.float64)
    v0 = np.zeros_like(x0)
    tgt = gpu_grads["target"][:n]
    ea = 1e-3 * alpha
    fd_a = (_loss64(x0, v0, alpha + ea, c0, tgt) - _loss64(x0, v0, alpha - ea, c0, tgt)) / (2 * ea)
    ec = 1e-5 * c0
    fd_c = (_loss64(x0, v0, alpha, c0 + ec, tgt) - _loss64(x0, v0, alpha, c0 - ec, tgt)) / (2 * ec)
    dp = gpu_grads["dp"][0]
    assert abs(dp[0] - fd_a) <= TOL * abs(fd_a), (dp[0], fd_a)
    assert abs(dp[1] - fd_c) <= TOL * abs(fd_c), (dp[1], fd_c)


@pytest.mark.parametrize("keep", [1, 2])
def test_checkpointing_reproduces_recording(gpu_grads, keep):
    roll = SphRollout(_instances(), STEPS, checkpoint_every=10, keep_segments=keep)
    x, _ = roll.forward()
    assert np.array_equal(x, gpu_grads["x"])
    dx0, dv0, dp = roll.backward(_dl_dx(x, gpu_grads["target"], roll))
    assert np.array_equal(dx0, gpu_grads["dx0"])
    assert np.array_equal(dv0, gpu_grads["dv0"])
    assert np.array_equal(dp, gpu_grads["dp"])
    roll.close()


def test_torch_autograd_harness(gpu_grads):
    torch = pytest.importorskip("torch")
    roll = SphRollout(_instances(), STEPS)
    fn = make_function()
    v0 = torch.zeros((roll.n, 3), dtype=torch.float32, requires_grad=True)
    params = torch.tensor(roll.params, dtype=torch.float64, requires_grad=True)
    x = fn.apply(v0, params, roll)
    target = torch.from_numpy(gpu_grads["target"].astype(np.float32))
    loss = 0
    for k in range(len(roll.instances)):
        a, b = int(roll.offsets[k]), int(roll.offsets[k + 1])
        loss = loss + ((x[a:b] - target[a:b]) ** 2).sum(dim=1).mean()
    loss.backward()
    np.testing.assert_allclose(params.grad.numpy(), gpu_grads["dp"], rtol=1e-4)
    np.testing.assert_allclose(v0.grad.numpy(), gpu_grads["dv0"], rtol=1e-3, atol=1e-9)
    roll.close()


def test_adjoint_row_order(gpu_grads):
    """The adjoint over the row-order cell table: same gradients up to float summation order."""
    from tay_gb300 import api
    try:
        api.set_tuning(cell_order=1)
        roll = SphRollout(_instances(), STEPS, checkpoint_every=10, keep_segments=2)
        x, _ = roll.forward()
        dx0, dv0, dp = roll.backward(_dl_dx(x, gpu_grads["target"], roll))
        roll.close()
    finally:
        api.set_tuning()
    assert normwise(x, gpu_grads["x"]) < 1e-5
    np.testing.assert_allclose(dp, gpu_grads["dp"], rtol=TOL)
    assert normwise(dx0, gpu_grads["dx0"]) < TOL
    assert normwise(dv0, gpu_grads["dv0"]) < TOL


def test_adjoint_pair_lists(gpu_grads):
    """The recorded forward and the backward's recomputed segments replay the density pass's
    pair lists in the force pass, and each backward step's density adjoint replays the force
    adjoint's list.  With the lists off the rollout is the same bits; the gradients agree to
    float rounding (the force adjoint records on the per-lane walk, which may round its
    sums differently from the warp-union walk it takes without lists)."""
    from tay_gb300 import api
    out = []
    for cap in (0, 320):
        try:
            api.set_tuning(pair_list_cap=cap)
            roll = SphRollout(_instances(), STEPS, checkpoint_every=10, keep_segments=2)
            x, _ = roll.forward()
            grads = roll.backward(_dl_dx(x, gpu_grads["target"], roll))
            roll.close()
        finally:
            api.set_tuning()
        out.append((x, grads))
    assert np.array_equal(out[0][0], out[1][0])
    for a, b in zip(out[0][1], out[1][1]):
        assert normwise(a, b) < 1e-6


def test_fit_viscosity_and_sound_speed_to_a_target_rollout(gpu):
    """The adjoint used as intended: two instances starting at (alpha, c0) = (0.05, 20) and
    (0.12, 18) fitted with Adam to a target rollout made with (0.08, 22), 100 steps."""
    from tay_gb300.adjoint import fit_parameters

    tank = (0.16, 0.12, 0.12)
    s = W.sph_dam(10, 10, 8, tank=tank)
    tgt = SphRollout([(s.points, 0.08, 22.0, (0.0, 0.0, 0.0), tank)] * 2, 100)
    target, _ = tgt.forward()
    tgt.close()
    roll = SphRollout([(s.points, 0.05, 20.0, (0.0, 0.0, 0.0), tank), (s.points, 0.12, 18.0, (0.0, 0.0, 0.0), tank)],
                      100, checkpoint_every=20)
    hist = fit_parameters(roll, target, iters=25, lr=0.05)
    roll.close()
    losses = [l for l, _ in hist]
    assert min(losses[-5:]) < 0.1 * losses[0], losses
    assert np.all(np.abs(roll.params[:, 0] - 0.08) < 0.012), roll.params
    assert np.all(np.abs(roll.params[:, 1] - 22.0) < 2.0), roll.params


def test_second_backward_needs_a_forward(gpu_grads):
    """A checkpointed backward that recomputed a segment recorded it over the forward run's
    records: a second backward is refused until the next forward; with every step recorded
    the backward can run again and gives the same gradients."""
    from tay_gb300 import api

    roll = SphRollout(_instances(), STEPS, checkpoint_every=10, keep_segments=1)
    x, _ = roll.forward()
    g = _dl_dx(x, gpu_grads["target"], roll)
    first = roll.backward(g)
    with pytest.raises(api.TayError, match="tgpu_adjoint_forward first"):
        roll.backward(g)
    roll.forward()
    again = roll.backward(g)
    for a, b in zip(first, again):
        assert np.array_equal(a, b)
    roll.close()
    roll = SphRollout(_instances(), STEPS, checkpoint_every=0)
    x, _ = roll.forward()
    first = roll.backward(g)
    again = roll.backward(g)
    for a, b in zip(first, again):
        assert np.array_equal(a, b)
    roll.close()
