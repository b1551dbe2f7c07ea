"""Differentiable SPH rollouts on the GPU: a driver over the engine's adjoint ABI
(tgpu_adjoint_*) and a thin torch.autograd.Function around it.

    roll = SphRollout(instances, steps=200, checkpoint_every=20)
    x_final, v_final = roll.forward()              # [N, 3] float32, instances concatenated
    dx0, dv0, dparams = roll.backward(dL_dx_final)  # dparams: [instances, 2] = dL/d(alpha, c0)

    x_final = SphRolloutFunction.apply(v0, params, roll)   # torch; gradients flow to v0 and
                                                           # params = [instances, 2] (alpha, c0)

    history = fit_parameters(roll, target_x, iters=20)     # (alpha, c0) fitted to a target

`instances` is a list of (PointSet, alpha, c0, tank_min, tank_max); every instance runs the
full SPH pass sequence (density, pressure, force, integrate) as one segment of one batch.
Rows of the per-particle arrays are the particles in instance order, each instance's
particles in their id order.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import api
from . import models as M


class SphRollout:
    def __init__(self, instances, steps: int, checkpoint_every: int = 0, h: float = 0.02, dx: float = 0.01,
                 mb: int = 64, keep_segments: int = 1):
        self.L = api.lib()
        self.steps = steps
        self.every = checkpoint_every
        self.keep = keep_segments
        self.instances = instances
        self.h, self.dx, self.mb = h, dx, mb
        self.counts = [ps.n for ps, *_ in instances]
        self.offsets = np.concatenate([[0], np.cumsum(self.counts)]).astype(np.int64)
        self.n = int(self.offsets[-1])
        self._batch = None
        self._adj = ctypes.c_void_p()
        self.v0 = np.concatenate([ps.v[:, :3] for ps, *_ in instances]).astype(np.float32)
        self.params = np.array([[a, c] for _, a, c, *_ in instances], np.float64)

    def _groups(self, v0, params):
        groups = []
        for k, (ps, _, _, tmin, tmax) in enumerate(self.instances):
            a, c = float(params[k, 0]), float(params[k, 1])
            setup = M.sph_setup(h=self.h, dx=self.dx, alpha=a, c0=c, tank_min=tmin, tank_max=tmax, mb=self.mb)
            v = np.zeros((ps.n, 4), np.float32)
            v[:, :3] = v0[self.offsets[k]:self.offsets[k + 1]]
            groups.append((setup, M.records(M.SPH_RECORD, ps.p, v)))
        return groups

    def close(self):
        if self._adj:
            self.L.tgpu_adjoint_destroy(self._adj)
            self._adj = ctypes.c_void_p()
        if self._batch is not None:
            self._batch.close()
            self._batch = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise api.TayError(f"{what}: {self.L.tgpu_last_error().decode()}")

    def forward(self, v0=None, params=None):
        """Runs the rollout from (v0, params) (defaults: the instances' own); returns the
        final positions and velocities, [N, 3] float32 each."""
        self.close()
        v0 = self.v0 if v0 is None else np.asarray(v0, np.float32)
        params = self.params if params is None else np.asarray(params, np.float64)
        self._batch = api.Batch(self._groups(v0, params))
        self._batch.push()
        self._check(self.L.tgpu_adjoint_create(self._batch.ptr, self.steps, self.every, self.keep,
                                               ctypes.byref(self._adj)),
                    "tgpu_adjoint_create")
        self._check(self.L.tgpu_adjoint_forward(self._adj), "tgpu_adjoint_forward")
        x = np.zeros((self.n, 3), np.float32)
        v = np.zeros((self.n, 3), np.float32)
        for k in range(len(self.instances)):
            rec = M.by_id(self._batch.fetch(k))
            x[self.offsets[k]:self.offsets[k + 1]] = rec["p"][:, :3]
            v[self.offsets[k]:self.offsets[k + 1]] = rec["v"][:, :3]
        return x, v

    def backward(self, dl_dx, dl_dv=None):
        """Gradients of a loss given dL/d(final positions) (and velocities), [N, 3]."""
        gx = np.zeros((self.n, 4), np.float32)
        gx[:, :3] = dl_dx
        gv = np.zeros((self.n, 4), np.float32)
        if dl_dv is not None:
            gv[:, :3] = dl_dv
        dx0 = np.zeros((self.n, 4), np.float32)
        dv0 = np.zeros((self.n, 4), np.float32)
        dp = np.zeros((len(self.instances), 2), np.float64)
        self._check(self.L.tgpu_adjoint_backward(self._adj, gx.ctypes.data, gv.ctypes.data, dx0.ctypes.data,
                                                 dv0.ctypes.data, dp.ctypes.data), "tgpu_adjoint_backward")
        return dx0[:, :3], dv0[:, :3], dp

    def forward_ms(self):
        return self.L.tgpu_adjoint_forward_ms(self._adj)

    def backward_ms(self):
        return self.L.tgpu_adjoint_backward_ms(self._adj)

    def device_bytes(self):
        return int(self.L.tgpu_adjoint_device_bytes(self._adj)) + int(self.L.tgpu_batch_device_bytes(self._batch.ptr))


def make_function():
    """The torch.autograd.Function (torch is imported only when it is used)."""
    import torch

    class SphRolloutFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, v0, params, roll):
            x, _ = roll.forward(v0.detach().cpu().numpy(), params.detach().cpu().numpy())
            ctx.roll = roll
            return torch.from_numpy(x)

        @staticmethod
        def backward(ctx, grad_x):
            _, dv0, dp = ctx.roll.backward(grad_x.detach().cpu().numpy())
            return torch.from_numpy(dv0.copy()), torch.from_numpy(dp.copy()), None

    return SphRolloutFunction


def fit_parameters(roll: SphRollout, target, iters: int = 20, lr: float = 0.05, scale=(0.05, 20.0)):
    """Fits every instance's (alpha, c0) to a target rollout: minimises each instance's mean
    squared distance of final positions to `target` ([N, 3], instances concatenated) with
    Adam on the parameters divided by `scale`, gradients from the adjoint.  Updates
    roll.params in place; returns the history [(loss summed over instances, params copy)]."""
    scale = np.asarray(scale, np.float64)
    z = roll.params / scale
    m = np.zeros_like(z)
    v = np.zeros_like(z)
    b1, b2, eps = 0.9, 0.999, 1e-12
    history = []
    target = np.asarray(target, np.float64)
    for it in range(1, iters + 1):
        roll.params = z * scale
        x, _ = roll.forward()
        g = np.zeros((roll.n, 3), np.float64)
        loss = 0.0
        for k in range(len(roll.instances)):
            a, b = roll.offsets[k], roll.offsets[k + 1]
            d = x[a:b].astype(np.float64) - target[a:b]
            loss += float(np.mean(np.sum(d * d, axis=1)))
            g[a:b] = 2.0 * d / (b - a)
        history.append((loss, roll.params.copy()))
        _, _, dp = roll.backward(g)
        gz = dp * scale
        m = b1 * m + (1 - b1) * gz
        v = b2 * v + (1 - b2) * gz * gz
        z = z - lr * (m / (1 - b1 ** it)) / (np.sqrt(v / (1 - b2 ** it)) + eps)
    roll.params = z * scale
    return history
