"""Reverse-mode gradients of a fixed-step RK4 LLG run as a ``torch.autograd.Function``.

The reference has no adjoint: this is an additive capability over the same FDM
problem description (the plan of ``make_plan``) and the same fixed-step RK4 integrator
(crates/fullmag-engine/src/fdm_integrators.rs:155-262).  The trainable quantity is a
per-cell applied field map B(x, y, z) in tesla, added to the effective field as
H = B / mu0 at active cells, next to the plan's uniform external field.

``FieldMapRK4.apply(m0, b_map, backend, dt, n_steps, checkpoint_every)`` runs
``n_steps`` RK4 steps on the GPU from ``m0`` under ``b_map`` and returns the final
magnetisation; its backward pass calls ``fullmag_fdm_adjoint_backward``, which
recomputes the run segment by segment from checkpoints kept every
``checkpoint_every`` steps (default ceil(sqrt(n_steps))) and integrates the adjoint
equations backwards on the device.  Gradients come back for ``m0`` (d loss / d m0,
taken with respect to the uploaded, un-normalised initial state) and ``b_map``.
An in-plane map of shape (n, 2) is zero-padded along z and gets an (n, 2) gradient.
"""
from __future__ import annotations

import numpy as np
import torch

from .backend import MU0, FdmBackend


def _as_f64(t: torch.Tensor) -> np.ndarray:
    return np.ascontiguousarray(t.detach().to("cpu", torch.float64).numpy())


class FieldMapRK4(torch.autograd.Function):
    @staticmethod
    def forward(ctx, m0: torch.Tensor, b_map: torch.Tensor, backend: FdmBackend, dt: float, n_steps: int,
                checkpoint_every: int = 0):
        n = backend.n
        if m0.shape != (n, 3):
            raise ValueError(f"m0 must have shape ({n}, 3), got {tuple(m0.shape)}")
        if b_map.dim() != 2 or b_map.shape[0] != n or b_map.shape[1] not in (2, 3):
            raise ValueError(f"b_map must have shape ({n}, 2) or ({n}, 3), got {tuple(b_map.shape)}")
        h = _as_f64(b_map) / MU0
        if h.shape[1] == 2:
            h = np.concatenate([h, np.zeros((n, 1))], axis=1)
        backend.upload(_as_f64(m0))
        backend.set_field_map(h)
        backend.adjoint_forward(dt, int(n_steps), int(checkpoint_every))
        m_final = backend.magnetization()
        ctx.backend = backend
        ctx.in_plane = b_map.shape[1] == 2
        ctx.meta = (m0.dtype, m0.device, b_map.dtype, b_map.device)
        return torch.from_numpy(m_final).to(device=m0.device, dtype=m0.dtype)

    @staticmethod
    def backward(ctx, grad_m: torch.Tensor):
        m_dtype, m_dev, b_dtype, b_dev = ctx.meta
        want_m0 = ctx.needs_input_grad[0]
        grad_h, lam0 = ctx.backend.adjoint_backward(_as_f64(grad_m), want_lambda0=want_m0)
        grad_b = grad_h / MU0
        if ctx.in_plane:
            grad_b = grad_b[:, :2]
        gb = torch.from_numpy(np.ascontiguousarray(grad_b)).to(device=b_dev, dtype=b_dtype)
        gm = torch.from_numpy(lam0).to(device=m_dev, dtype=m_dtype) if want_m0 else None
        return gm, gb, None, None, None, None


def rk4_final_state(m0: torch.Tensor, b_map: torch.Tensor, backend: FdmBackend, dt: float, n_steps: int,
                    checkpoint_every: int = 0) -> torch.Tensor:
    """Differentiable final magnetisation of ``n_steps`` RK4 steps under ``b_map`` (tesla)."""
    return FieldMapRK4.apply(m0, b_map, backend, dt, n_steps, checkpoint_every)
