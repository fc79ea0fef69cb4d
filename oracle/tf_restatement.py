"""Torch-autograd restatement of the TF backend's gradient path -- TEST
INFRASTRUCTURE ONLY (timed as a CPU baseline by ``bench.py``; never product).

TensorFlow is not installed here, so the reference's ``tf`` backend cannot
run ("tf backend GradientTape: unavailable on this box").  This module
restates what a ``GradientTape`` over ``eng.run(prog, args=...)`` on that
backend computes, with the same structure and precision:

* gate matrices at the state's precision (complex64), each a custom-gradient
  node whose backward is ``grad_p = Re sum(dy * conj(dU/dp))`` -- the pattern
  of ``strawberryfields/backends/tfbackend/ops.py:190-454``
  (``single_squeezing_matrix``, ``single_displacement_matrix``,
  ``single_beamsplitter_matrix``, ``single_two_mode_squeezing_matrix``; the
  matrices and derivative matrices come from the oracle's FP64 builders, as
  the TF backend takes them from thewalrus), and diagonal gates (rotation,
  Kerr) as dense diagonal matrices built from the parameter
  (``phase_shifter_matrix``, ``kerr_interaction_matrix``, :221-256);
* every gate applied as one dense ``einsum`` on the state, a D x D matrix on
  one mode or a D^4 tensor ``[out1, in1, out2, in2]`` on two
  (``single_mode_gate`` :688-758, ``two_mode_gate`` :761-854, pure states);
* the state's gradient by reverse-mode autodiff of those einsums (torch
  autograd in place of TF's), the loss ``1 - |<target|psi>|^2``.

It runs on the host cores with torch's intra-op threads.
"""

import string

import numpy as np
import torch

from . import fock_oracle as fo

_IDX = string.ascii_lowercase


class _GateMatrix(torch.autograd.Function):
    """Gate matrix of (kind, p) at complex64, with the TF backend's custom
    gradient Re sum(dy * conj(dU/dp))."""

    @staticmethod
    def forward(ctx, p, kind, D):
        vals = [float(v) for v in p.detach()]
        U, dUs = fo.gate_matrix(kind, vals, D)
        ctx.dUs = [torch.as_tensor(d, dtype=torch.complex64) for d in dUs]
        return torch.as_tensor(U, dtype=torch.complex64)

    @staticmethod
    def backward(ctx, dy):
        g = torch.stack([torch.real(torch.sum(dy * torch.conj(d))) for d in ctx.dUs]).to(torch.float64)
        return g, None, None


def _single_mode_eqn(mode, n):
    """'ab,<...b...>-><...a...>' for a pure n-mode state."""
    other = _IDX[2:2 + n]
    ins = other[:mode] + "b" + other[mode + 1:n]
    outs = other[:mode] + "a" + other[mode + 1:n]
    return "ab," + ins + "->" + outs


def _two_mode_eqn(m1, m2, n):
    """'abcd,<...b...d...>-><...a...c...>' (gate [out1, in1, out2, in2])."""
    other = list(_IDX[4:4 + n])
    ins, outs = list(other), list(other)
    ins[m1], ins[m2] = "b", "d"
    outs[m1], outs[m2] = "a", "c"
    return "abcd," + "".join(ins) + "->" + "".join(outs)


def tf_style_loss(gates, params, N, D, target):
    """Forward of the gate list as the TF backend runs it; returns the loss
    (a differentiable function of ``params``, a float64 torch tensor)."""
    psi = torch.zeros([D] * N, dtype=torch.complex64)
    psi.view(-1)[0] = 1.0
    for kind, m1, m2, pi in gates:
        npar = fo.NPARAMS[kind]
        U = _GateMatrix.apply(params[pi:pi + npar], kind, D)
        if U.dim() == 2:
            psi = torch.einsum(_single_mode_eqn(m1, N), U, psi)
        else:
            psi = torch.einsum(_two_mode_eqn(m1, m2, N), U, psi)
    s = torch.sum(torch.conj(target) * psi)
    return 1 - (s.real ** 2 + s.imag ** 2)


def tf_style_gradient(gates, params, N, D, target):
    """(loss, gradient) of one GradientTape-style step."""
    p = torch.as_tensor(params, dtype=torch.float64).clone().requires_grad_(True)
    loss = tf_style_loss(gates, p, N, D, torch.as_tensor(target, dtype=torch.complex64))
    loss.backward()
    return float(loss.detach()), p.grad.numpy()
