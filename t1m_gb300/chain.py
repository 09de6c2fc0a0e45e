"""Left-to-right contraction sequences with a recomputing adjoint.

A chain contracts inputs X0, X1, ..., Xn step by step:

    R0 = X0,   R_i = contract(R_{i-1}[l_{i-1}], X_i[x_i]) -> R_i[l_i]

(the caller side of t1m::contract in a tensor-network sweep; the reference has
no such driver).  ``forward`` keeps only the running intermediate.
``backward`` returns the gradient of every input for an upstream gradient of
the final result, in PyTorch's conjugate-Wirtinger convention, through
t1m_contract_vjp; it stores no intermediates from the forward pass and instead
recomputes R_{i-1} from the inputs when step i needs it (n(n-1)/2 extra
contractions for n steps, memory of one intermediate at a time).

Tensors are torch tensors (device memory, row-major, i.e. C-contiguous), so a
tensor's dims are its shape; labels are strings with one character per mode.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Sequence

from . import (FLAG_NO_TIMING, Context, contract_raw, contract_vjp, default_context,
               row_major, tensor)


@dataclass(frozen=True)
class Step:
    left: str    # labels of the running intermediate
    right: str   # labels of the next input
    out: str     # labels of the result


def _view(x) -> tensor:
    return tensor(list(x.shape), x, row_major)


class ContractionChain:
    def __init__(self, input_labels: Sequence[str], out_labels: Sequence[str]):
        """input_labels[i] labels X_i; out_labels[i] labels R_{i+1}."""
        if len(out_labels) != len(input_labels) - 1:
            raise ValueError("one output label string per step")
        self.steps = []
        cur = input_labels[0]
        for x, o in zip(input_labels[1:], out_labels):
            self.steps.append(Step(cur, x, o))
            cur = o
        self.input_labels = list(input_labels)

    def _extents(self, xs) -> dict:
        ext = {}
        for x, lab in zip(xs, self.input_labels):
            if len(lab) != x.dim():
                raise ValueError(f"labels {lab!r} do not match a rank-{x.dim()} tensor")
            for ch, d in zip(lab, x.shape):
                if ext.setdefault(ch, d) != d:
                    raise ValueError(f"extent mismatch for label {ch!r}")
        return ext

    def _step(self, i, left, right, ext, ctx):
        import torch
        st = self.steps[i]
        out = torch.empty([ext[ch] for ch in st.out], dtype=left.dtype, device=left.device)
        contract_raw(1.0, _view(left), st.left, _view(right), st.right, 0.0, _view(out), st.out,
                     FLAG_NO_TIMING, ctx)
        # The context's stream is not torch's: finish before torch may reuse
        # or read any buffer of this step.
        ctx.synchronize()
        return out

    def forward(self, xs, upto: int | None = None, ctx: Context | None = None):
        """R_upto (default: the final result); keeps one intermediate at a time."""
        ctx = ctx or default_context()
        ext = self._extents(xs)
        upto = len(self.steps) if upto is None else upto
        r = xs[0]
        for i in range(upto):
            r = self._step(i, r, xs[i + 1], ext, ctx)
        return r

    def backward(self, xs, grad_out, ctx: Context | None = None):
        """Gradients of all inputs; intermediates are recomputed, not stored."""
        import torch
        ctx = ctx or default_context()
        ext = self._extents(xs)
        grads = [None] * len(xs)
        g = grad_out
        for i in range(len(self.steps) - 1, -1, -1):
            st = self.steps[i]
            left = self.forward(xs, upto=i, ctx=ctx)  # recompute R_i's left operand
            d_left = torch.empty_like(left)
            d_right = torch.empty_like(xs[i + 1])
            contract_vjp(_view(g), st.out, _view(left), st.left, _view(xs[i + 1]), st.right,
                         _view(d_left), _view(d_right), ctx=ctx, timed=False)
            ctx.synchronize()
            grads[i + 1] = d_right
            g = d_left
            del left
        grads[0] = g
        return grads
