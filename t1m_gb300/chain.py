"""Left-to-right contraction sequences with an adjoint, one call per step or
one grouped launch per pass.

A chain contracts inputs X0, X1, ..., Xn step by step:

    R0 = X0,   R_i = contract(R_{i-1}[l_{i-1}], X_i[x_i]) -> R_i[l_i]

(the caller side of t1m::contract in a tensor-network sweep; the reference has
no such driver).  ``backward`` returns the gradient of every input for an
upstream gradient of the final result, in PyTorch's conjugate-Wirtinger
convention:

    d right_i = conj(left_i) * g_i        g_{i-1} = g_i * conj(right_i)

Two modes:

* ``"recompute"`` (default): one t1m_contract / t1m_contract_vjp call per step.
  ``forward`` keeps only the running intermediate; ``backward`` stores no
  intermediates and recomputes R_{i-1} from the inputs when step i needs it
  (n(n-1)/2 extra contractions for n steps, memory of one intermediate at a
  time).
* ``"grouped"``: each pass is ONE grouped launch (t1m_group_*, captured in a
  CUDA graph): the forward as n items chained by in-launch dependencies, with
  every intermediate kept in device memory; the backward as 2n items (the
  adjoint products, conjugation as item flags), each gradient step depending
  on the one before.  Groups are planned once per set of buffers and shapes
  and replayed afterwards.  Memory: all n intermediates and n gradients of
  intermediates.  Labels of A, B and C alike (batch labels) are not taken by
  grouped launches; such chains run in the recompute mode.

Tensors are torch tensors (device memory, row-major, i.e. C-contiguous), so a
tensor's dims are its shape; labels are strings with one character per mode.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Sequence

from . import (FLAG_CONJ_A, FLAG_CONJ_B, FLAG_NO_TIMING, Context, Group, contract_raw,
               contract_vjp, default_context, row_major, tensor)


@dataclass(frozen=True)
class Step:
    left: str    # labels of the running intermediate
    right: str   # labels of the next input
    out: str     # labels of the result


def _view(x) -> tensor:
    return tensor(list(x.shape), x, row_major)


class ContractionChain:
    def __init__(self, input_labels: Sequence[str], out_labels: Sequence[str],
                 mode: str = "recompute"):
        """input_labels[i] labels X_i; out_labels[i] labels R_{i+1}."""
        if len(out_labels) != len(input_labels) - 1:
            raise ValueError("one output label string per step")
        if mode not in ("recompute", "grouped"):
            raise ValueError(f"unknown chain mode {mode!r}")
        self.steps = []
        cur = input_labels[0]
        for x, o in zip(input_labels[1:], out_labels):
            self.steps.append(Step(cur, x, o))
            cur = o
        self.input_labels = list(input_labels)
        batch = any(set(st.left) & set(st.right) & set(st.out) for st in self.steps)
        self.mode = "recompute" if batch else mode
        self._fwd = None   # (key, group, intermediates)
        self._bwd = None   # (key, group, gradients)

    def _extents(self, xs) -> dict:
        ext = {}
        for x, lab in zip(xs, self.input_labels):
            if len(lab) != x.dim():
                raise ValueError(f"labels {lab!r} do not match a rank-{x.dim()} tensor")
            for ch, d in zip(lab, x.shape):
                if ext.setdefault(ch, d) != d:
                    raise ValueError(f"extent mismatch for label {ch!r}")
        return ext

    # ------------------------------------------------------ recompute mode ---
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

    def _forward_calls(self, xs, upto, ext, ctx):
        r = xs[0]
        for i in range(upto):
            r = self._step(i, r, xs[i + 1], ext, ctx)
        return r

    # -------------------------------------------------------- grouped mode ---
    @staticmethod
    def _key(*tensors):
        return tuple((t.data_ptr(), tuple(t.shape), str(t.dtype)) for t in tensors)

    def _forward_group(self, xs, ext, ctx):
        """The forward pass as one grouped launch; returns the intermediates
        R_1..R_n (kept by the chain until the next forward on other buffers)."""
        import torch
        key = (self._key(*xs), id(ctx))
        if self._fwd is None or self._fwd[0] != key:
            if self._fwd is not None:
                self._fwd[1].close()
            dev, dt = xs[0].device, xs[0].dtype
            rs = [torch.empty([ext[ch] for ch in st.out], dtype=dt, device=dev)
                  for st in self.steps]
            items = []
            for i, st in enumerate(self.steps):
                left = xs[0] if i == 0 else rs[i - 1]
                items.append((1.0, _view(left), st.left, _view(xs[i + 1]), st.right, 0.0,
                              _view(rs[i]), st.out, i - 1))
            self._fwd = (key, Group(items, ctx=ctx, graph=True), rs)
        self._fwd[1].launch(timed=False)
        ctx.synchronize()
        return self._fwd[2]

    def _backward_group(self, xs, rs, grad_out, ctx):
        import torch
        n = len(self.steps)
        key = (self._key(*xs, *rs, grad_out), id(ctx))
        if self._bwd is None or self._bwd[0] != key:
            if self._bwd is not None:
                self._bwd[1].close()
            # gs[i]: gradient of the step-i left operand (R_i's left), i = 0..n-1;
            # grads[i + 1]: gradient of X_{i+1}.
            gs = [torch.empty_like(xs[0] if i == 0 else rs[i - 1]) for i in range(n)]
            dxs = [torch.empty_like(xs[i + 1]) for i in range(n)]
            items, producer = [], {}
            for i in range(n - 1, -1, -1):
                st = self.steps[i]
                g = grad_out if i == n - 1 else gs[i + 1]
                dep = -1 if i == n - 1 else producer[i + 1]
                left = xs[0] if i == 0 else rs[i - 1]
                # d X_{i+1} = conj(left) * g
                items.append((1.0, _view(left), st.left, _view(g), st.out, 0.0, _view(dxs[i]),
                              st.right, dep, FLAG_CONJ_A))
                # g_{i} (gradient of left) = g * conj(X_{i+1})
                items.append((1.0, _view(g), st.out, _view(xs[i + 1]), st.right, 0.0,
                              _view(gs[i]), st.left, dep, FLAG_CONJ_B))
                producer[i] = len(items) - 1
            self._bwd = (key, Group(items, ctx=ctx, graph=True), gs, dxs)
        self._bwd[1].launch(timed=False)
        ctx.synchronize()
        _, _, gs, dxs = self._bwd
        return [gs[0]] + list(dxs)

    # ------------------------------------------------------------- public ---
    def forward(self, xs, upto: int | None = None, ctx: Context | None = None):
        """R_upto (default: the final result)."""
        ctx = ctx or default_context()
        ext = self._extents(xs)
        upto = len(self.steps) if upto is None else upto
        if self.mode == "grouped" and upto == len(self.steps) and upto > 0:
            return self._forward_group(xs, ext, ctx)[-1]
        return self._forward_calls(xs, upto, ext, ctx)

    def backward(self, xs, grad_out, ctx: Context | None = None):
        """Gradients of all inputs.  Recompute mode: intermediates recomputed,
        not stored; grouped mode: one grouped launch per pass."""
        import torch
        ctx = ctx or default_context()
        ext = self._extents(xs)
        if self.mode == "grouped" and self.steps:
            rs = self._forward_group(xs, ext, ctx)
            return self._backward_group(xs, rs, grad_out.contiguous(), ctx)
        grads = [None] * len(xs)
        g = grad_out
        for i in range(len(self.steps) - 1, -1, -1):
            st = self.steps[i]
            left = self._forward_calls(xs, i, ext, ctx)  # recompute R_i's left operand
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

    def close(self) -> None:
        """Free the planned groups (grouped mode)."""
        for slot in (self._fwd, self._bwd):
            if slot is not None:
                slot[1].close()
        self._fwd = self._bwd = None
