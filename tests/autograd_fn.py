"""torch.autograd.Function over t1m_gb300 (test harness only, for gradcheck).

forward: C = A*B through t1m_contract; backward: t1m_contract_vjp.  Tensors
are CUDA, C-contiguous (row-major), labels one character per mode.
"""
import torch

import t1m_gb300 as t1m


class T1MContract(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, b, la, lb, lc, method):
        ext = dict(zip(la, a.shape))
        ext.update(zip(lb, b.shape))
        out = torch.empty([ext[ch] for ch in lc], dtype=a.dtype, device=a.device)
        c = _context(method)
        t1m.contract_raw(1.0, t1m.tensor(list(a.shape), a.contiguous(), t1m.row_major), la,
                         t1m.tensor(list(b.shape), b.contiguous(), t1m.row_major), lb, 0.0,
                         t1m.tensor(list(out.shape), out, t1m.row_major), lc, 0, c)
        ctx.save_for_backward(a, b)
        ctx.labels = (la, lb, lc)
        ctx.method = method
        return out

    @staticmethod
    def backward(ctx, grad):
        a, b = ctx.saved_tensors
        la, lb, lc = ctx.labels
        g = grad.contiguous()
        da = torch.empty_like(a)
        db = torch.empty_like(b)
        view = lambda x: t1m.tensor(list(x.shape), x, t1m.row_major)  # noqa: E731
        t1m.contract_vjp(view(g), lc, view(a.contiguous()), la, view(b.contiguous()), lb,
                         view(da), view(db), ctx=_context(ctx.method))
        return da, db, None, None, None, None


_contexts = {}


def _context(method):
    if method not in _contexts:
        c = t1m.Context()
        c.set_method(method)
        _contexts[method] = c
    return _contexts[method]


def contract(a, b, la, lb, lc, method="auto"):
    return T1MContract.apply(a, b, la, lb, lc, method)
