"""torch.autograd bridge: the saved states of a NeuralODE solve as a
differentiable tensor whose backward is the library's adjoint kernel.

This plays the part of SciMLSensitivity's ``ChainRulesCore.rrule`` on
``solve`` (selected by ``sensealg`` at src/neural_de.jl:57): the forward keeps
the checkpoints on the device, the backward receives dL/d(saved states) and
returns dL/du0 and dL/dp.
"""
import torch

from . import _lib


def _sync(t):
    if t.is_cuda:
        torch.cuda.current_stream(t.device).synchronize()


class _SolveSaveat(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, p, node):
        solver = node.solver
        S, B = u0.shape
        desc = node.desc()
        ns = desc.nsave
        if u0.is_cuda:
            pc = p.detach().to(torch.float32).contiguous()
            u0_cm = u0.detach().to(torch.float32).t().contiguous()      # column-major S x B
            out = torch.empty((ns, B, S), dtype=torch.float32, device=u0.device)
            _sync(u0_cm)
            solver.set_params_device(pc)
            stats = solver.forward_device(u0_cm, out, desc, S, B)
            ctx._keep = (u0_cm, out, pc, desc)
            arr = out.permute(2, 1, 0)
        else:
            pn = p.detach().cpu().numpy()
            un = u0.detach().cpu().numpy()
            solver.set_params(pn)
            a, stats = solver.forward(un, desc)
            ctx._keep = (un, pn, desc)
            arr = torch.from_numpy(a.copy())
        # the library differentiates the context's last forward: remember
        # which one this is
        ctx.generation = solver.generation
        ctx.node = node
        ctx.stats = stats
        node.last_stats = stats
        ctx.is_cuda = u0.is_cuda
        return arr

    @staticmethod
    def backward(ctx, g):
        node = ctx.node
        solver = node.solver
        if ctx.stats.retcode != _lib.RET_SUCCESS:
            raise RuntimeError("cannot differentiate a failed solve (retcode %d)" % ctx.stats.retcode)
        if solver.generation != ctx.generation:
            # Another solve ran on this context after this node's forward (the
            # layer was called twice before backward, or a training step ran):
            # solve this node's forward again, from the same u0 and p, so that
            # the adjoint reads its own checkpoints. The solve is deterministic,
            # so the checkpoints are the ones the saved states came from.
            if ctx.is_cuda:
                u0_cm, out, pc, desc = ctx._keep
                B, S = u0_cm.shape   # column-major S x B
                redo = torch.empty_like(out)
                solver.set_params_device(pc)
                solver.forward_device(u0_cm, redo, desc, S, B)
            else:
                un, pn, desc = ctx._keep
                solver.set_params(pn)
                solver.forward(un, desc)
            ctx.generation = solver.generation
        if ctx.is_cuda:
            g_cm = g.to(torch.float32).permute(2, 1, 0).contiguous()
            S, B, _ = g.shape
            du0 = torch.empty((B, S), dtype=torch.float32, device=g.device)
            dp = torch.empty(solver.nparams, dtype=torch.float32, device=g.device)
            _sync(g_cm)
            node.last_adj_stats = solver.backward_device(g_cm, du0, dp)
            return du0.t(), dp, None
        du0, dp, node.last_adj_stats = solver.backward(g.detach().cpu().numpy())
        return torch.from_numpy(du0.copy()), torch.from_numpy(dp), None


def solve_saveat(node, u0, p):
    """Differentiable saved states (S, B, nsave) of ``node`` from ``u0`` with ``p``;
    returns (tensor, forward stats)."""
    arr = _SolveSaveat.apply(u0, p, node)
    return arr, node.last_stats
