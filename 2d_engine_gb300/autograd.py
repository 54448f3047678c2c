"""Optional torch.autograd wrappers of the gb2d adjoints (for gradient checks).

LevelsetAdvection and Projection are torch.autograd.Functions over CPU float64
tensors in the field layouts of the C ABI; their backward passes call
gb2d_weno5_adjoint and gb2d_projection_adjoint.  centroid_height and
levelset_rk3_frozen build the differentiation workload of a rising-bubble window:
the bubble's centroid height after K level-set TVD-RK3 steps (reinitialisation off)
in a frozen advecting velocity, with torch.utils.checkpoint segments so that only
every `checkpoint_every`-th level set is kept for the backward pass.
"""
import math

import numpy as np
import torch
import torch.utils.checkpoint

from . import FIELD_PHI, FIELD_U, FIELD_UA, FIELD_V, FIELD_VA, FIELD_P, solve_opts


def _np(t):
    return t.detach().cpu().numpy().astype(np.float64, copy=False)


class LevelsetAdvection(torch.autograd.Function):
    """phi' = Levelset_Advection(phi; UA, VA, dt) (one WENO5 sweep + ghost extrapolation)."""

    @staticmethod
    def forward(ctx, phi, ua, va, gb_ctx, dt):
        gb_ctx.set(FIELD_PHI, _np(phi))
        gb_ctx.set(FIELD_UA, _np(ua))
        gb_ctx.set(FIELD_VA, _np(va))
        gb_ctx.levelset_advection(dt)
        out = torch.from_numpy(gb_ctx.get(FIELD_PHI))
        ctx.save_for_backward(phi, ua, va)
        ctx.gb, ctx.dt = gb_ctx, dt
        return out

    @staticmethod
    def backward(ctx, grad):
        phi, ua, va = ctx.saved_tensors
        g = ctx.gb
        g.set(FIELD_PHI, _np(phi))  # linearisation point: the step's input
        g.set(FIELD_UA, _np(ua))
        g.set(FIELD_VA, _np(va))
        need_vel = ctx.needs_input_grad[1] or ctx.needs_input_grad[2]
        mu, mua, mva = g.weno5_adjoint(ctx.dt, _np(grad.contiguous()), velocity=need_vel)
        return (torch.from_numpy(mu), torch.from_numpy(mua) if need_vel else None,
                torch.from_numpy(mva) if need_vel else None, None, None)


class Projection(torch.autograd.Function):
    """(u', v', p) = PROJECTION_2D::Solve(u*, v*; phi, dt) with the context's level set."""

    @staticmethod
    def forward(ctx, u, v, p0, gb_ctx, dt, opts):
        gb_ctx.set(FIELD_U, _np(u))
        gb_ctx.set(FIELD_V, _np(v))
        gb_ctx.set(FIELD_P, _np(p0))
        gb_ctx.projection(dt, opts)
        ctx.gb, ctx.dt, ctx.opts = gb_ctx, dt, opts
        return (torch.from_numpy(gb_ctx.get(FIELD_U)), torch.from_numpy(gb_ctx.get(FIELD_V)),
                torch.from_numpy(gb_ctx.get(FIELD_P)))

    @staticmethod
    def backward(ctx, gu, gv, gp):
        # Linearised at the context's last projection (its level set and system).
        mu, mv, _ = ctx.gb.projection_adjoint(ctx.dt, _np(gu.contiguous()), _np(gv.contiguous()),
                                              None if gp is None else _np(gp.contiguous()), ctx.opts)
        return torch.from_numpy(mu), torch.from_numpy(mv), None, None, None, None


def _interior(ni, nj):
    return (slice(2, 2 + nj), slice(2, 2 + ni))


def levelset_rk3_frozen(gb_ctx, phi, ua, va, dt):
    """One level-set TVD-RK3 step (EULERIAN_FLUID_SOLVER_2D.h:1694-1717) without the
    reinitialisation; the blends act on the interior, the ghosts follow the last sweep."""
    it = _interior(gb_ctx.ni, gb_ctx.nj)
    p1 = LevelsetAdvection.apply(phi, ua, va, gb_ctx, dt)
    p2 = LevelsetAdvection.apply(p1, ua, va, gb_ctx, dt)
    p3 = p2.clone()
    p3[it] = 0.75 * phi[it] + 0.25 * p2[it]
    p4 = LevelsetAdvection.apply(p3, ua, va, gb_ctx, dt)
    p5 = p4.clone()
    p5[it] = (1 / 3.0) * phi[it] + (2 / 3.0) * p4[it]
    return p5


def centroid_height(phi, ni, nj, x_max=1.0, y_max=1.0, eps=None):
    """Bubble centroid height  sum y H(-phi) / sum H(-phi)  over the nodes, with the
    smeared Heaviside of width 1.5 dx (a differentiable indicator of phi < 0)."""
    dx, dy = x_max / (ni - 1), y_max / (nj - 1)
    eps = 1.5 * dx if eps is None else eps
    p = phi[_interior(ni, nj)]
    x = -p / eps
    h = torch.where(x < -1, torch.zeros_like(x), torch.where(x > 1, torch.ones_like(x),
                    0.5 + 0.5 * x + 0.5 / math.pi * torch.sin(math.pi * x)))
    y = (torch.arange(nj, dtype=phi.dtype) * dy)[:, None]
    return (y * h).sum() / h.sum()


def window_loss(gb_ctx, phi0, ua, va, dt, steps, checkpoint_every=10, x_max=1.0, y_max=1.0):
    """Centroid height after `steps` frozen-velocity level-set RK3 steps from phi0."""
    phi = phi0
    k = 0
    while k < steps:
        n = min(checkpoint_every, steps - k)

        def segment(p, n=n):
            for _ in range(n):
                p = levelset_rk3_frozen(gb_ctx, p, ua, va, dt)
            return p

        phi = torch.utils.checkpoint.checkpoint(segment, phi, use_reentrant=False) if phi.requires_grad else segment(phi)
        k += n
    return centroid_height(phi, gb_ctx.ni, gb_ctx.nj, x_max, y_max)
