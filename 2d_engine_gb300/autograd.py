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


class ReinitSweep(torch.autograd.Function):
    """phi' = one WENO5thReinitialization sweep (ADVECTION_METHOD_2D.h:1401-1658) of phi with the
    sign field S held (gb2d_reinit_sweep_apply; backward gb2d_reinit_sweep_adjoint)."""

    @staticmethod
    def forward(ctx, phi, sign, gb_ctx):
        out = torch.from_numpy(gb_ctx.reinit_sweep(_np(phi), _np(sign)))
        ctx.save_for_backward(phi, sign)
        ctx.gb = gb_ctx
        return out

    @staticmethod
    def backward(ctx, grad):
        phi, sign = ctx.saved_tensors
        mu, ms = ctx.gb.reinit_sweep_adjoint(_np(phi), _np(sign), _np(grad.contiguous()))
        return torch.from_numpy(mu), torch.from_numpy(ms), None


def reinitialization(gb_ctx, phi):
    """LEVELSET_2D Reinitialization (EULERIAN_FLUID_SOLVER_2D.h:2425-2445): S = phi / sqrt(phi^2 +
    dx^2) of the starting level set, then the context's reinit_iterations sweeps with pseudo time
    step dx / reinit_scaling.  S is a torch expression, so the sweeps' derivative in S flows back
    into the starting level set."""
    g = gb_ctx.grid
    dx = (g.x_max - g.x_min) / (gb_ctx.ni - 1)
    p = phi[_interior(gb_ctx.ni, gb_ctx.nj)]
    sign = p / torch.sqrt(p * p + dx * dx)
    for _ in range(gb_ctx.params.reinit_iterations):
        phi = ReinitSweep.apply(phi, sign, gb_ctx)
    return phi


def _blend(keep, phi, c0, c1, it):
    out = phi.clone()
    out[it] = c0 * keep[it] + c1 * phi[it]
    return out


def levelset_rk3(gb_ctx, phi, ua, va, dt):
    """The whole level-set update of one order-3 time step (EULERIAN_FLUID_SOLVER_2D.h:1694-1741):
    the advection TVD-RK3, then the reinitialisation TVD-RK3 of three Reinitialization calls with
    the interior blends; the forward equals gb2d_levelset_rk3 (to the rounding of S)."""
    it = _interior(gb_ctx.ni, gb_ctx.nj)
    b = levelset_rk3_frozen(gb_ctx, phi, ua, va, dt)
    r = reinitialization(gb_ctx, reinitialization(gb_ctx, b))
    r = reinitialization(gb_ctx, _blend(b, r, 0.75, 0.25, it))
    return _blend(b, r, 1 / 3.0, 2 / 3.0, it)


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


class ProjectDensities(torch.autograd.Function):
    """(u', v') = projection of a fixed intermediate velocity as a function of the two densities
    (water, air: 0-d tensors); backward through gb2d_projection_adjoint and
    gb2d_projection_density_gradient."""

    @staticmethod
    def forward(ctx, water, air, make_context, state, dt, opts):
        c = make_context(float(water), float(air))
        for f, k in ((FIELD_PHI, "phi"), (FIELD_U, "u"), (FIELD_V, "v"), (FIELD_P, "p")):
            c.set(f, state[k])
        c.projection(dt, opts, allow_max_iters=True)
        ctx.c, ctx.dt, ctx.opts = c, dt, opts
        return torch.from_numpy(c.get(FIELD_U)), torch.from_numpy(c.get(FIELD_V))

    @staticmethod
    def backward(ctx, gu, gv):
        c = ctx.c
        c.projection_adjoint(ctx.dt, _np(gu.contiguous()), _np(gv.contiguous()), None, ctx.opts)
        dw, da = c.projection_density_gradient(ctx.dt)
        c.close()
        return (torch.tensor(dw, dtype=torch.float64), torch.tensor(da, dtype=torch.float64), None, None, None, None)


def advecting_copy(u, g_in=2, g_out=3):
    """The advecting copy of a MAC component, as Solve_Velocity makes it (FillGhostCellsFrom,
    FIELD_STRUCTURE_2D.h:374-449): interior copied, every ghost layer the second interior line,
    corners zero.  Differentiable."""
    nJ, nI = u.shape[0] - 2 * g_in, u.shape[1] - 2 * g_in
    inner = u[g_in:g_in + nJ, g_in:g_in + nI]
    out = torch.zeros((nJ + 2 * g_out, nI + 2 * g_out), dtype=u.dtype)
    out[g_out:g_out + nJ, g_out:g_out + nI] = inner
    out[g_out:g_out + nJ, :g_out] = inner[:, 1:2].expand(nJ, g_out)
    out[g_out:g_out + nJ, g_out + nI:] = inner[:, nI - 2:nI - 1].expand(nJ, g_out)
    out[:g_out, g_out:g_out + nI] = inner[1:2, :].expand(g_out, nI)
    out[g_out + nJ:, g_out:g_out + nI] = inner[nJ - 2:nJ - 1, :].expand(g_out, nI)
    return out


def buoyant_window_loss(gb, ni, nj, state, water, air, dt, steps, checkpoint_every=10, opts=None):
    """A coupled differentiation window: the intermediate velocity u* of one gravity step
    projected with densities (water, air) gives the advecting velocity, the bubble's level set
    is advected `steps` level-set TVD-RK3 steps by it (reinitialisation off), and the loss is
    the centroid height.  Differentiable in the densities (projection adjoint) and in the
    advected level set's initial values (WENO5 adjoint); the projection's own level set is
    held fixed."""
    opts = opts or solve_opts(tolerance=1e-11, max_iterations=20000)

    def make(w, a):
        from . import Context
        return Context(ni, nj, 0.0, 0.0, state["x_max"], state["y_max"], water_density=w, air_density=a)

    u, v = ProjectDensities.apply(water, air, make, state, dt, opts)
    ua, va = advecting_copy(u), advecting_copy(v)
    c = make(1000.0, 1.0)
    phi0 = torch.from_numpy(state["phi"].copy())
    phi = phi0
    k = 0
    while k < steps:
        n = min(checkpoint_every, steps - k)

        def segment(p, a_, b_, n=n):
            for _ in range(n):
                p = levelset_rk3_frozen(c, p, a_, b_, dt)
            return p

        phi = torch.utils.checkpoint.checkpoint(segment, phi, ua, va, use_reentrant=False)
        k += n
    loss = centroid_height(phi, ni, nj, state["x_max"], state["y_max"])
    return loss, c


class Project(torch.autograd.Function):
    """(u', v') = projection of a fixed intermediate velocity as a function of the level set
    (PHI's layout, ghost 2) and the two densities (0-d tensors); backward through
    gb2d_projection_adjoint, gb2d_projection_phi_gradient and gb2d_projection_density_gradient."""

    @staticmethod
    def forward(ctx, phi, water, air, make_context, state, dt, opts):
        c = make_context(float(water), float(air))
        c.set(FIELD_PHI, _np(phi.detach().contiguous()))
        for f, k in ((FIELD_U, "u"), (FIELD_V, "v"), (FIELD_P, "p")):
            c.set(f, state[k])
        c.projection(dt, opts, allow_max_iters=True)
        ctx.c, ctx.dt, ctx.opts = c, dt, opts
        return torch.from_numpy(c.get(FIELD_U)), torch.from_numpy(c.get(FIELD_V))

    @staticmethod
    def backward(ctx, gu, gv):
        c = ctx.c
        c.projection_adjoint(ctx.dt, _np(gu.contiguous()), _np(gv.contiguous()), None, ctx.opts)
        dphi = torch.from_numpy(c.projection_phi_gradient(ctx.dt))
        dw, da = c.projection_density_gradient(ctx.dt)
        c.close()
        return (dphi, torch.tensor(dw, dtype=torch.float64), torch.tensor(da, dtype=torch.float64), None, None, None, None)


def coupled_window_loss(gb, ni, nj, state, phi0, water, air, dt, steps, checkpoint_every=10, opts=None):
    """The fully coupled window: the level set phi0 (PHI's layout) and the densities set the
    projection of the intermediate velocity of one gravity step; the projected faces, copied
    into the advecting velocity, carry phi0 through `steps` level-set TVD-RK3 steps
    (reinitialisation off); the loss is the centroid height.  Differentiable in phi0 through
    both paths (the projection's face weights, jump terms, curvature and velocity update, and
    the WENO5 advection) and in the two densities."""
    opts = opts or solve_opts(tolerance=1e-11, max_iterations=20000)

    def make(w, a):
        from . import Context
        return Context(ni, nj, 0.0, 0.0, state["x_max"], state["y_max"], water_density=w, air_density=a,
                       surface_tension=state.get("sigma", 0.0728))

    u, v = Project.apply(phi0, water, air, make, state, dt, opts)
    ua, va = advecting_copy(u), advecting_copy(v)
    c = make(1000.0, 1.0)
    phi = phi0
    k = 0
    while k < steps:
        n = min(checkpoint_every, steps - k)

        def segment(p, a_, b_, n=n):
            for _ in range(n):
                p = levelset_rk3_frozen(c, p, a_, b_, dt)
            return p

        phi = torch.utils.checkpoint.checkpoint(segment, phi, ua, va, use_reentrant=False)
        k += n
    return centroid_height(phi, ni, nj, state["x_max"], state["y_max"]), c


def ghost_copy_transpose(mu, nI, nJ, g_src=2, g_dst=3):
    """Transpose of the ghost-filled copy (FillGhostCellsFrom: interior copied, each ghost layer the
    second interior line, corners left alone) of a field with ghost g_src into one with ghost
    g_dst: the cotangent mu of the copy (ghost g_dst layout) summed back onto the source's cells
    (ghost g_src layout).  numpy, float64."""
    out = np.zeros((nJ + 2 * g_src, nI + 2 * g_src))
    inner = mu[g_dst:g_dst + nJ, g_dst:g_dst + nI]
    out[g_src:g_src + nJ, g_src:g_src + nI] += inner
    rows = mu[g_dst:g_dst + nJ, :]                    # in-range rows, ghost columns
    out[g_src:g_src + nJ, g_src + 1] += rows[:, :g_dst].sum(axis=1)
    out[g_src:g_src + nJ, g_src + nI - 2] += rows[:, g_dst + nI:].sum(axis=1)
    cols = mu[:, g_dst:g_dst + nI]                    # in-range columns, ghost rows
    out[g_src + 1, g_src:g_src + nI] += cols[:g_dst, :].sum(axis=0)
    out[g_src + nJ - 2, g_src:g_src + nI] += cols[g_dst + nJ:, :].sum(axis=0)
    return out


class VelocityAdvection(torch.autograd.Function):
    """(u', v') = Velocity_Advection of (u, v): the advecting copies UA, VA refreshed from u, v,
    then ENO3 on both MAC components (gb2d_velocity_advection, FP64 forms).  Backward:
    gb2d_velocity_advection_adjoint on the copies, mapped back through the copy's transpose,
    plus the identity part of u' = u - dt (...)."""

    @staticmethod
    def forward(ctx, u, v, make_context, dt):
        c = make_context()
        c.set(FIELD_U, _np(u.detach().contiguous()))
        c.set(FIELD_V, _np(v.detach().contiguous()))
        c.velocity_advection(dt)
        ctx.c, ctx.dt = c, dt
        return torch.from_numpy(c.get(FIELD_U)), torch.from_numpy(c.get(FIELD_V))

    @staticmethod
    def backward(ctx, gu, gv):
        c = ctx.c
        gu_np, gv_np = _np(gu.contiguous()), _np(gv.contiguous())
        mu_ua, mu_va = c.velocity_advection_adjoint(ctx.dt, gu_np, gv_np)
        ni, nj = c.ni, c.nj
        du = gu_np + ghost_copy_transpose(mu_ua, ni + 1, nj)
        dv = gv_np + ghost_copy_transpose(mu_va, ni, nj + 1)
        c.close()
        return torch.from_numpy(du), torch.from_numpy(dv), None, None


class ProjectVelocity(torch.autograd.Function):
    """(u', v') = projection of (u, v) with level set phi and the two densities; backward through
    gb2d_projection_adjoint (velocity), gb2d_projection_phi_gradient and
    gb2d_projection_density_gradient.  p is the warm start (the solve's result does not depend
    on it beyond its tolerance); the projected pressure is left in state["p"]."""

    @staticmethod
    def forward(ctx, phi, u, v, water, air, make_context, state, dt, opts):
        c = make_context(float(water), float(air))
        c.set(FIELD_PHI, _np(phi.detach().contiguous()))
        c.set(FIELD_U, _np(u.detach().contiguous()))
        c.set(FIELD_V, _np(v.detach().contiguous()))
        c.set(FIELD_P, state["p"])
        c.projection(dt, opts, allow_max_iters=True)
        state["p"] = c.get(FIELD_P)
        ctx.c, ctx.dt, ctx.opts = c, dt, opts
        return torch.from_numpy(c.get(FIELD_U)), torch.from_numpy(c.get(FIELD_V))

    @staticmethod
    def backward(ctx, gu, gv):
        c = ctx.c
        mu, mv, _ = c.projection_adjoint(ctx.dt, _np(gu.contiguous()), _np(gv.contiguous()), None, ctx.opts, allow_max_iters=True)
        dphi = c.projection_phi_gradient(ctx.dt)
        dw, da = c.projection_density_gradient(ctx.dt)
        c.close()
        t = lambda x: torch.tensor(x, dtype=torch.float64)
        return (torch.from_numpy(dphi), torch.from_numpy(mu), torch.from_numpy(mv), t(dw), t(da), None, None, None, None)


def gravity_walls(u, v, dt, gravity=(0.0, -9.8), g=2, walls=True, gravity_on=True):
    """The flow stage without viscosity (k_flow with gravity and walls): every interior face
    gains dt * gravity, then the wall-normal faces (U at i = 0 and i = ni, V at j = 0 and
    j = nj) become zero; ghost faces are left as they are.  Differentiable.  With viscosity the
    stage is gravity (walls=False), Viscosity, then the walls (gravity_on=False)."""
    nj, ni1 = u.shape[0] - 2 * g, u.shape[1] - 2 * g
    nj1, ni = v.shape[0] - 2 * g, v.shape[1] - 2 * g
    u2, v2 = u.clone(), v.clone()
    if gravity_on:
        u2[g:g + nj, g:g + ni1] = u[g:g + nj, g:g + ni1] + dt * gravity[0]
        v2[g:g + nj1, g:g + ni] = v[g:g + nj1, g:g + ni] + dt * gravity[1]
    if not walls:
        return u2, v2
    u2[g:g + nj, g] = 0.0
    u2[g:g + nj, g + ni1 - 1] = 0.0
    v2[g, g:g + ni] = 0.0
    v2[g + nj1 - 1, g:g + ni] = 0.0
    return u2, v2


class Viscosity(torch.autograd.Function):
    """(u', v') = ApplyViscosity (VISCOSITY_2D.h:460-532) of (u, v) with the level set phi, as
    gb2d_sourcing applies it (no gravity, no walls); backward gb2d_viscosity_adjoint, in u, v,
    phi (the smeared viscosities and face densities) and the two densities.  make_context(w, a)
    returns a context with those densities; flow holds set_flow_params' viscosities."""

    @staticmethod
    def forward(ctx, phi, u, v, water, air, make_context, flow, dt):
        c = make_context(float(water), float(air))
        c.set_flow_params(viscosity=True, **flow)
        c.set(FIELD_PHI, _np(phi))
        c.set(FIELD_U, _np(u))
        c.set(FIELD_V, _np(v))
        c.sourcing(dt)
        out = torch.from_numpy(c.get(FIELD_U)), torch.from_numpy(c.get(FIELD_V))
        c.set(FIELD_U, _np(u))  # the linearisation point: the stage's inputs
        c.set(FIELD_V, _np(v))
        ctx.c, ctx.dt = c, dt
        return out

    @staticmethod
    def backward(ctx, gu, gv):
        c = ctx.c
        mu, mv, mp, (dw, da) = c.viscosity_adjoint(ctx.dt, _np(gu.contiguous()), _np(gv.contiguous()))
        c.close()
        t = lambda x: torch.tensor(x, dtype=torch.float64)
        return torch.from_numpy(mp), torch.from_numpy(mu), torch.from_numpy(mv), t(dw), t(da), None, None, None


def extrapolate_ghost1(phi, g=2):
    """phi with its ghost-1 ring (not the corners) linearly extrapolated from the interior, as the
    projection's in-place ghost extrapolation leaves it (k_extrapolate: 2 f(0) - f(1) on each
    side).  Differentiable."""
    nj, ni = phi.shape[0] - 2 * g, phi.shape[1] - 2 * g
    out = phi.clone()
    r = slice(g, g + nj)
    c = slice(g, g + ni)
    out[r, g - 1] = 2.0 * phi[r, g] - phi[r, g + 1]
    out[r, g + ni] = 2.0 * phi[r, g + ni - 1] - phi[r, g + ni - 2]
    out[g - 1, c] = 2.0 * phi[g, c] - phi[g + 1, c]
    out[g + nj, c] = 2.0 * phi[g + nj - 1, c] - phi[g + nj - 2, c]
    return out


def time_step(gb_ls, phi, u, v, ua, va, water, air, dt, make_context, state, opts, gravity=(0.0, -9.8), reinit=False,
              viscosity=None):
    """One order-3 AdvanceOneTimeStepThread (EULERIAN_FLUID_SOLVER_2D.h:1694-1794) as autograd
    operations: the level-set TVD-RK3 in the advecting copies ua, va of the previous step's last
    velocity stage (with reinit, followed by the reinitialisation TVD-RK3 of gb_ls's
    reinit_iterations sweeps), then the velocity TVD-RK3 of three SolveForRK stages (ENO3
    advection, gravity, the explicit viscosity when `viscosity` holds set_flow_params'
    viscosities, walls, projection).  Returns the new (phi, u, v) and the advecting copies the
    last stage read (the next step's ua, va).  Differentiable in phi, u, v, ua, va and the two
    densities."""
    phi = levelset_rk3(gb_ls, phi, ua, va, dt) if reinit else levelset_rk3_frozen(gb_ls, phi, ua, va, dt)
    uk, vk = u, v
    for stage in range(3):
        ua, va = advecting_copy(u), advecting_copy(v)
        u, v = VelocityAdvection.apply(u, v, lambda: make_context(1000.0, 1.0), dt)
        if viscosity is None:
            u, v = gravity_walls(u, v, dt, gravity)
        else:
            # Stage 1 reads the level set's ghosts as the level-set update left them; the later
            # stages read them after the first projection's extrapolation.
            u, v = gravity_walls(u, v, dt, gravity, walls=False)
            u, v = Viscosity.apply(phi if stage == 0 else extrapolate_ghost1(phi), u, v, water, air, make_context, viscosity,
                                   dt)
            u, v = gravity_walls(u, v, dt, (0.0, 0.0), gravity_on=False)
        u, v = ProjectVelocity.apply(phi, u, v, water, air, make_context, state, dt, opts)
        if stage == 1:
            u, v = 0.75 * uk + 0.25 * u, 0.75 * vk + 0.25 * v
        elif stage == 2:
            u, v = (1 / 3.0) * uk + (2 / 3.0) * u, (1 / 3.0) * vk + (2 / 3.0) * v
    return phi, u, v, ua, va


def time_step_window_loss(gb, ni, nj, phi0, u0, v0, water, air, dt, steps, checkpoint_every=10, opts=None, surface_tension=0.0728,
                          viscosity=None, gravity=(0.0, -9.8), p0=None, x_max=1.0, y_max=1.0):
    """The bubble's centroid height after `steps` whole order-3 time steps (time_step, the
    reinitialisation off inside the window) from (phi0, u0, v0) at rest-frame advecting copies of
    u0, v0, with torch.utils.checkpoint segments of `checkpoint_every` steps.  Differentiable in
    phi0, u0, v0 and the densities water, air (0-d tensors).  viscosity: set_flow_params'
    viscosities, or None.

    Memory: the segments run their forward without building a graph (re-entrant checkpoint),
    so the GPU contexts that the velocity-advection, viscosity and projection operations hold
    for their backward exist only while one segment is recomputed and differentiated; between
    segments only each segment's starting state and its starting warm-start pressure are kept.
    The recompute starts every projection from the same warm start as the first forward did, so
    it repeats that forward exactly."""
    opts = solve_opts(precision=0, tolerance=1e-10, max_iterations=20000) if opts is None else opts
    kw = dict(x_max=x_max, y_max=y_max, surface_tension=surface_tension, reinit_iterations=0, advection_precision=0)

    def make(w, a):
        return gb.Context(ni, nj, 0.0, 0.0, water_density=w, air_density=a, **kw)

    ls = gb.Context(ni, nj, 0.0, 0.0, **kw)
    state = {"p": np.zeros(ls.shape(FIELD_P)) if p0 is None else p0.copy()}
    phi, u, v = phi0, u0, v0
    ua, va = advecting_copy(u0), advecting_copy(v0)
    k = 0
    while k < steps:
        n = min(checkpoint_every, steps - k)

        def segment(p, uu, vv, aa, bb, w, a, n=n, p_start=state["p"].copy()):
            state["p"] = p_start.copy()  # the warm start this segment began from, also when recomputed
            for _ in range(n):
                p, uu, vv, aa, bb = time_step(ls, p, uu, vv, aa, bb, w, a, dt, make, state, opts, gravity, viscosity=viscosity)
            return p, uu, vv, aa, bb

        args = (phi, u, v, ua, va, water, air)
        if torch.is_grad_enabled() and any(isinstance(x, torch.Tensor) and x.requires_grad for x in args):
            phi, u, v, ua, va = torch.utils.checkpoint.checkpoint(segment, *args, use_reentrant=True)
        else:
            phi, u, v, ua, va = segment(*args)
        k += n
    # ls stays open: the checkpointed segments run again through it in the backward pass
    # (Context frees its device state when it is collected).
    return centroid_height(phi, ni, nj, x_max, y_max)
