"""Seeded synthetic inputs shared by the golden generator, the tests and bench.py.

The standalone-projection workload follows the benchmark description: node grid
on [0,1]^2, level set = signed distance to the union of 8 circles with centres
U[0.1,0.9]^2 and radii U[0.03,0.12] (phi < 0 inside, the light phase),
MAC velocity U[-1,1] smoothed by 4 Jacobi passes with wall faces zero.
numpy's PCG64 (default_rng) makes every case reproducible from its seed.
All arrays use the ghost-inclusive ARRAY_2D layout (rows = j, cols = i).
"""
import numpy as np


def node_coords(ni, nj, x_min=0.0, y_min=0.0, x_max=1.0, y_max=1.0, ghost=2):
    dx = (x_max - x_min) / (ni - 1)
    dy = (y_max - y_min) / (nj - 1)
    i = np.arange(-ghost, ni + ghost)
    j = np.arange(-ghost, nj + ghost)
    return np.meshgrid(x_min + i * dx, y_min + j * dy)


def circles_sdf(X, Y, centres, radii):
    d = np.full(X.shape, np.inf)
    for (cx, cy), r in zip(centres, radii):
        d = np.minimum(d, np.sqrt((X - cx) ** 2 + (Y - cy) ** 2) - r)
    return d


def smooth_faces(a, passes, axis_walls):
    """Jacobi smoothing: each interior face becomes the mean of itself and its 4 neighbours."""
    for _ in range(passes):
        b = a.copy()
        b[1:-1, 1:-1] = (a[1:-1, 1:-1] + a[:-2, 1:-1] + a[2:, 1:-1] + a[1:-1, :-2] + a[1:-1, 2:]) / 5.0
        a = b
        axis_walls(a)
    return a


def mac_velocity(rng, ni, nj, passes=4):
    """Interior MAC faces: u (nj, ni+1), v (nj+1, ni); wall-normal faces zero."""
    u = rng.uniform(-1.0, 1.0, (nj, ni + 1))
    v = rng.uniform(-1.0, 1.0, (nj + 1, ni))

    def uw(a):
        a[:, 0] = 0.0
        a[:, -1] = 0.0

    def vw(a):
        a[0, :] = 0.0
        a[-1, :] = 0.0
    uw(u)
    vw(v)
    return smooth_faces(u, passes, uw), smooth_faces(v, passes, vw)


def embed(interior, ghost):
    nj, ni = interior.shape
    out = np.zeros((nj + 2 * ghost, ni + 2 * ghost))
    out[ghost:ghost + nj, ghost:ghost + ni] = interior
    return out


def copy_ghosts(interior, ghost):
    """FillGhostCellsFrom semantics: ghosts copy the second interior line, corners zero."""
    out = embed(interior, ghost)
    g, (nj, ni) = ghost, interior.shape
    out[g:g + nj, :g] = interior[:, 1:2]
    out[g:g + nj, g + ni:] = interior[:, ni - 2:ni - 1]
    out[:g, g:g + ni] = interior[1:2, :]
    out[g + nj:, g:g + ni] = interior[nj - 2:nj - 1, :]
    return out


def bubbles_case(ni, nj=None, seed=0, n_circles=8, x_max=1.0, y_max=1.0):
    """Standalone projection / advection input: phi (ghost 2, SDF evaluated on the
    whole ghost-inclusive array), u, v (ghost 2), ua, va (ghost 3, snapshot of u, v)."""
    nj = ni if nj is None else nj
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.1, 0.9, (n_circles, 2)) * np.array([x_max, y_max])
    radii = rng.uniform(0.03, 0.12, n_circles)
    X, Y = node_coords(ni, nj, 0.0, 0.0, x_max, y_max, ghost=2)
    phi = circles_sdf(X, Y, centres, radii)
    u_int, v_int = mac_velocity(rng, ni, nj)
    return dict(phi=np.ascontiguousarray(phi), u=embed(u_int, 2), v=embed(v_int, 2),
                ua=copy_ghosts(u_int, 3), va=copy_ghosts(v_int, 3), p=np.zeros((nj + 2, ni + 2)),
                ni=ni, nj=nj, x_max=x_max, y_max=y_max)


def rising_bubble_case(ni, nj=None, seed=0):
    """Single bubble of radius 0.15 at (0.5, 0.3) on [0,1]^2 with quiescent-ish flow."""
    nj = ni if nj is None else nj
    rng = np.random.default_rng(seed)
    X, Y = node_coords(ni, nj, ghost=2)
    phi = np.sqrt((X - 0.5) ** 2 + (Y - 0.3) ** 2) - 0.15
    u_int, v_int = mac_velocity(rng, ni, nj)
    u_int *= 0.1
    v_int *= 0.1
    return dict(phi=np.ascontiguousarray(phi), u=embed(u_int, 2), v=embed(v_int, 2),
                ua=copy_ghosts(u_int, 3), va=copy_ghosts(v_int, 3), p=np.zeros((nj + 2, ni + 2)),
                ni=ni, nj=nj, x_max=1.0, y_max=1.0)
