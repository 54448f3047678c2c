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


def bubble_level_set(ni, nj, y_max, cx, cy, r):
    """Signed distance to a circle at (cx, cy) on [0,1] x [0,y_max] (dx = dy when
    y_max = (nj-1)/(ni-1)), built as the reference builds its bubbles: interior values,
    ghosts copied from the second interior line, corners at dx."""
    dx = 1.0 / (ni - 1)
    phi = np.full((nj + 4, ni + 4), dx)
    X, Y = np.meshgrid(np.arange(ni) * dx, np.arange(nj) * (y_max / (nj - 1)))
    phi[2:2 + nj, 2:2 + ni] = np.sqrt((X - cx) ** 2 + (Y - cy) ** 2) - r
    phi[2:2 + nj, 0:2] = phi[2:2 + nj, 3:4]
    phi[2:2 + nj, 2 + ni:] = phi[2:2 + nj, ni:ni + 1]
    phi[0:2, 2:2 + ni] = phi[3:4, 2:2 + ni]
    phi[2 + nj:, 2:2 + ni] = phi[nj:nj + 1, 2:2 + ni]
    return phi


def batched_bubbles(n, seed=0, sizes=(64, 128, 256, 512)):
    """Independent rising bubbles: grid N^2 with N uniform over `sizes`, radius U[0.1,0.2],
    centre (0.5, U[0.2,0.4]), density ratio log-uniform in [10,1000] (air 1), viscosity
    ratio log-uniform in [1,100] (air 0.01).  Returns (grid sizes, level sets, params, flows)."""
    rng = np.random.default_rng(seed)
    grids, phis, params, flows = [], [], [], []
    for _ in range(n):
        N = int(rng.choice(sizes))
        r, cy = rng.uniform(0.1, 0.2), rng.uniform(0.2, 0.4)
        rho = float(np.exp(rng.uniform(np.log(10), np.log(1000))))
        mu = float(np.exp(rng.uniform(np.log(1), np.log(100))))
        grids.append((N, N, 1.0, 1.0))
        phis.append(bubble_level_set(N, N, 1.0, 0.5, cy, r))
        params.append(dict(water_density=rho, air_density=1.0))
        flows.append(dict(water_viscosity=0.01 * mu, air_viscosity=0.01, viscosity=True))
    return grids, phis, params, flows


def rayleigh_taylor_level_set(ni, nj, y_max=2.0, amplitude=0.05):
    """phi = y - y_max/2 - amplitude cos(2 pi x) on [0,1] x [0,y_max] (heavy fluid where
    phi > 0, above the interface), ghosts copied from the second interior line, corners at dx."""
    dx = 1.0 / (ni - 1)
    phi = np.full((nj + 4, ni + 4), dx)
    X, Y = np.meshgrid(np.arange(ni) * dx, np.arange(nj) * (y_max / (nj - 1)))
    phi[2:2 + nj, 2:2 + ni] = Y - 0.5 * y_max - amplitude * np.cos(2 * np.pi * X)
    phi[2:2 + nj, 0:2] = phi[2:2 + nj, 3:4]
    phi[2:2 + nj, 2 + ni:] = phi[2:2 + nj, ni:ni + 1]
    phi[0:2, 2:2 + ni] = phi[3:4, 2:2 + ni]
    phi[2 + nj:, 2:2 + ni] = phi[nj:nj + 1, 2:2 + ni]
    return phi
