"""Seeded synthetic node sets for the RBF-FD hot path.

The reference reads node sets from CSV / CGNS files (test/data, examples/*.cgns); the
benchmarks here use synthetic sets of the documented shapes instead.  Random numbers come
from a counter-based splitmix64 stream, so a (seed, stream, index) triple always gives the
same double on every machine.
"""
import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x):
    """splitmix64 finaliser of a uint64 array (wrapping arithmetic)."""
    z = np.asarray(x, dtype=np.uint64) + np.uint64(0x9E3779B97F4A7C15)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform(seed, stream, n, start=0):
    """n doubles in [0, 1): (splitmix64(key + i) >> 11) * 2^-53."""
    key = splitmix64(np.array([(seed << 20) ^ stream], dtype=np.uint64))[0]
    with np.errstate(over="ignore"):
        ctr = key + np.arange(start, start + n, dtype=np.uint64)
    return (splitmix64(ctr) >> np.uint64(11)).astype(np.float64) * (2.0**-53)


def jittered_grid(nx, ny=None, jitter=0.3, seed=1, box=((0.0, 1.0), (0.0, 1.0))):
    """Cell-centred nx x ny grid over `box`, each coordinate moved by U(-jitter*h, jitter*h).
    Nodes are ordered row by row (x fastest).  Returns (X (N,2) float64, hx, hy)."""
    ny = nx if ny is None else ny
    (x0, x1), (y0, y1) = box
    hx, hy = (x1 - x0) / nx, (y1 - y0) / ny
    ix = np.tile(np.arange(nx, dtype=np.float64), ny)
    iy = np.repeat(np.arange(ny, dtype=np.float64), nx)
    N = nx * ny
    ux = uniform(seed, 1, N)
    uy = uniform(seed, 2, N)
    X = np.empty((N, 2), np.float64)
    X[:, 0] = (x0 + (ix + 0.5) * hx) + (2.0 * ux - 1.0) * (jitter * hx)
    X[:, 1] = (y0 + (iy + 0.5) * hy) + (2.0 * uy - 1.0) * (jitter * hy)
    return X, hx, hy


def manufactured(X):
    """f = sin(2 pi x) cos(3 pi y) and its exact derivatives (fx, fy, Laplacian)."""
    x, y = X[:, 0], X[:, 1]
    f = np.sin(2 * np.pi * x) * np.cos(3 * np.pi * y)
    fx = 2 * np.pi * np.cos(2 * np.pi * x) * np.cos(3 * np.pi * y)
    fy = -3 * np.pi * np.sin(2 * np.pi * x) * np.sin(3 * np.pi * y)
    lap = -13 * np.pi**2 * f
    return f, fx, fy, lap


# (stencil size, polynomial degree) classes of the uneven batch
SIZE_CLASSES = ((20, 2), (30, 3), (45, 4), (60, 5))


def rectangle_with_ghosts(total=2_097_152, seed=4, main_fraction=0.85):
    """Rectangle [0,2] x [0,1] with boundary nodes on its four edges (left, right, top, bottom
    = boundaries 1..4, the marker order of examples/adv_diff_test.jl:27), one ghost node per
    boundary node at offset h along the outward normal (src/genghostnodes.jl:4), and a jittered
    interior trimmed (seeded) so that the set has exactly `total` nodes.

    Returns dict(X, node_class, n, deg, h, counts): node_class 0 interior, +b boundary b,
    -b ghost of b; n/deg per node: main_fraction of nodes (k=30, deg 3), the rest spread
    evenly over the other SIZE_CLASSES."""
    ny = 8
    while 2 * ny * ny + 12 * ny < total:
        ny += 1
    h = 1.0 / ny
    nx = 2 * ny
    Xi, _, _ = jittered_grid(nx, ny, 0.3, seed, box=((0.0, 2.0), (0.0, 1.0)))
    n_b = 6 * ny
    excess = len(Xi) + 2 * n_b - total
    if excess > 0:
        order = np.argsort(uniform(seed, 7, len(Xi)), kind="stable")
        keep = np.sort(order[excess:])
        Xi = Xi[keep]
    t_y = (np.arange(ny) + 0.5) * h
    t_x = (np.arange(nx) + 0.5) * h
    edges = [
        (np.stack([np.zeros(ny), t_y], 1), (-1.0, 0.0)),  # left
        (np.stack([np.full(ny, 2.0), t_y], 1), (1.0, 0.0)),  # right
        (np.stack([t_x, np.ones(nx)], 1), (0.0, 1.0)),  # top
        (np.stack([t_x, np.zeros(nx)], 1), (0.0, -1.0)),  # bottom
    ]
    parts = [Xi]
    cls = [np.zeros(len(Xi), np.int32)]
    for b, (P, _) in enumerate(edges, start=1):
        parts.append(P)
        cls.append(np.full(len(P), b, np.int32))
    for b, (P, nrm) in enumerate(edges, start=1):
        parts.append(P + np.array(nrm) * h)  # genghostnodes: element + normal * offset
        cls.append(np.full(len(P), -b, np.int32))
    X = np.ascontiguousarray(np.concatenate(parts))
    node_class = np.concatenate(cls)
    assert len(X) == total, (len(X), total)
    u = uniform(seed, 9, total)
    main = SIZE_CLASSES.index((30, 3))
    others = [i for i in range(len(SIZE_CLASSES)) if i != main]
    k = np.full(total, main, np.int64)
    rest = u >= main_fraction
    pick = ((u[rest] - main_fraction) / (1 - main_fraction) * len(others)).astype(np.int64)
    k[rest] = np.array(others)[np.minimum(pick, len(others) - 1)]
    n = np.array([c[0] for c in SIZE_CLASSES], np.int32)[k]
    deg = np.array([c[1] for c in SIZE_CLASSES], np.int32)[k]
    counts = {
        "interior": int((node_class == 0).sum()),
        "boundary": int((node_class > 0).sum()),
        "ghost": int((node_class < 0).sum()),
        "per_class": {f"k{c[0]}_d{c[1]}": int((k == i).sum()) for i, c in enumerate(SIZE_CLASSES)},
    }
    return dict(X=X, node_class=node_class, n=n, deg=deg, h=h, counts=counts)
