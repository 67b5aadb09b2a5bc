"""Explicit (unstructured) test meshes for the general assembly path, shared by the
fixture generator (make_golden.py) and the tests.  Each case is a dict: kind, coords,
conn, E (per element), V, t, fixed (node, dof, value) and loads (node, dof, value).
Deterministic: numpy's PCG64 with fixed seeds; node ids are permuted so that the
numbering follows no grid order."""
import numpy as np

Q4_PLANE_STRAIN, Q4_HEAT, H8_SOLID, T3_PLANE_STRAIN = 0, 1, 2, 3


def planestrain_sample():
    """sample/planestrain/sample_planestrain.cpp:20-60 in full: 6 nodes, 4 T3, its Dirichlet
    list, point load, body force (0, -300) and edge traction (0, -200) on edges {3,4}, {4,5}."""
    coords = np.array([[0, 0], [1, 0], [2, 0], [2, 1], [1, 1], [0, 1]], float)
    conn = np.array([[0, 1, 4], [1, 2, 3], [3, 4, 1], [4, 5, 0]])
    return dict(kind=T3_PLANE_STRAIN, coords=coords, conn=conn, E=np.full(4, 210000.0), V=0.3, t=1.0,
                fixed=[(0, 0, 0.0), (0, 1, 0.0), (5, 0, 0.0)], loads=[(3, 1, -100.0)],
                body=(0.0, -300.0), edges=[(3, 4), (4, 5)], traction=(0.0, -200.0))


def _jittered_grid(nx, ny, seed, jitter=0.2):
    rng = np.random.default_rng(seed)
    ii, jj = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="ij")
    xy = np.stack([ii.ravel(), jj.ravel()], 1).astype(float)
    inner = (xy[:, 0] > 0) & (xy[:, 0] < nx) & (xy[:, 1] > 0) & (xy[:, 1] < ny)
    xy[inner] += rng.uniform(-jitter, jitter, (inner.sum(), 2))
    perm = rng.permutation(len(xy))          # new id of grid node k
    coords = np.zeros_like(xy)
    coords[perm] = xy
    nid = lambda i, j: perm[(ny + 1) * i + j]  # noqa: E731
    return coords, nid, rng


def q4_jitter(nx=8, ny=5, seed=1, heat=False):
    coords, nid, rng = _jittered_grid(nx, ny, seed)
    conn = np.array([[nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)]
                     for i in range(nx) for j in range(ny)])
    E = rng.uniform(0.1, 1.0, len(conn))
    if heat:
        fixed = [(nid(0, j), 0, 1.0) for j in range(ny + 1)] + [(nid(nx, j), 0, 0.0) for j in range(0, ny + 1, 2)]
        loads = [(nid(i, ny), 0, 0.5) for i in range(1, nx)]
        return dict(kind=Q4_HEAT, coords=coords, conn=conn, E=E, V=0.3, t=1.0, fixed=fixed, loads=loads)
    fixed = [(nid(0, j), d, 0.0) for j in range(ny + 1) for d in (0, 1)] + [(nid(nx, 0), 0, 0.01)]
    loads = [(nid(nx, j), 1, -1.0 / (ny + 1)) for j in range(ny + 1)]
    edges = [(nid(i, ny), nid(i + 1, ny)) for i in range(nx)]
    return dict(kind=Q4_PLANE_STRAIN, coords=coords, conn=conn, E=E, V=0.3, t=1.0, fixed=fixed, loads=loads,
                body=(0.05, -0.1), edges=edges, traction=(0.0, -0.3))


def t3_jitter(nx=9, ny=6, seed=2):
    coords, nid, rng = _jittered_grid(nx, ny, seed)
    conn = []
    for i in range(nx):
        for j in range(ny):
            a, b, c, d = nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)
            if (i + j) % 2 == 0:
                conn += [[a, b, c], [c, d, a]]
            else:
                conn += [[a, b, d], [b, c, d]]
    conn = np.array(conn)
    E = rng.uniform(0.1, 1.0, len(conn))
    fixed = [(nid(0, j), d, 0.0) for j in range(ny + 1) for d in (0, 1)] + [(nid(nx, ny), 0, -0.02)]
    loads = [(nid(i, ny), 1, -0.5) for i in range(1, nx + 1)]
    edges = [(nid(nx, j), nid(nx, j + 1)) for j in range(ny)]
    return dict(kind=T3_PLANE_STRAIN, coords=coords, conn=conn, E=E, V=0.3, t=0.5, fixed=fixed, loads=loads,
                body=(-0.02, -0.07), edges=edges, traction=(0.1, 0.0))


def h8_jitter(nx=3, ny=2, nz=2, seed=3):
    rng = np.random.default_rng(seed)
    idx = lambda i, j, k: ((ny + 1) * i + j) * (nz + 1) + k  # noqa: E731
    xyz = np.array([[i, j, k] for i in range(nx + 1) for j in range(ny + 1) for k in range(nz + 1)], float)
    inner = np.all((xyz > 0) & (xyz < [nx, ny, nz]), axis=1)
    xyz[inner] += rng.uniform(-0.15, 0.15, (inner.sum(), 3))
    perm = rng.permutation(len(xyz))
    coords = np.zeros_like(xyz)
    coords[perm] = xyz
    nid = lambda i, j, k: perm[idx(i, j, k)]  # noqa: E731
    conn = np.array([[nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
                      nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)]
                     for i in range(nx) for j in range(ny) for k in range(nz)])
    E = rng.uniform(0.1, 1.0, len(conn))
    fixed = [(nid(0, j, k), d, 0.0) for j in range(ny + 1) for k in range(nz + 1) for d in range(3)]
    loads = [(nid(nx, j, 0), 2, -0.25) for j in range(ny + 1)]
    return dict(kind=H8_SOLID, coords=coords, conn=conn, E=E, V=0.3, t=1.0, fixed=fixed, loads=loads)


FEM_CASES = {
    "fem_planestrain_sample": planestrain_sample,
    "fem_q4_jitter": q4_jitter,
    "fem_q4_heat_jitter": lambda: q4_jitter(7, 6, seed=4, heat=True),
    "fem_t3_jitter": t3_jitter,
    "fem_h8_jitter": h8_jitter,
}


def write_mesh(case, path):
    nen = case["conn"].shape[1]
    with open(path, "w") as fh:
        fh.write(f"{case['kind']} {len(case['coords'])} {len(case['conn'])} {nen}\n")
        for x in case["coords"]:
            fh.write(" ".join(repr(float(v)) for v in x) + "\n")
        for e in case["conn"]:
            fh.write(" ".join(str(int(v)) for v in e) + "\n")
        fh.write(" ".join(repr(float(v)) for v in case["E"]) + "\n")
        fh.write(f"{case['V']!r} {case['t']!r}\n")
        fh.write(f"{len(case['fixed'])}\n")
        for n, d, v in case["fixed"]:
            fh.write(f"{int(n)} {int(d)} {float(v)!r}\n")
        fh.write(f"{len(case['loads'])}\n")
        for n, d, v in case["loads"]:
            fh.write(f"{int(n)} {int(d)} {float(v)!r}\n")
        body = case.get("body")
        edges = case.get("edges", [])
        tx, ty = case.get("traction", (0.0, 0.0))
        fh.write(f"{1 if body else 0} {float(body[0]) if body else 0.0!r} {float(body[1]) if body else 0.0!r} "
                 f"{len(edges)} {float(tx)!r} {float(ty)!r}\n")
        for a0, a1 in edges:
            fh.write(f"{int(a0)} {int(a1)}\n")
