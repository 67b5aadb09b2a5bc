"""Structured-grid SIMP problem definitions (the benchmark configurations).

A problem is a plain dict understood by both the GPU driver and the CPU
oracle.  Boundary-condition lists follow SquareMesh::GenerateFixedlist
(src/PrePost/Mesher/SquareMesh.h:192-207): nodes in i-major order
((ny+1)*i + j), the requested dofs in list order for each matching node.
"""
import numpy as np

Q4_PLANE_STRAIN, Q4_HEAT, H8_SOLID = 0, 1, 2


def _fixedlist(nx, ny, dofs, pred):
    nodes, ds = [], []
    for i in range(nx + 1):
        for j in range(ny + 1):
            if pred(i, j):
                for d in dofs:
                    nodes.append((ny + 1) * i + j)
                    ds.append(d)
    return nodes, ds


def _base(kind, nx, ny, nz=0, **kw):
    pr = dict(kind=kind, nx=nx, ny=ny, nz=nz, lx=float(nx), ly=float(ny), lz=float(nz),
              V=0.3, t=1.0, E1=1.0, E0=1e-9, p=3.0, vf=0.5, R=1.5, scale0=1.0, scale1=1.0,
              optimizer=0, oc_iota=0.5, oc_lmin=0.0, oc_lmax=1e4, oc_leps=1e-3, oc_move=0.2,
              mma_raa0=1e-5, mma_albefa=0.1, mma_move=0.2, mma_asyinit=0.5, mma_asydecr=0.7,
              mma_asyincr=1.2, mma_eps=1e-6, mma_a0=1.0, mma_c=1e4, mma_d=0.0, mma_xmin=0.01,
              mma_xmax=1.0, cg_eps=1e-10, cg_itmax=100000, heaviside=0)
    pr.update(kw)
    if "rho0" not in pr:
        pr["rho0"] = pr["vf"]
    return pr


def cantilever_q4(nx=60, ny=30, **kw):
    """Config 1: left edge clamped, unit downward load at the right-edge midpoint."""
    assert ny % 2 == 0
    fn, fd = _fixedlist(nx, ny, (0, 1), lambda i, j: i == 0)
    ln, ld = _fixedlist(nx, ny, (1,), lambda i, j: i == nx and 2 * j == ny)
    return _base(Q4_PLANE_STRAIN, nx, ny, fix_node=fn, fix_dof=fd, load_node=ln, load_dof=ld,
                 load_val=[-1.0] * len(ln), **kw)


def conlin_cantilever_q4(nx=60, ny=40, **kw):
    """The CONLIN sample's problem (sample_optimize_density_CONLIN.cpp:23-90): the
    cantilever with E1 = 210000, E0 = 1e-4, scale0 = 1e5, weight limit 0.5, the
    Heaviside filter (beta doubled every 40 iterations from 0.5) and CONLIN with
    move 0.2 and convergence 1e-6 (optimizer 2 reads the mma_a0/c/d/xmin/xmax/move/eps
    fields)."""
    for k, v in dict(E1=210000.0, E0=1e-4, scale0=1e5, vf=0.5, R=1.5, optimizer=2, heaviside=1,
                     mma_move=0.2, mma_eps=1e-6).items():
        kw.setdefault(k, v)
    return cantilever_q4(nx, ny, **kw)


def mbb_q4(nx=1024, ny=512, load_right=None, **kw):
    """Config 2: MBB half beam.  u_x = 0 on the left edge, u_y = 0 at the bottom-right
    node, unit downward load at the top-left node; MMA, vf 0.4, filter radius 3.
    load_right = j moves the load to the right-edge node (nx, j) (the learned
    preconditioner's training runs)."""
    fn, fd = _fixedlist(nx, ny, (0,), lambda i, j: i == 0)
    fn2, fd2 = _fixedlist(nx, ny, (1,), lambda i, j: i == nx and j == 0)
    if load_right is None:
        ln, ld = _fixedlist(nx, ny, (1,), lambda i, j: i == 0 and j == ny)
    else:
        ln, ld = _fixedlist(nx, ny, (1,), lambda i, j: i == nx and j == load_right)
    kw.setdefault("vf", 0.4)
    kw.setdefault("R", 3.0)
    kw.setdefault("optimizer", 1)
    return _base(Q4_PLANE_STRAIN, nx, ny, fix_node=fn + fn2, fix_dof=fd + fd2, load_node=ln,
                 load_dof=ld, load_val=[-1.0] * len(ln), **kw)


def heat_patch(nx, ny, edge, w, i0):
    """Predicate of the zero-temperature patch: nodes t = i0 .. i0 + w along edge
    0 (j = 0), 1 (j = ny), 2 (i = 0) or 3 (i = nx)."""
    if edge == 0:
        return lambda i, j: j == 0 and i0 <= i <= i0 + w
    if edge == 1:
        return lambda i, j: j == ny and i0 <= i <= i0 + w
    if edge == 2:
        return lambda i, j: i == 0 and i0 <= j <= i0 + w
    return lambda i, j: i == nx and i0 <= j <= i0 + w


def heatsink_q4(nx=64, ny=64, patch_w=None, patch_i0=None, edge=0, **kw):
    """Config 5 instance: zero-temperature patch on an edge (default the bottom
    one), uniform unit heat source lumped to the nodes (area/4 per adjacent
    element)."""
    w = patch_w if patch_w is not None else max(1, nx // 10)
    i0 = patch_i0 if patch_i0 is not None else ((nx if edge < 2 else ny) - w) // 2
    fn, fd = _fixedlist(nx, ny, (0,), heat_patch(nx, ny, edge, w, i0))
    h2 = (1.0 * 1.0) * 0.25
    ln, ld, lv = [], [], []
    for i in range(nx + 1):
        for j in range(ny + 1):
            c = (i > 0 and j > 0) + (i < nx and j > 0) + (i > 0 and j < ny) + (i < nx and j < ny)
            ln.append((ny + 1) * i + j)
            ld.append(0)
            lv.append(c * h2)
    kw.setdefault("E0", 1e-3)
    return _base(Q4_HEAT, nx, ny, fix_node=fn, fix_dof=fd, load_node=ln, load_dof=ld, load_val=lv,
                 patch_w=w, patch_i0=i0, edge=edge, **kw)


def heat_batch(n=256, seed=0, sides=(64, 96, 128, 192, 256, 384)):
    """Config 5: n independent square heat-sink instances, side drawn uniformly
    from `sides`, patch edge and position and volume fraction (uniform in
    [0.3, 0.5]) drawn with a seeded generator."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        side = int(rng.choice(sides))
        w = max(1, side // 10)
        edge = int(rng.integers(0, 4))
        i0 = int(rng.integers(0, side - w + 1))
        vf = float(rng.uniform(0.3, 0.5))
        out.append(dict(side=side, edge=edge, patch_w=w, patch_i0=i0, vf=vf))
    return out


def cantilever_h8(nx=128, ny=64, nz=64, **kw):
    """Config 3: clamped at x = 0, unit line load (equal split) along the bottom edge
    (z = 0) of the x = L face, in -z."""
    fn, fd, ln, ld, lv = [], [], [], [], []
    for j in range(ny + 1):
        for k in range(nz + 1):
            for d in range(3):
                fn.append(j * (nz + 1) + k)
                fd.append(d)
    for j in range(ny + 1):
        ln.append(((ny + 1) * nx + j) * (nz + 1))
        ld.append(2)
        lv.append(-1.0 / (ny + 1))
    kw.setdefault("vf", 0.15)
    kw.setdefault("R", 2.0)
    return _base(H8_SOLID, nx, ny, nz, fix_node=fn, fix_dof=fd, load_node=ln, load_dof=ld,
                 load_val=lv, **kw)


def counts(pr):
    kind, nx, ny, nz = pr["kind"], pr["nx"], pr["ny"], pr.get("nz", 0)
    if kind == H8_SOLID:
        return nx * ny * nz, (nx + 1) * (ny + 1) * (nz + 1), 3
    return nx * ny, (nx + 1) * (ny + 1), (2 if kind == Q4_PLANE_STRAIN else 1)


def fixed_mask(pr):
    ne, nn, nd = counts(pr)
    m = np.zeros(nn * nd, np.uint8)
    m[np.asarray(pr["fix_node"], np.int64) * nd + np.asarray(pr["fix_dof"], np.int64)] = 1
    return m


def jittered_q4_mesh(nx=1024, ny=512, seed=0, jitter=0.2):
    """An explicit Q4 plane-strain mesh for the general assembly path: an nx x ny grid with
    every node moved by up to `jitter` of a cell and the node ids permuted (so neighbours are
    far apart in memory, as in meshes read from files), per-element moduli uniform in
    [0.1, 1], the left edge clamped, a downward point load at the top right corner, a
    uniform body force and a uniform traction on the top edge.  Returns a dict of the
    arrays FemMesh takes."""
    rng = np.random.default_rng(seed)
    nn = (nx + 1) * (ny + 1)
    perm = rng.permutation(nn).astype(np.int32)
    i, j = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="ij")
    grid = np.stack([i, j], -1).reshape(-1, 2).astype(float)
    coords = np.empty_like(grid)
    coords[perm] = grid + rng.uniform(-jitter, jitter, grid.shape)
    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    nid = lambda a, b: perm[a * (ny + 1) + b]  # noqa: E731
    conn = np.stack([nid(I, J), nid(I + 1, J), nid(I + 1, J + 1), nid(I, J + 1)], -1).reshape(-1, 4)
    left = nid(np.zeros(ny + 1, int), np.arange(ny + 1))
    fixed = np.column_stack([np.repeat(left, 2), np.tile([0, 1], ny + 1), np.zeros(2 * (ny + 1))])
    loads = np.array([[nid(nx, ny), 1, -1.0]])
    top = nid(np.arange(nx + 1), np.full(nx + 1, ny))
    edges = np.column_stack([top[:-1], top[1:]]).astype(np.int32)
    return dict(kind=0, coords=coords, conn=conn.astype(np.int32), E=rng.uniform(0.1, 1.0, nx * ny), V=0.3, t=1.0,
                fixed=fixed, loads=loads, body=(0.0, -1e-3), edges=edges, traction=(0.0, -1e-2))
