"""Seeded synthetic inputs for the narrowband level-set step.

The reference ships no benchmark inputs (its README lists only demo meshes),
so the workloads are generated: jittered structured meshes with analytic
signed-distance initial conditions.

  square: (n+1)^2 vertices on [0,1]^2, two triangles per cell with a fixed
          diagonal; vertex (i, j) has index j*(n+1) + i (x fastest).
  cube:   (n+1)^3 vertices on [0,1]^3, Freudenthal split (6 tetrahedra per
          cell, one per ordering of the three axes); vertex (i, j, k) has
          index (k*(n+1) + j)*(n+1) + i (x fastest), the numbering of the
          reference fixture CubeMesh_size256step8_correct.node.
Interior vertices are jittered uniformly per axis; boundary vertices stay on
the boundary.
"""
import itertools

import numpy as np


def square_mesh(n, jitter=0.0, seed=0, scale=1.0):
    h = 1.0 / n
    j, i = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    xy = np.stack([i.ravel() * h, j.ravel() * h], 1)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter * h, jitter * h, size=xy.shape)
        interior = (i.ravel() > 0) & (i.ravel() < n) & (j.ravel() > 0) & (j.ravel() < n)
        xy[interior] += d[interior]
    xyz = np.zeros((len(xy), 3), np.float64)
    xyz[:, :2] = xy
    ci, cj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    ci, cj = ci.ravel(), cj.ravel()
    a = cj * (n + 1) + ci
    b = a + 1
    c = a + (n + 1)
    d = c + 1
    tris = np.concatenate([np.stack([a, b, d], 1), np.stack([a, d, c], 1)])
    return (xyz * scale).astype(np.float32), tris.astype(np.int32)


def cube_mesh(n, jitter=0.0, seed=0, scale=1.0):
    h = 1.0 / n
    N = n + 1
    k, j, i = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    xyz = np.stack([i * h, j * h, k * h], 1).astype(np.float64)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter * h, jitter * h, size=xyz.shape)
        interior = (i > 0) & (i < n) & (j > 0) & (j < n) & (k > 0) & (k < n)
        xyz[interior] += d[interior]
    ck, cj, ci = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    idx = lambda a, b, c: (c * N + b) * N + a
    tets = []
    for perm in itertools.permutations(range(3)):
        off = np.zeros(3, np.int64)
        t = [idx(ci, cj, ck)]
        for ax in perm:
            off[ax] += 1
            t.append(idx(ci + off[0], cj + off[1], ck + off[2]))
        tets.append(np.stack(t, 1))
    # cell-major order: the six tets of a cell are consecutive
    tets = np.stack(tets, 1).reshape(-1, 4)
    return (xyz * scale).astype(np.float32), tets.astype(np.int32)


def phi_circle(xyz, center=(0.5, 0.5), r=0.3):
    p = xyz[:, :2].astype(np.float64) - np.asarray(center)
    return (np.sqrt((p ** 2).sum(1)) - r).astype(np.float32)


def phi_spheres(xyz, centers, radii):
    p = xyz.astype(np.float64)
    d = np.full(len(p), np.inf)
    for c, r in zip(centers, radii):
        d = np.minimum(d, np.sqrt(((p - np.asarray(c)) ** 2).sum(1)) - r)
    return d.astype(np.float32)


def phi_torus(xyz, center=(0.5, 0.5, 0.5), R=0.3, r=0.1):
    p = xyz.astype(np.float64) - np.asarray(center)
    q = np.sqrt(p[:, 0] ** 2 + p[:, 1] ** 2) - R
    return (np.sqrt(q ** 2 + p[:, 2] ** 2) - r).astype(np.float32)


def centroids(xyz, elems):
    return xyz[elems].astype(np.float64).mean(1)


def velocity_rotation(xyz, elems, omega, center=(0.5, 0.5, 0.5), axis=(0.0, 0.0, 1.0)):
    """Rigid rotation omega * axis x (x - c) evaluated at element centroids."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    x = centroids(xyz, elems) - np.asarray(center)
    return (omega * np.cross(a, x)).astype(np.float32)


def velocity_constant(ne, v):
    out = np.zeros((ne, 3), np.float32)
    out[:, : len(v)] = v
    return out


def structured_partition(dim, nside, block):
    """GraphPartition_Square labels (meshFIM3d.cu:316-326) in numpy."""
    nb = -(-nside // block)
    ids = np.arange(nside ** dim)
    c = [(ids // nside ** a) % nside for a in range(dim)]
    part = np.zeros(len(ids), np.int64)
    for a in range(dim):
        part += (c[a] // block) * nb ** a
    return part.astype(np.int32), nb ** dim


def workload(name, seed=0, scale=1.0, n=None):
    """The benchmark configurations, as dictionaries of arrays and parameters.

    c1: 2D advection, 64x64 cells, circle r=0.3, velocity (1, 0.5), 20 steps.
    c2: 3D advection, 32^3 cells, torus R=0.3 r=0.1, rotation about z at 2 pi.
    c3: 3D mean-curvature flow, 128^3 cells, union of 3 spheres, dt = 0.5 h^2.
    `n` overrides the cells per side (smaller cases of the same family);
    `scale` multiplies coordinates (lengths, dt and the bandwidth follow).
    """
    rng = np.random.default_rng(1000 + seed)
    if name == "c1":
        n = n or 64
        h = 1.0 / n
        xyz, el = square_mesh(n, 0.2, seed)
        phi = phi_circle(xyz)
        vel = velocity_constant(len(el), (1.0, 0.5))
        spd = np.sqrt(1.0 + 0.25)
        npart, nparts = structured_partition(2, n + 1, 5)
        cfg = dict(dim=2, steps=20, dt=0.5 * h / spd, bandwidth=5 * h, update="advect", block=5)
    elif name == "c2":
        n = n or 32
        h = 1.0 / n
        xyz, el = cube_mesh(n, 0.15, seed)
        phi = phi_torus(xyz)
        vel = velocity_rotation(xyz, el, 2 * np.pi)
        vmax = float(np.sqrt((vel.astype(np.float64) ** 2).sum(1)).max())
        npart, nparts = structured_partition(3, n + 1, 3)
        cfg = dict(dim=3, steps=100, dt=0.5 * h / vmax, bandwidth=5 * h, update="advect", block=3)
    elif name == "c3":
        n = n or 128
        h = 1.0 / n
        xyz, el = cube_mesh(n, 0.15, seed)
        centers = rng.uniform(0.25, 0.75, size=(3, 3))
        radii = rng.uniform(0.1, 0.25, size=3)
        phi = phi_spheres(xyz, centers, radii)
        vel = np.zeros((len(el), 3), np.float32)
        npart, nparts = structured_partition(3, n + 1, 3)
        cfg = dict(dim=3, steps=50, dt=0.5 * h * h, bandwidth=6 * h, update="curvature", block=3,
                   centers=centers, radii=radii)
    else:
        raise ValueError(name)
    cfg.update(name=name, n=n, h=h * scale, seed=seed)
    if scale != 1.0:
        xyz = (xyz.astype(np.float64) * scale).astype(np.float32)
        phi = (phi.astype(np.float64) * scale).astype(np.float32)
        cfg["bandwidth"] *= scale
        if cfg["update"] == "curvature":
            cfg["dt"] *= scale * scale
        else:
            vel = (vel.astype(np.float64) * scale).astype(np.float32)
            cfg["dt"] *= 1.0
    return dict(xyz=xyz, elems=el, phi0=phi, vel=vel, npart=npart, nparts=nparts, **cfg)


def workload_batch(seed=0, nmesh=64, nmin=16, nmax=64, steps=100):
    """The batched configuration: nmesh independent jittered unit cubes with
    cells per side log-uniform in [nmin, nmax], each with a union of 1-3
    spheres (centres U[0.25, 0.75]^3, radii U(0.1, 0.25)) and a rigid rotation
    about a random axis (uniform on the sphere) through the cube centre with
    omega U(1, 6); dt = 0.5 h / max|v| (CFL 0.5), narrowband 5h, 3^3-vertex
    patches, advection.  Returns a list of workload() dictionaries."""
    rng = np.random.default_rng(5000 + seed)
    out = []
    for k in range(nmesh):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        h = 1.0 / n
        xyz, el = cube_mesh(n, 0.15, seed=10000 * (seed + 1) + k)
        ns = int(rng.integers(1, 4))
        centers = rng.uniform(0.25, 0.75, size=(ns, 3))
        radii = rng.uniform(0.1, 0.25, size=ns)
        phi = phi_spheres(xyz, centers, radii)
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        omega = float(rng.uniform(1.0, 6.0))
        vel = velocity_rotation(xyz, el, omega, axis=axis)
        vmax = float(np.sqrt((vel.astype(np.float64) ** 2).sum(1)).max())
        npart, nparts = structured_partition(3, n + 1, 3)
        out.append(dict(xyz=xyz, elems=el, phi0=phi, vel=vel, npart=npart, nparts=nparts, dim=3, steps=steps,
                        dt=0.5 * h / vmax, bandwidth=5 * h, update="advect", block=3, name="c5-%d" % k, n=n, h=h,
                        seed=seed, omega=omega, axis=axis, centers=centers, radii=radii))
    return out


def write_tetgen(base, xyz, tets, first=0):
    """tetgen .node/.ele pair (index base `first`, with a comment line)."""
    xyz = np.asarray(xyz, np.float64)
    with open(base + ".node", "w") as f:
        f.write("# generated mesh\n%d 3 0 0\n" % len(xyz))
        for i, p in enumerate(xyz):
            f.write("%d %.9g %.9g %.9g\n" % (i + first, p[0], p[1], p[2]))
    with open(base + ".ele", "w") as f:
        f.write("%d 4 0\n" % len(tets))
        for i, t in enumerate(np.asarray(tets)):
            f.write("%d %d %d %d %d\n" % (i + first, t[0] + first, t[1] + first, t[2] + first, t[3] + first))


def write_ply(path, xyz, faces):
    """ASCII PLY; faces is a list of vertex-index sequences (any length >= 3)."""
    xyz = np.asarray(xyz, np.float64)
    with open(path, "w") as f:
        f.write("ply\nformat ascii 1.0\ncomment generated mesh\nelement vertex %d\n" % len(xyz))
        f.write("property float x\nproperty float y\nproperty float z\n")
        f.write("element face %d\nproperty list uchar int vertex_indices\nend_header\n" % len(faces))
        for p in xyz:
            f.write("%.9g %.9g %.9g\n" % (p[0], p[1], p[2]))
        for fc in faces:
            f.write("%d %s\n" % (len(fc), " ".join(str(int(v)) for v in fc)))


def reorient(xyz, tets):
    """Positive signed volume for every tet: swap the last two vertices of
    the negative ones (the loader's orientation rule)."""
    xyz = np.asarray(xyz, np.float64)
    t = np.array(tets, np.int32, copy=True)
    a, b, c, d = (xyz[t[:, k]] for k in range(4))
    vol = np.einsum("ij,ij->i", b - a, np.cross(c - a, d - a))
    neg = vol < 0
    t[neg, 2], t[neg, 3] = tets[neg, 3], tets[neg, 2]
    return t
