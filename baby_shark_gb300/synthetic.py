"""Seeded synthetic meshes with the shapes of the benchmark workloads.

No public dataset is involved; every mesh is generated from a seed with
numpy's PCG64 generator (numpy.random.default_rng):

  icosphere(subdiv, radius, noise, seed)
      icosahedron subdivided `subdiv` times (20 * 4**subdiv triangles), vertices
      on the sphere, each displaced radially by uniform noise in [-noise, noise].
  torus(R, r, nu, nv, noise, seed, rotate_x_deg, shift)
      parametric grid of nu (major) x nv (minor) quads, 2*nu*nv triangles,
      displaced along the tube normal by noise * gradient_noise(4 * p), then
      rotated about x and translated.
  gradient_noise(p, seed)
      3-D gradient (Perlin-style) noise in roughly [-1, 1]: a seeded 256-entry
      permutation, 12 edge gradients, quintic fade, trilinear blend.
  open_icosphere(subdiv, amplitude, octaves, remove, seed)
      icosphere displaced radially by `octaves` octaves of gradient noise
      (frequency doubling, amplitude halving, peak displacement `amplitude`),
      then a `remove` fraction of its faces dropped uniformly at random — a
      triangle soup with holes.
  uneven_batch(n, seed)
      n meshes alternating icospheres and displaced tori, triangle counts
      log-uniform in [1k, 500k] (icospheres take the nearest subdivision),
      noise amplitude uniform in [0.01, 0.1], and a voxel size that makes the
      bounding grid log-uniform between 64^3 and 512^3.
All triangles are oriented with outward normals.
"""
import numpy as np


def icosphere(subdiv=4, radius=1.0, noise=0.0, seed=0):
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid])
        nf = len(f)
        m01, m12, m20 = inv[:nf] + base, inv[nf:2 * nf] + base, inv[2 * nf:] + base
        f = np.concatenate([np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
                            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    rng = np.random.default_rng(seed)
    r = radius + (rng.uniform(-noise, noise, len(v)) if noise else 0.0)
    v = v * np.asarray(r)[..., None] if noise else v * radius
    # orient outward
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    flip = np.einsum("ij,ij->i", np.cross(b - a, c - a), a + b + c) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v.astype(np.float32), f.astype(np.uint32)


_GRAD = np.array([[1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1],
                  [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1]], np.float64)


def gradient_noise(p, seed=0):
    p = np.asarray(p, np.float64)
    perm = np.random.default_rng(seed).permutation(256)
    perm = np.concatenate([perm, perm])
    pi = np.floor(p).astype(np.int64)
    pf = p - pi
    pi &= 255
    fade = pf * pf * pf * (pf * (pf * 6 - 15) + 10)
    out = np.zeros(len(p))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                hsh = perm[perm[perm[pi[:, 0] + dx] + pi[:, 1] + dy] + pi[:, 2] + dz] % 12
                g = _GRAD[hsh]
                d = pf - np.array([dx, dy, dz])
                w = (fade[:, 0] if dx else 1 - fade[:, 0]) * (fade[:, 1] if dy else 1 - fade[:, 1]) * \
                    (fade[:, 2] if dz else 1 - fade[:, 2])
                out += w * np.einsum("ij,ij->i", g, d)
    return out


def torus(R=1.0, r=0.3, nu=1024, nv=512, noise=0.0, seed=0, rotate_x_deg=0.0, shift=(0.0, 0.0, 0.0)):
    u = np.arange(nu) * (2 * np.pi / nu)
    w = np.arange(nv) * (2 * np.pi / nv)
    U, W = np.meshgrid(u, w, indexing="ij")
    n = np.stack([np.cos(W) * np.cos(U), np.cos(W) * np.sin(U), np.sin(W)], -1).reshape(-1, 3)
    ring = np.stack([R * np.cos(U), R * np.sin(U), np.zeros_like(U)], -1).reshape(-1, 3)
    p = ring + r * n
    if noise:
        p = p + (noise * gradient_noise(4.0 * p + 17.0, seed))[:, None] * n
    ang = np.deg2rad(rotate_x_deg)
    rot = np.array([[1, 0, 0], [0, np.cos(ang), -np.sin(ang)], [0, np.sin(ang), np.cos(ang)]])
    p = p @ rot.T + np.asarray(shift, np.float64)
    i = np.arange(nu)[:, None]
    j = np.arange(nv)[None, :]
    a = (i * nv + j)
    b = (((i + 1) % nu) * nv + j)
    c = (((i + 1) % nu) * nv + (j + 1) % nv)
    d = (i * nv + (j + 1) % nv)
    f = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    # orient outward (normal along the tube normal)
    pa, pb, pc = p[f[:, 0]], p[f[:, 1]], p[f[:, 2]]
    cen = (pa + pb + pc) / 3
    cu = np.arctan2(cen[:, 1] - shift[1], cen[:, 0] - shift[0]) if not rotate_x_deg else None
    nrm = np.cross(pb - pa, pc - pa)
    tube_n = n[f[:, 0]] @ rot.T
    flip = np.einsum("ij,ij->i", nrm, tube_n) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    del cu
    return p.astype(np.float32), f.astype(np.uint32)


def remove_faces(faces, fraction, seed=0):
    rng = np.random.default_rng(seed)
    keep = rng.random(len(faces)) >= fraction
    return faces[keep]


def config1(seed=1):
    """Icosphere subdivision 4 (5,120 triangles), radius 1, radial noise 0.05."""
    return icosphere(4, 1.0, 0.05, seed)


def config2(seed=2, nu=1024, nv=512):
    """Two displaced tori (R 1, r 0.3, 512x1024 grid, gradient noise 0.02); the
    second is rotated 90 degrees about x and shifted 0.5 in x."""
    a = torus(1.0, 0.3, nu, nv, 0.02, seed)
    b = torus(1.0, 0.3, nu, nv, 0.02, seed + 1, rotate_x_deg=90.0, shift=(0.5, 0.0, 0.0))
    return a, b


def uneven_batch(n=256, seed=4):
    """[(vertices, triangles, voxel_size)] of the batched workload (band 3)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        target = float(np.exp(rng.uniform(np.log(1000.0), np.log(500000.0))))
        noise = float(rng.uniform(0.01, 0.1))
        res = float(np.exp(rng.uniform(np.log(64.0), np.log(512.0))))
        if k % 2 == 0:
            sub = int(np.clip(np.round(np.log(target / 20.0) / np.log(4.0)), 3, 7))
            v, f = icosphere(sub, 1.0, noise, seed=seed * 100003 + k)
        else:
            nv = max(8, int(round((target / 4.0) ** 0.5)))
            v, f = torus(1.0, float(rng.uniform(0.2, 0.4)), 2 * nv, nv, noise, seed=seed * 100003 + k)
        extent = float((v.max(axis=0) - v.min(axis=0)).max())
        out.append((v, f, np.float32(extent / res)))
    return out


def random_rotation(rng):
    """Uniform random rotation matrix (unit quaternion from four normal deviates)."""
    q = rng.normal(size=4)
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def large_union(n=16, seed=5, tri_min=524288, tri_max=1048576):
    """Large combined workload: n displaced tori with major radius in
    [0.5, 1.5], minor radius in [0.1, 0.4], a random rotation, centre in
    [-1, 1]^3 and tri_min..tri_max triangles each (grid aspect nu / nv = R / r),
    gradient-noise displacement of amplitude 0.02 r / 0.3.  Returns
    [(vertices, triangles)]; the defaults give about 12 M triangles."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        R = float(rng.uniform(0.5, 1.5))
        r = float(rng.uniform(0.1, 0.4))
        target = float(rng.uniform(tri_min, tri_max))
        nv = max(8, int(round((target / 2.0 * r / R) ** 0.5)))
        nu = max(8, int(round(target / 2.0 / nv)))
        rot = random_rotation(rng)
        centre = rng.uniform(-1.0, 1.0, size=3)
        v, f = torus(R, r, nu, nv, 0.02 * r / 0.3, seed=seed * 1000 + k)
        v = (v.astype(np.float64) @ rot.T + centre).astype(np.float32)
        out.append((v, f))
    return out


def open_icosphere(subdiv=9, amplitude=0.1, octaves=4, remove=0.1, seed=3):
    """Non-watertight workload: subdivision-9 icosphere (5,242,880 triangles),
    4-octave radial noise of amplitude 0.1, 10 % of faces removed."""
    v, f = icosphere(subdiv, 1.0, 0.0, seed)
    p = v.astype(np.float64)
    disp = np.zeros(len(p))
    for k in range(octaves):
        disp += 0.5 ** k * gradient_noise(2.0 ** k * 2.0 * p + 31.0 * (k + 1), seed + k)
    p = p * (1.0 + amplitude * disp / np.abs(disp).max())[:, None]  # peak displacement = amplitude
    return p.astype(np.float32), remove_faces(f, remove, seed + 99)
