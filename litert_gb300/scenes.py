"""Seeded synthetic scenes and cameras of the benchmark configurations.

* sphere SBS (radius 0.6 in [-1,1]^3) seen from (0,0,3), fov 60 -- the reference
  test camera (tests/tests.cpp:29-41);
* Perlin-displaced icosphere mesh (7 subdivisions, 327,680 triangles) seen from
  a seeded point of the radius-3 sphere, fov 45, 1920x1080;
* smooth union of 48 spheres and 16 rounded boxes (polynomial smooth minimum,
  k = 0.05) sampled into 8-voxel bricks at octree depth 7 (1024^3 effective
  grid), 16 views of uneven size on a radius-3 orbit placed like
  get_cameras_uniform_sphere (diff_render/DR_common.cpp:224-241).

All randomness is numpy's PCG64 with fixed seeds; the reference's own scenes
(rand()-based) are not reproduced bit for bit.
"""
import numpy as np

from . import lrt

# ---------------------------------------------------------------- cameras
def camera(eye, target, up, fov_deg, width, height, znear=0.1, zfar=100.0):
    wv = lrt.look_at(eye, target, up)
    pj = lrt.perspective(fov_deg, float(width) / float(height), znear, zfar)
    return (int(width), int(height), wv, pj)


def uniform_sphere_cameras(rng, count, radius, center=(0.0, 0.0, 0.0)):
    """get_cameras_uniform_sphere semantics: (eye, center, up) per camera."""
    c = np.asarray(center, np.float32)
    out = []
    for _ in range(count):
        phi = 2 * np.pi * rng.random()
        psi = (np.pi / 2) * (1 - np.sqrt(rng.random()))
        if rng.random() > 0.5:
            psi = -psi
        vd = np.array([np.cos(psi) * np.sin(phi), np.sin(psi), np.cos(psi) * np.cos(phi)], np.float32)
        tangent = np.cross(vd, -np.array([0, 1, 0], np.float32))
        tangent /= np.linalg.norm(tangent)
        up = np.cross(vd, tangent)
        up /= np.linalg.norm(up)
        out.append((c - radius * vd, c, up))
    return out


# ---------------------------------------------------------------- config 1: sphere
SPHERE_SDF = dict(spheres=np.array([[0.0, 0.0, 0.0, 0.6]], np.float32), boxes=None, k=0.0)


def sphere_sdf():
    return lrt.Sdf(**SPHERE_SDF)


def sphere_view(width=256, height=256):
    return camera((0, 0, 3), (0, 0, 0), (0, 1, 0), 60.0, width, height)


# ---------------------------------------------------------------- config 3: smooth union
def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def union_params(seed=3, n_spheres=48, n_boxes=16, k=0.05):
    rng = np.random.default_rng(seed)
    sph = np.zeros((n_spheres, 4), np.float32)
    sph[:, :3] = rng.uniform(-0.8, 0.8, (n_spheres, 3))
    sph[:, 3] = rng.uniform(0.05, 0.3, n_spheres)
    box = np.zeros((n_boxes, 16), np.float32)
    for i in range(n_boxes):
        box[i, :3] = rng.uniform(-0.8, 0.8, 3)
        box[i, 3:6] = rng.uniform(0.05, 0.25, 3)
        box[i, 6] = 0.02
        box[i, 7:16] = _random_rotation(rng).T.reshape(9)   # world -> local = R^T
    return dict(spheres=sph, boxes=box, k=k)


def union_sdf(seed=3):
    return lrt.Sdf(**union_params(seed))


def union_views(n_views=16, size_seed=4, cam_seed=5, lo=512, hi=2048, fov=60.0):
    rs = np.random.default_rng(size_seed)
    sizes = [(int(rs.integers(lo, hi + 1)), int(rs.integers(lo, hi + 1))) for _ in range(n_views)]
    cams = uniform_sphere_cameras(np.random.default_rng(cam_seed), n_views, 3.0)
    return [camera(e, c, u, fov, w, h) for (w, h), (e, c, u) in zip(sizes, cams)]


# ---------------------------------------------------------------- config 2: displaced icosphere
def icosphere(subdiv):
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = np.array(v, np.float64)
    verts /= np.linalg.norm(verts, axis=1, keepdims=True)
    faces = np.array(f, np.int64)
    for _ in range(subdiv):
        e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]], 0)
        e.sort(1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = verts[uniq[:, 0]] + verts[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = verts.shape[0]
        verts = np.concatenate([verts, mid], 0)
        nf = faces.shape[0]
        a, b, c = faces[:, 0], faces[:, 1], faces[:, 2]
        ab, bc, ca = base + inv[:nf], base + inv[nf:2 * nf], base + inv[2 * nf:]
        faces = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1),
                                np.stack([ab, bc, ca], 1)], 0)
    return verts, faces


def _perlin(p, perm):
    """Improved gradient noise (Perlin 2002) at points p (n,3), float64."""
    def fade(t):
        return t * t * t * (t * (t * 6 - 15) + 10)

    def grad(h, x, y, z):
        h = h & 15
        u = np.where(h < 8, x, y)
        v = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, z))
        return np.where(h & 1, -u, u) + np.where(h & 2, -v, v)

    pi = np.floor(p).astype(np.int64)
    f = p - pi
    X, Y, Z = pi[:, 0] & 255, pi[:, 1] & 255, pi[:, 2] & 255
    x, y, z = f[:, 0], f[:, 1], f[:, 2]
    u, v, w = fade(x), fade(y), fade(z)
    A = perm[X] + Y
    AA, AB = perm[A] + Z, perm[A + 1] + Z
    B = perm[X + 1] + Y
    BA, BB = perm[B] + Z, perm[B + 1] + Z

    def lerp(t, a, b):
        return a + t * (b - a)

    return lerp(w, lerp(v, lerp(u, grad(perm[AA], x, y, z), grad(perm[BA], x - 1, y, z)),
                        lerp(u, grad(perm[AB], x, y - 1, z), grad(perm[BB], x - 1, y - 1, z))),
                lerp(v, lerp(u, grad(perm[AA + 1], x, y, z - 1), grad(perm[BA + 1], x - 1, y, z - 1)),
                     lerp(u, grad(perm[AB + 1], x, y - 1, z - 1), grad(perm[BB + 1], x - 1, y - 1, z - 1))))


def displaced_icosphere(subdiv=7, amplitude=0.05, octaves=3, seed=1, frequency=2.0):
    verts, faces = icosphere(subdiv)
    rng = np.random.default_rng(seed)
    p = rng.permutation(256)
    perm = np.concatenate([p, p]).astype(np.int64)
    fbm = np.zeros(verts.shape[0])
    amp, freq = 1.0, frequency
    for _ in range(octaves):
        fbm += amp * _perlin(verts * freq, perm)
        amp *= 0.5
        freq *= 2.0
    r = 1.0 + amplitude * fbm
    return (verts * r[:, None]).astype(np.float32), faces.astype(np.uint32)


def mesh_view(seed=2, width=1920, height=1080, fov=45.0):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    eye = 3.0 * d
    up = np.array([0, 1, 0], np.float32) if abs(d[1]) < 0.99 else np.array([1, 0, 0], np.float32)
    return camera(eye, (0, 0, 0), up, fov, width, height)


# ---------------------------------------------------------------- config 5: differentiable reconstruction
def turntable_cameras(count, center=(0.0, 0.0, 0.0), radius=3.0, height=1.0):
    """get_cameras_turntable semantics (diff_render/DR_common.cpp:243-257): cameras on a
    circle at the given height, (eye, center, up) each."""
    c = np.asarray(center, np.float32)
    out = []
    for i in range(count):
        phi = 2.0 * np.pi * i / count
        vd = np.array([np.sin(phi), -height / radius, np.cos(phi)], np.float32)
        tangent = np.cross(vd, -np.array([0, 1, 0], np.float32))
        tangent /= np.linalg.norm(tangent)
        up = np.cross(vd, tangent)
        up /= np.linalg.norm(up)
        out.append((c - radius * vd, c, up))
    return out


def dr_views(n_views=8, size=512, fov=60.0, radius=3.0, height=1.0):
    """The reconstruction's cameras: a turntable of n_views at `size` x `size`."""
    return [camera(e, c, u, fov, size, size, znear=0.01, zfar=100.0)
            for e, c, u in turntable_cameras(n_views, radius=radius, height=height)]


def dr_workload(target_bricks=32, target_brick_size=8, opt_bricks=32, opt_brick_size=4, n_views=8, size=512):
    """Differentiable SDF reconstruction: targets are the smooth-union scene sampled
    on a dense 256^3 grid (32^3 bricks of 8 voxels) with position colours,
    rendered from the turntable; the optimised grid is 128^3 (32^3 bricks of 4
    voxels) initialised to a sphere of radius 0.5 with a single colour.
    Returns (target sbs, initial sbs, views); each sbs = [hdr, nodes, values, params]."""
    from . import dr
    up = union_params()
    target = list(dr.grid_sbs(target_bricks, target_brick_size, lrt.Sdf(up["spheres"], up["boxes"], up["k"]), None))
    init = list(dr.grid_sbs(opt_bricks, opt_brick_size, lrt.Sdf(spheres=np.array([[0, 0, 0, 0.5]], np.float32)),
                            [1.0, 0.0, 0.0]))
    return target, init, dr_views(n_views, size)


# ---------------------------------------------------------------- config 4: learned proposal on the config-3 scene
def proposal_views(n_views, size=1024, seed=6, fov=60.0):
    """Square views from cameras uniform on the radius-3 sphere (training: seed 6,
    64 views; evaluation: seed 8, 16 views)."""
    cams = uniform_sphere_cameras(np.random.default_rng(seed), n_views, 3.0)
    return [camera(e, c, u, fov, size, size) for e, c, u in cams]
