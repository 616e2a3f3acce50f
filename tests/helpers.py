"""Shared test helpers: golden-file parsing, meshes, CHIEF candidates."""
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")

# Reference driver constants (main.cpp:25-26): f = 171.5 Hz, k = 2*pi*f/343.21 in float.
F_GOLDEN = 171.5
K_GOLDEN = float(np.float32(2 * 3.1415926535897932 * F_GOLDEN / 343.21))
# Field points of the golden files (main.cpp:75-96): (-(1 + 0.2 i), 0, 0), i = 1..10,
# preceded by surface node 0.
FIELD_GOLDEN = np.array([[-(1 + 0.2 * i), 0.0, 0.0] for i in range(1, 11)])


def read_cplx_file(path):
    """Parse the wrtCplxMat format '(re,im) (re,im) ...'."""
    vals = []
    for tok in open(path).read().split():
        re, im = tok.strip("()").split(",")
        vals.append(complex(float(re), float(im)))
    return np.array(vals)


def golden(name):
    return read_cplx_file(os.path.join(GOLDEN, name))


def chief_candidates():
    rows = [list(map(float, l.split()[1:])) for l in open(os.path.join(GOLDEN, "chief_candidates.txt"))
            if not l.startswith("#")]
    return np.array(rows, dtype=np.float32).astype(np.float64)


def float_bb(pts, threshold):
    """mesh::findBB in float (mesh.cu:1369-1409)."""
    p = np.asarray(pts, dtype=np.float32)
    t = np.float32(threshold)
    return np.array([p[:, 0].min() - t, p[:, 0].max() + t, p[:, 1].min() - t, p[:, 1].max() + t,
                     p[:, 2].min() - t, p[:, 2].max() + t], dtype=np.float32).astype(np.float64)


def icosphere(subdiv, radius=1.0):
    """Plain numpy icosphere with inward winding (test-side mesh builder)."""
    t = (1 + 5 ** 0.5) / 2
    v = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    v = [list(np.array(p) / np.linalg.norm(p)) for p in v]
    f = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
         [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11],
         [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                p = (np.array(v[a]) + np.array(v[b])) / 2
                v.append(list(p / np.linalg.norm(p)))
                cache[key] = len(v) - 1
            return cache[key]
        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        f = nf
    v = np.array(v) * radius
    f = np.array(f, dtype=np.int32)
    for i, (a, b, c) in enumerate(f):
        n = np.cross(v[a] - v[c], v[b] - v[c])
        if n @ (v[a] + v[b] + v[c]) > 0:
            f[i] = [b, a, c]
    return v, f


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


def uv_sphere(n_lat, n_lon, radius=1.0):
    """Closed latitude-longitude sphere: two poles and n_lat rings of n_lon
    nodes (2 + n_lat n_lon nodes, odd when n_lat and n_lon are odd)."""
    pts = [[0.0, 0.0, radius]]
    for i in range(1, n_lat + 1):
        th = np.pi * i / (n_lat + 1)
        for j in range(n_lon):
            ph = 2 * np.pi * j / n_lon
            pts.append([radius * np.sin(th) * np.cos(ph), radius * np.sin(th) * np.sin(ph), radius * np.cos(th)])
    pts.append([0.0, 0.0, -radius])
    south = len(pts) - 1
    ring = lambda i, j: 1 + (i - 1) * n_lon + (j % n_lon)
    tri = []
    for j in range(n_lon):
        tri.append([0, ring(1, j), ring(1, j + 1)])
        tri.append([south, ring(n_lat, j + 1), ring(n_lat, j)])
    for i in range(1, n_lat):
        for j in range(n_lon):
            a, b, c, d = ring(i, j), ring(i, j + 1), ring(i + 1, j), ring(i + 1, j + 1)
            tri += [[a, c, b], [b, c, d]]
    return np.array(pts), np.array(tri, dtype=np.int32)
