"""Seeded synthetic point sets for the H-matrix workloads.

The reference publishes no benchmark inputs, so every workload is generated
here from a fixed seed (numpy PCG64): points on a cylinder, a sphere, a cube
surface or an ellipsoid, laid out as htool expects them -- an (N, 3) array of
doubles, C-contiguous, i.e. xyz interleaved per point (the ``const double *x``
argument of ``Cluster::build``, include/htool/clustering/cluster.hpp:57).
"""
import ctypes
import ctypes.util
import math

import numpy as np


def cylinder(n, seed=1):
    """Uniform on the lateral surface of the cylinder r=1, z in [0, 1)."""
    g = np.random.default_rng(seed)
    th = g.uniform(0.0, 2.0 * np.pi, n)
    z = g.uniform(0.0, 1.0, n)
    return np.ascontiguousarray(np.stack([np.cos(th), np.sin(th), z], 1))


def sphere(n, seed=1):
    """Uniform on the unit sphere (normalised Gaussian triples)."""
    g = np.random.default_rng(seed)
    p = g.standard_normal((n, 3))
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    return np.ascontiguousarray(p)


def cube_surface(n, seed=1):
    """Uniform on the surface of the unit cube [0,1]^3 (faces have equal area)."""
    g = np.random.default_rng(seed)
    face = g.integers(0, 6, n)
    uv = g.uniform(0.0, 1.0, (n, 2))
    p = np.empty((n, 3))
    axis = face // 2
    side = (face % 2).astype(np.float64)
    for a in range(3):
        m = axis == a
        others = [b for b in range(3) if b != a]
        p[m, a] = side[m]
        p[m, others[0]] = uv[m, 0]
        p[m, others[1]] = uv[m, 1]
    return np.ascontiguousarray(p)


def ellipsoid(n, axes, seed=1):
    """Normalised Gaussian triples scaled by the three semi-axes."""
    g = np.random.default_rng(seed)
    p = g.standard_normal((n, 3))
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    return np.ascontiguousarray(p * np.asarray(axes, dtype=np.float64)[None, :])


def disk_glibc(n, z, srand_seed=None):
    """htool's test geometry create_disk (include/htool/testing/geometry.hpp:10-22):
    points in the unit disk at height z drawn with the C library's rand().
    When srand_seed is given, srand() is called first (the reference tests call
    srand(1) and then draw the target and source disks one after the other)."""
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    libc.rand.restype = ctypes.c_int
    if srand_seed is not None:
        libc.srand(ctypes.c_uint(srand_seed))
    rand_max = 2147483647.0
    p = np.empty((n, 3))
    for j in range(n):
        rho = libc.rand() / rand_max
        theta = libc.rand() / rand_max
        p[j, 0] = math.sqrt(rho) * math.cos(2 * math.pi * theta)
        p[j, 1] = math.sqrt(rho) * math.sin(2 * math.pi * theta)
        p[j, 2] = z
    return p


def rhs(n, mu=1, seed=2, dtype=np.float64):
    """N(0,1) right-hand sides, column-major n x mu as htool's mvprod expects."""
    g = np.random.default_rng(seed)
    if np.dtype(dtype).kind == "c":
        v = g.standard_normal((mu, n)) + 1j * g.standard_normal((mu, n))
    else:
        v = g.standard_normal((mu, n))
    return np.ascontiguousarray(v.reshape(-1).astype(dtype))
