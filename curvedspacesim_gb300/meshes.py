"""Synthetic triangulated surfaces and particle initial conditions.

Every mesh is returned as ``(V, F)``: ``V`` float64 ``(nV, 3)`` vertex positions and ``F`` int32 ``(nF, 3)``
vertex indices, counter-clockwise when seen from outside (outward normals).  These generators stand in for the
``.off`` meshes the reference loads through CGAL (``triangulatedMeshSpace::loadMeshFromFile``,
src/models/triangulatedMeshSpace.cpp:42-72); ``read_off`` reads those files directly.

Particle placement is area-weighted (random face with probability proportional to its area, uniform barycentric
coordinates via the square-root rule).  The reference's own ``randomPosition`` picks faces uniformly
(src/models/triangulatedMeshSpace.cpp:108-116), so positions are injected the way
``simpleModel::setParticlePositions`` does (src/models/simpleModel.cpp:204-212).  Velocities follow
``randomVectorAtPosition`` (src/models/triangulatedMeshSpace.cpp:118-138) scaled by sqrt(T) as in
``simpleModel::setMaxwellBoltzmannVelocities`` (src/models/simpleModel.cpp:223-230).
"""
from __future__ import annotations

import math

import numpy as np


# ----------------------------------------------------------------------------------------------------------------
# basic meshes
# ----------------------------------------------------------------------------------------------------------------
def icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    V = np.array(
        [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
         [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    F = np.array(
        [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
         [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
         [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
         [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    return V, F


def _subdivide(V, F):
    """Split every triangle into four through edge midpoints (midpoints shared between faces)."""
    nV = V.shape[0]
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], axis=0)
    e_sorted = np.sort(e, axis=1)
    key = e_sorted[:, 0].astype(np.int64) * (nV + 1) + e_sorted[:, 1]
    uniq, inv = np.unique(key, return_inverse=True)
    a = uniq // (nV + 1)
    b = uniq % (nV + 1)
    mids = 0.5 * (V[a] + V[b])
    nF = F.shape[0]
    m01 = nV + inv[0:nF]
    m12 = nV + inv[nF:2 * nF]
    m20 = nV + inv[2 * nF:3 * nF]
    v0, v1, v2 = F[:, 0], F[:, 1], F[:, 2]
    F2 = np.concatenate([
        np.stack([v0, m01, m20], axis=1),
        np.stack([v1, m12, m01], axis=1),
        np.stack([v2, m20, m12], axis=1),
        np.stack([m01, m12, m20], axis=1)], axis=0)
    return np.concatenate([V, mids], axis=0), F2


def icosphere(subdivisions: int, radius: float = 1.0):
    """Icosphere: subdivision 4 gives 2,562 vertices / 5,120 faces; subdivision 7 gives 163,842 / 327,680."""
    V, F = icosahedron()
    for _ in range(subdivisions):
        V, F = _subdivide(V, F)
        V /= np.linalg.norm(V, axis=1, keepdims=True)
    return V * radius, F.astype(np.int32)


def ellipsoid(subdivisions: int, axes):
    V, F = icosphere(subdivisions)
    return V * np.asarray(axes, dtype=np.float64)[None, :], F


def torus(nu: int, nv: int, R: float = 3.0, r: float = 1.0):
    """Torus from an ``nu x nv`` parametric grid with alternating diagonals (200x100: 20,000 V / 40,000 F)."""
    i = np.arange(nu)
    j = np.arange(nv)
    u = 2.0 * np.pi * i / nu
    v = 2.0 * np.pi * j / nv
    U, Vv = np.meshgrid(u, v, indexing="ij")
    X = (R + r * np.cos(Vv)) * np.cos(U)
    Y = (R + r * np.cos(Vv)) * np.sin(U)
    Z = r * np.sin(Vv)
    V = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    I, J = np.meshgrid(i, j, indexing="ij")
    I = I.ravel()
    J = J.ravel()
    a = I * nv + J
    b = ((I + 1) % nu) * nv + J
    c = ((I + 1) % nu) * nv + (J + 1) % nv
    d = I * nv + (J + 1) % nv
    alt = ((I + J) % 2) == 0
    # quad a-b-c-d is counter-clockwise seen from outside (u then v increasing)
    f1 = np.where(alt[:, None], np.stack([a, b, c], 1), np.stack([a, b, d], 1))
    f2 = np.where(alt[:, None], np.stack([a, c, d], 1), np.stack([b, c, d], 1))
    F = np.concatenate([f1, f2], axis=0).astype(np.int32)
    return V, F


def planar_grid(n: int, size: float = 1.0, jitter: float = 0.0, seed: int = 0):
    """Flat ``n x n`` square grid in z=0, alternating diagonals (an open mesh, used by known-answer tests)."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, size, n + 1)
    X, Y = np.meshgrid(x, x, indexing="ij")
    V = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)
    if jitter > 0:
        h = size / n
        inner = (X.ravel() > 0) & (X.ravel() < size) & (Y.ravel() > 0) & (Y.ravel() < size)
        V[inner, :2] += rng.uniform(-jitter * h, jitter * h, size=(inner.sum(), 2))
    F = []
    for i in range(n):
        for j in range(n):
            a = i * (n + 1) + j
            b = (i + 1) * (n + 1) + j
            c = (i + 1) * (n + 1) + j + 1
            d = i * (n + 1) + j + 1
            if (i + j) % 2 == 0:
                F += [[a, b, c], [a, c, d]]
            else:
                F += [[a, b, d], [b, c, d]]
    return V, np.array(F, dtype=np.int32)


def prism(nsides: int, nz: int, radius: float = 1.0, height: float = 2.0):
    """Open triangulated prism (polygonal cylinder, no caps): developable, every interior vertex is flat."""
    V = []
    for k in range(nz + 1):
        z = height * k / nz
        for s in range(nsides):
            a = 2.0 * np.pi * s / nsides
            V.append([radius * math.cos(a), radius * math.sin(a), z])
    F = []
    for k in range(nz):
        for s in range(nsides):
            a = k * nsides + s
            b = k * nsides + (s + 1) % nsides
            c = (k + 1) * nsides + (s + 1) % nsides
            d = (k + 1) * nsides + s
            if (k + s) % 2 == 0:
                F += [[a, b, c], [a, c, d]]
            else:
                F += [[a, b, d], [b, c, d]]
    return np.array(V, dtype=np.float64), np.array(F, dtype=np.int32)


def silo(nsides: int = 48, ncap: int = 12, nz: int = 24, radius: float = 2.0, height: float = 4.0):
    """Open "silo": a hemispherical bowl of the given radius (pole at the bottom) continued by a cylinder of the
    same radius up to z = height, open at the top rim (a border loop of nsides vertices)."""
    V = [[0.0, 0.0, -radius]]
    rings = []
    for i in range(1, ncap + 1):  # hemisphere latitudes from the pole to the equator (z = 0)
        th = 0.5 * np.pi * i / ncap
        r, z = radius * math.sin(th), -radius * math.cos(th)
        rings.append(len(V))
        for s in range(nsides):
            a = 2.0 * np.pi * (s + 0.5 * (i % 2)) / nsides
            V.append([r * math.cos(a), r * math.sin(a), z])
    for k in range(1, nz + 1):
        z = height * k / nz
        rings.append(len(V))
        for s in range(nsides):
            a = 2.0 * np.pi * (s + 0.5 * ((ncap + k) % 2)) / nsides
            V.append([radius * math.cos(a), radius * math.sin(a), z])
    F = []
    r0 = rings[0]
    for s in range(nsides):
        F.append([0, r0 + (s + 1) % nsides, r0 + s])
    for i in range(len(rings) - 1):
        lo, hi = rings[i], rings[i + 1]
        odd = (i + 1) % 2  # the upper ring is rotated by half a step when the lower one is not
        for s in range(nsides):
            a, b = lo + s, lo + (s + 1) % nsides
            if odd:
                c, d = hi + s, hi + (s + 1) % nsides
                F += [[a, b, c], [b, d, c]]
            else:
                c, d = hi + (s - 1) % nsides, hi + s
                F += [[a, d, c], [a, b, d]]
    return np.array(V, dtype=np.float64), np.array(F, dtype=np.int32)


def pyramid_cone(nsides: int, nrings: int, radius: float = 1.0, height: float = 1.0):
    """Open polygonal cone (apex + rings, no base): developable except at the apex (angle < 2*pi)."""
    V = [[0.0, 0.0, height]]
    for k in range(1, nrings + 1):
        t = k / nrings
        for s in range(nsides):
            a = 2.0 * np.pi * s / nsides
            V.append([t * radius * math.cos(a), t * radius * math.sin(a), height * (1.0 - t)])
    F = []
    for s in range(nsides):
        F.append([0, 1 + s, 1 + (s + 1) % nsides])
    for k in range(1, nrings):
        for s in range(nsides):
            a = 1 + (k - 1) * nsides + s
            b = 1 + (k - 1) * nsides + (s + 1) % nsides
            c = 1 + k * nsides + (s + 1) % nsides
            d = 1 + k * nsides + s
            F += [[a, d, c], [a, c, b]]
    return np.array(V, dtype=np.float64), np.array(F, dtype=np.int32)


def cube_surface(n: int, size: float = 1.0):
    """Closed cube surface, each side an ``n x n`` grid (two triangles per cell), outward orientation."""
    verts = {}
    V = []
    F = []

    def vid(p):
        key = tuple(int(round(c * n / size * 2)) for c in p)
        if key not in verts:
            verts[key] = len(V)
            V.append(list(p))
        return verts[key]

    h = size / n
    for axis in range(3):
        for side in (0, 1):
            u_ax = (axis + 1) % 3
            v_ax = (axis + 2) % 3
            for i in range(n):
                for j in range(n):
                    def P(ii, jj):
                        p = [0.0, 0.0, 0.0]
                        p[axis] = side * size
                        p[u_ax] = ii * h
                        p[v_ax] = jj * h
                        return vid(p)
                    a, b, c, d = P(i, j), P(i + 1, j), P(i + 1, j + 1), P(i, j + 1)
                    if side == 1:
                        F += [[a, b, c], [a, c, d]]
                    else:
                        F += [[a, c, b], [a, d, c]]
    return np.array(V, dtype=np.float64), np.array(F, dtype=np.int32)


def read_off(path: str):
    """Read a triangle ``.off`` file (the reference's exampleMeshes format)."""
    with open(path) as fh:
        tokens = []
        for line in fh:
            line = line.split("#")[0].strip()
            if line:
                tokens.extend(line.split())
    if tokens[0].upper() == "OFF":
        tokens = tokens[1:]
    nv, nf = int(tokens[0]), int(tokens[1])
    pos = 3
    V = np.array(tokens[pos:pos + 3 * nv], dtype=np.float64).reshape(nv, 3)
    pos += 3 * nv
    F = []
    for _ in range(nf):
        k = int(tokens[pos])
        idx = [int(x) for x in tokens[pos + 1:pos + 1 + k]]
        pos += 1 + k
        if k != 3:
            raise ValueError("Non-triangular mesh")
        F.append(idx)
    return V, np.array(F, dtype=np.int32)


# ----------------------------------------------------------------------------------------------------------------
# perturbed meshes (bumpy sphere, noisy torus)
# ----------------------------------------------------------------------------------------------------------------
def _real_sph_harm_all(lmax: int, theta: np.ndarray, phi: np.ndarray):
    """Orthonormal real spherical harmonics Y_lm(theta=polar, phi=azimuth) for all l <= lmax.

    Associated Legendre functions by the standard three-term recurrence (Condon-Shortley phase omitted; the sign
    convention is irrelevant for random coefficients)."""
    x = np.cos(theta)
    sx = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    P = {}
    P[(0, 0)] = np.ones_like(x)
    for m in range(1, lmax + 1):
        P[(m, m)] = (2 * m - 1) * sx * P[(m - 1, m - 1)]
    for m in range(0, lmax):
        P[(m + 1, m)] = (2 * m + 1) * x * P[(m, m)]
    for m in range(0, lmax + 1):
        for l in range(m + 2, lmax + 1):
            P[(l, m)] = ((2 * l - 1) * x * P[(l - 1, m)] - (l + m - 1) * P[(l - 2, m)]) / (l - m)
    out = []
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            am = abs(m)
            norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
            if m == 0:
                out.append(norm * P[(l, 0)])
            elif m > 0:
                out.append(math.sqrt(2.0) * norm * P[(l, am)] * np.cos(am * phi))
            else:
                out.append(math.sqrt(2.0) * norm * P[(l, am)] * np.sin(am * phi))
    return out


def bumpy_sphere(subdivisions: int = 7, amplitude: float = 0.05, lmax: int = 8, seed: int = 0):
    """Icosphere with radial displacement r = 1 + amplitude * sum_{l<=lmax} a_lm Y_lm, a_lm ~ N(0,1) from ``seed``."""
    V, F = icosphere(subdivisions)
    theta = np.arccos(np.clip(V[:, 2], -1.0, 1.0))
    phi = np.arctan2(V[:, 1], V[:, 0])
    rng = np.random.default_rng(seed)
    Ys = _real_sph_harm_all(lmax, theta, phi)
    a = rng.standard_normal(len(Ys))
    r = 1.0 + amplitude * sum(ai * Y for ai, Y in zip(a, Ys))
    return V * r[:, None], F


def _vertex_neighbors(F, nV):
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], axis=0)
    e = np.concatenate([e, e[:, ::-1]], axis=0)
    e = np.unique(e, axis=0)
    return e[:, 0], e[:, 1]


def noisy_torus(nu: int = 1000, nv: int = 500, R: float = 3.0, r: float = 1.0, std: float = 0.01,
                smoothing_rings: int = 3, seed: int = 0):
    """Torus grid with radial (tube-normal) Gaussian noise smoothed by ``smoothing_rings`` 1-ring averages.

    The smoothed field is rescaled to the stated standard deviation so the amplitude matches ``std``."""
    V, F = torus(nu, nv, R, r)
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(V.shape[0]) * std
    src, dst = _vertex_neighbors(F, V.shape[0])
    deg = np.bincount(src, minlength=V.shape[0]).astype(np.float64)
    for _ in range(smoothing_rings):
        acc = np.bincount(src, weights=noise[dst], minlength=V.shape[0])
        noise = (noise + acc) / (1.0 + deg)
    s = noise.std()
    if s > 0:
        noise = noise * (std / s)
    # tube-normal direction: from the tube centre circle to the vertex
    u = np.arctan2(V[:, 1], V[:, 0])
    centre = np.stack([R * np.cos(u), R * np.sin(u), np.zeros_like(u)], axis=1)
    nrm = V - centre
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    return V + noise[:, None] * nrm, F


# ----------------------------------------------------------------------------------------------------------------
# mesh properties and initial conditions
# ----------------------------------------------------------------------------------------------------------------
def face_areas(V, F):
    a = V[F[:, 1]] - V[F[:, 0]]
    b = V[F[:, 2]] - V[F[:, 0]]
    return 0.5 * np.linalg.norm(np.cross(a, b), axis=1)


def total_area(V, F):
    return float(face_areas(V, F).sum())


def face_normals(V, F):
    a = V[F[:, 1]] - V[F[:, 0]]
    b = V[F[:, 2]] - V[F[:, 0]]
    n = np.cross(a, b)
    return n / np.linalg.norm(n, axis=1, keepdims=True)


def area_weighted_positions(V, F, n: int, rng: np.random.Generator):
    """``n`` uniform random surface points: face ~ area, barycentrics by the square-root rule."""
    A = face_areas(V, F)
    cdf = np.cumsum(A)
    cdf /= cdf[-1]
    faces = np.searchsorted(cdf, rng.random(n), side="right").astype(np.int32)
    faces = np.minimum(faces, F.shape[0] - 1)
    r1 = np.sqrt(rng.random(n))
    r2 = rng.random(n)
    bary = np.stack([1.0 - r1, r1 * (1.0 - r2), r1 * r2], axis=1)
    return faces, bary


def tangent_velocities(V, F, faces, T: float, rng: np.random.Generator):
    """Gaussian tangent-plane velocities with the reference's in-face basis, scaled by sqrt(T)."""
    nrm = face_normals(V, F)[faces]
    orth = np.stack([nrm[:, 1], -nrm[:, 0], np.zeros(len(faces))], axis=1)
    degenerate = (nrm[:, 0] == 0) & (nrm[:, 1] == 0)
    if degenerate.any():
        n = nrm[degenerate]
        orth[degenerate] = np.stack([n[:, 1] - n[:, 2], n[:, 2] - n[:, 0], n[:, 0] - n[:, 1]], axis=1)
    orth /= np.linalg.norm(orth, axis=1, keepdims=True)
    t2 = np.cross(nrm, orth)
    g = rng.standard_normal((len(faces), 2))
    return math.sqrt(T) * (g[:, :1] * orth + g[:, 1:] * t2)


def bary_to_r3(V, F, faces, bary):
    P = V[F[faces]]
    return np.einsum("ni,nij->nj", bary, P)


def sigma_for_area_fraction(area: float, n: int, phi: float) -> float:
    """Interaction range from a target area fraction, the rule of curvedSpaceSimulation.cpp:76."""
    return 2.0 * math.sqrt(phi * area / (n * math.pi))
