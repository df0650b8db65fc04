"""Boundary-correction geometry of a sphere in a box, the way the reference runner's
crates/fullmag-plan/src/boundary_geometry.rs samples it: volume fractions phi from
R^3 sub-samples of each cell, face-link fractions from R^2 sub-samples of each face,
and boundary distances delta along +-x, +-y, +-z from the cell centre (capped at the
cell size)."""
import numpy as np


def sphere_geometry(nx, ny, nz, d, radius, centre=None, sub=4, corr_stencil=0, seed=0):
    dx, dy, dz = d
    if centre is None:
        centre = (0.5 * nx * dx, 0.5 * ny * dy, 0.5 * nz * dz)
    cx, cy, cz = centre

    def inside(x, y, z):
        return (x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 <= radius ** 2

    s = (np.arange(sub) + 0.5) / sub
    zz, yy, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    X, Y, Z = xx.reshape(-1).astype(float), yy.reshape(-1).astype(float), zz.reshape(-1).astype(float)
    n = nx * ny * nz
    phi = np.zeros(n)
    for a in s:
        for b in s:
            for c in s:
                phi += inside((X + a) * dx, (Y + b) * dy, (Z + c) * dz)
    phi /= sub ** 3

    def face(axis, side):
        f = np.zeros(n)
        for a in s:
            for b in s:
                if axis == 0:
                    f += inside((X + side) * dx, (Y + a) * dy, (Z + b) * dz)
                elif axis == 1:
                    f += inside((X + a) * dx, (Y + side) * dy, (Z + b) * dz)
                else:
                    f += inside((X + a) * dx, (Y + b) * dy, (Z + side) * dz)
        return f / sub ** 2

    faces = [face(0, 1.0), face(0, 0.0), face(1, 1.0), face(1, 0.0), face(2, 1.0), face(2, 0.0)]
    pc = np.stack([(X + 0.5) * dx - cx, (Y + 0.5) * dy - cy, (Z + 0.5) * dz - cz], axis=1)

    def distance(axis, sign, h):
        # distance from the centre to the sphere surface along sign * e_axis, capped at h
        b = sign * pc[:, axis]
        c = (pc ** 2).sum(axis=1) - radius ** 2
        disc = b * b - c
        t = -b + np.sqrt(np.maximum(disc, 0.0))
        t = np.where((disc >= 0) & (t > 0), t, h)
        return np.minimum(t, h)

    deltas = [distance(0, 1, dx), distance(0, -1, dx), distance(1, 1, dy), distance(1, -1, dy),
              distance(2, 1, dz), distance(2, -1, dz)]
    geo = {"volume_fraction": phi, "face": faces, "delta": deltas, "phi_floor": 0.05, "delta_min": 0.1 * min(d)}
    if corr_stencil:
        # a seeded symmetric correction tensor on the partially filled cells, sources = the
        # cell itself and its +x / -x neighbours (out-of-range sources marked -1)
        rng = np.random.default_rng(seed)
        tgt = np.nonzero((phi > 0) & (phi < 1))[0].astype(np.int32)
        src = np.full((tgt.size, corr_stencil), -1, dtype=np.int32)
        offs = [0, 1, -1, nx, -nx][:corr_stencil]
        for q, o in enumerate(offs):
            j = tgt + o
            ok = (j >= 0) & (j < n)
            src[ok, q] = j[ok]
        ten = rng.normal(0.0, 0.02, size=(tgt.size, corr_stencil, 6))
        geo["corr"] = (tgt, src.reshape(-1), ten.reshape(-1))
    return geo
