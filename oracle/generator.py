"""numpy restatement of the project's procedural terrain generator (test infrastructure only).

The product library generates grids on the device (``tdag_generate_*`` in libtdag.so); this
module is the independent CPU statement of the same integer-only definition, used by the tests
to check the device generator bit for bit and to feed the CPU oracle.

Definition (written for this project, not taken from any noise library): fBm of value noise,
5 octaves, lacunarity 2, gain 0.5, base frequency 1/64, evaluated in fixed point so that the
CPU and GPU agree exactly.

* Octave ``o`` (0..4) uses lattice cells of ``64 >> o`` voxels.
* Lattice value: a 32-bit integer hash of (ix, iy, iz, octave, seed), top 16 bits.
* Sample point: voxel centre, fraction ``(2a + 1) / (2 cell)`` inside its cell.
* Smoothstep weight in Q16: ``floor(65536 * f^2 (3 - 2f))`` computed with integers.
* Trilinear interpolation: ``(v0 * (65536 - w) + v1 * w) >> 16`` along x, then y, then z.
* fbm = sum over octaves of ``value_o * (16 >> o)`` (max 31 * 65535).
* A voxel is solid where ``fbm / (31 * 65535) - z / res > 0``, i.e. ``fbm * res > z * 31 * 65535``.
"""
from __future__ import annotations

import numpy as np

M32 = np.uint64(0xFFFFFFFF)


def _mix32(h):
    h = h & M32
    h ^= h >> np.uint64(15)
    h = (h * np.uint64(0x2C1B3C6D)) & M32
    h ^= h >> np.uint64(12)
    h = (h * np.uint64(0x297A2D39)) & M32
    h ^= h >> np.uint64(15)
    return h


def lattice_value(ix, iy, iz, octave: int, seed: int):
    """16-bit lattice value (uint64 array)."""
    h = np.uint64((seed * 0x9E3779B1 + octave * 0x85EBCA77) & 0xFFFFFFFF)
    h = _mix32(h ^ ((ix.astype(np.uint64) * np.uint64(0x27D4EB2F)) & M32))
    h = _mix32(h ^ ((iy.astype(np.uint64) * np.uint64(0x165667B1)) & M32))
    h = _mix32(h ^ ((iz.astype(np.uint64) * np.uint64(0xD3A2646D)) & M32))
    return h >> np.uint64(16)


def smooth_weight(a, cell: int):
    """Q16 smoothstep weight of fraction (2a+1)/(2 cell)."""
    num = 2 * a.astype(np.int64) + 1
    den = 2 * cell
    return (num * num * (3 * den - 2 * num) * 65536) // (den * den * den)


def fbm_value(x, y, z, seed: int):
    """Integer fBm in [0, 31 * 65535] at integer voxel coordinates (broadcastable int64 arrays)."""
    total = np.zeros(np.broadcast(x, y, z).shape, dtype=np.int64)
    for o in range(5):
        cell = 64 >> o
        ix, ax = np.divmod(x, cell)
        iy, ay = np.divmod(y, cell)
        iz, az = np.divmod(z, cell)
        wx, wy, wz = smooth_weight(ax, cell), smooth_weight(ay, cell), smooth_weight(az, cell)

        def lv(dx, dy, dz):
            return lattice_value(ix + dx, iy + dy, iz + dz, o, seed).astype(np.int64)

        def lerp(a, b, w):
            return (a * (65536 - w) + b * w) >> 16

        x00 = lerp(lv(0, 0, 0), lv(1, 0, 0), wx)
        x10 = lerp(lv(0, 1, 0), lv(1, 1, 0), wx)
        x01 = lerp(lv(0, 0, 1), lv(1, 0, 1), wx)
        x11 = lerp(lv(0, 1, 1), lv(1, 1, 1), wx)
        y0 = lerp(x00, x10, wy)
        y1 = lerp(x01, x11, wy)
        total += lerp(y0, y1, wz) * (16 >> o)
    return total


PERMS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))


def primitives_scene(res: int, prims: list, shell: bool = True) -> np.ndarray:
    """Dense [z, y, x] grid of a primitive-union scene (tdag_primitive semantics, see include/tdag.h),
    optionally reduced to its 1-voxel surface shell (a solid voxel with a 6-neighbour outside, where
    voxels beyond the grid count as outside)."""
    inside = np.zeros((res, res, res), dtype=bool)  # [z, y, x]
    for p in prims:
        perm = PERMS[p["xform"] & 7]
        mirror = p["xform"] >> 3
        ext = [p["size"][perm[k]] for k in range(3)]
        lo = list(p["offset"])
        hi = [min(lo[k] + ext[k], res) for k in range(3)]
        if any(hi[k] <= lo[k] for k in range(3)):
            continue
        xs = np.arange(lo[0], hi[0]); ys = np.arange(lo[1], hi[1]); zs = np.arange(lo[2], hi[2])
        Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
        w = [X - lo[0], Y - lo[1], Z - lo[2]]
        for k in range(3):
            if (mirror >> k) & 1:
                w[k] = ext[k] - 1 - w[k]
        u = [None, None, None]
        for k in range(3):
            u[perm[k]] = w[k]
        if p["type"] == 0:
            m = np.ones(X.shape, bool)
        elif p["type"] == 1:
            r = p["radius"]
            m = (u[0] - r) ** 2 + (u[1] - r) ** 2 + (u[2] - r) ** 2 <= r * r
        else:
            s = p["size"][0]
            m = fbm_value(u[0].astype(np.int64), u[1].astype(np.int64), u[2].astype(np.int64), p["seed"]) * s > u[2].astype(np.int64) * 31 * 65535
        inside[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] |= m
    if not shell:
        return inside.astype(np.uint8)
    pad = np.pad(inside, 1, constant_values=False)
    allin = (pad[1:-1, 1:-1, :-2] & pad[1:-1, 1:-1, 2:] & pad[1:-1, :-2, 1:-1] & pad[1:-1, 2:, 1:-1]
             & pad[:-2, 1:-1, 1:-1] & pad[2:, 1:-1, 1:-1])
    return (inside & ~allin).astype(np.uint8)


def terrain(res: int, seed: int = 1) -> np.ndarray:
    """Config-0 grid: dense[z, y, x] uint8, solid where fBm - z/res > 0.

    Same definition as :func:`fbm_value`, evaluated with the lattice values of each octave
    precomputed once (a (res/cell + 2)^3 array) and gathered per voxel."""
    coords = np.arange(res, dtype=np.int64)
    total = np.zeros((res, res, res), dtype=np.int64)  # [z, y, x]
    for o in range(5):
        cell = 64 >> o
        nl = res // cell + 2
        li = np.arange(nl, dtype=np.int64)
        LZ, LY, LX = np.meshgrid(li, li, li, indexing="ij")
        lat = lattice_value(LX, LY, LZ, o, seed).astype(np.int64)  # [iz, iy, ix]
        i, a = np.divmod(coords, cell)
        w = smooth_weight(a, cell)

        def lerp(p, q, ww):
            return (p * (65536 - ww) + q * ww) >> 16

        # x interpolation -> [iz, iy, x]
        lx = lerp(lat[:, :, i], lat[:, :, i + 1], w[None, None, :])
        # y interpolation -> [iz, y, x]
        ly = lerp(lx[:, i, :], lx[:, i + 1, :], w[None, :, None])
        # z interpolation -> [z, y, x]
        lz = lerp(ly[i, :, :], ly[i + 1, :, :], w[:, None, None])
        total += lz * (16 >> o)
    zz = coords[:, None, None]
    return (total * res > zz * 31 * 65535).astype(np.uint8)
