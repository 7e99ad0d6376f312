"""Seeded synthetic inputs: cylinder and random-ellipsoid phantoms, helix rays, Poisson data.

The reference's demos use toolbox phantoms (``phantom``/Shepp-Logan) that are not
available here; these seeded generators stand in for them with the shapes, sizes and
value distributions of the workloads this library is measured on.  All arrays are
float32, MATLAB column-major (``order='F'``): volume index ``x + W*y + W*W*z``.
"""
from __future__ import annotations

import numpy as np


def centred_grid(n: int) -> np.ndarray:
    """Voxel-centre coordinates -(n-1)/2 ... (n-1)/2 (the reference's world frame)."""
    return np.arange(n, dtype=np.float64) - (n - 1) / 2.0


def cylinder(W: int, H: int | None = None, radius: float = 47.0, value: float = 0.02,
             inclusive: bool = True) -> np.ndarray:
    """Uniform cylinder along z: voxels with x^2+y^2 <= radius^2 set to ``value``."""
    H = W if H is None else H
    c = centred_grid(W)
    x, y = np.meshgrid(c, c, indexing="ij")
    r2 = x * x + y * y
    mask = (r2 <= radius * radius) if inclusive else (r2 < radius * radius)
    sl = np.where(mask, np.float32(value), np.float32(0)).astype(np.float32)
    return np.asfortranarray(np.repeat(sl[:, :, None], H, axis=2))


def _random_rotation(rng: np.random.Generator) -> np.ndarray:
    # Uniform rotation from a uniform unit quaternion (Shoemake 1992).
    u1, u2, u3 = rng.random(3)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    q = np.array([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                  b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)])
    x, y, z, w = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def ellipsoid_params(n: int, count: int, seed: int, axes=(10.0, 150.0), values=(-0.01, 0.03),
                     inner: float = 0.70):
    """Seeded ellipsoid list: (centre[3], semi_axes[3], rotation[3,3], value).

    Centres are uniform in the inner ``inner`` fraction of the field of view, semi-axes
    uniform in ``axes`` voxels (capped at the volume half-size for small volumes), uniform
    random 3D rotations, additive values uniform in ``values``."""
    rng = np.random.default_rng(seed)
    lo, hi = axes
    hi = min(hi, n / 2.0)
    lo = min(lo, hi)
    out = []
    half = inner * n / 2.0
    for _ in range(count):
        c = rng.uniform(-half, half, size=3)
        a = rng.uniform(lo, hi, size=3)
        R = _random_rotation(rng)
        v = rng.uniform(values[0], values[1])
        out.append((c, a, R, float(v)))
    return out


def ellipsoids(n: int, count: int = 12, seed: int = 0, nz: int | None = None, **kw) -> np.ndarray:
    """Random-ellipsoid phantom [n, n, nz] float32, additive values clipped at 0."""
    nz = n if nz is None else nz
    vol = np.zeros((n, n, nz), dtype=np.float32, order="F")
    cx, cz = centred_grid(n), centred_grid(nz)
    for c, a, R, v in ellipsoid_params(n, count, seed, **kw):
        # Axis-aligned half extents of the rotated ellipsoid.
        r = np.sqrt(((R * a[None, :]) ** 2).sum(axis=1))
        lo = [int(np.clip(np.floor(c[i] - r[i] + (n - 1) / 2.0), 0, n)) for i in range(2)]
        hi = [int(np.clip(np.ceil(c[i] + r[i] + (n - 1) / 2.0) + 1, 0, n)) for i in range(2)]
        lz = int(np.clip(np.floor(c[2] - r[2] + (nz - 1) / 2.0), 0, nz))
        hz = int(np.clip(np.ceil(c[2] + r[2] + (nz - 1) / 2.0) + 1, 0, nz))
        if lo[0] >= hi[0] or lo[1] >= hi[1] or lz >= hz:
            continue
        X = cx[lo[0]:hi[0]][:, None] - c[0]
        Y = cx[lo[1]:hi[1]][None, :] - c[1]
        inv = 1.0 / (a * a)
        # q(p) = sum_k (R^T p)_k^2 / a_k^2 = p^T M p with M = R diag(1/a^2) R^T
        M = (R * inv) @ R.T
        for k0 in range(lz, hz, 64):
            k1 = min(hz, k0 + 64)
            Z = cz[k0:k1][None, None, :] - c[2]
            q = (M[0, 0] * X[:, :, None] ** 2 + M[1, 1] * Y[:, :, None] ** 2 + M[2, 2] * Z ** 2
                 + 2 * M[0, 1] * X[:, :, None] * Y[:, :, None]
                 + 2 * M[0, 2] * X[:, :, None] * Z + 2 * M[1, 2] * Y[:, :, None] * Z)
            sub = vol[lo[0]:hi[0], lo[1]:hi[1], k0:k1]
            sub += np.where(q <= 1.0, np.float32(v), np.float32(0))
    np.maximum(vol, 0, out=vol)
    return vol


def angles_full(n_views: int, turns: float = 1.0) -> np.ndarray:
    """float32 linspace(0, 2*pi*turns, n_views) as MATLAB's single(linspace(...))."""
    return np.linspace(0.0, 2.0 * np.pi * turns, n_views).astype(np.float32)


def parallel_pts(W: int, H: int, L: float = 1000.0) -> np.ndarray:
    """Parallel rays along x as a general3D points array [W,H,6] (x1,y1,z1,x2,y2,z2)."""
    y = (np.arange(W) - (W - 1) / 2.0)[:, None].repeat(H, axis=1)
    z = (np.arange(H) - (H - 1) / 2.0)[None, :].repeat(W, axis=0)
    pts = np.zeros((W, H, 6), dtype=np.float32, order="F")
    pts[:, :, 0] = -L
    pts[:, :, 1] = y
    pts[:, :, 2] = z
    pts[:, :, 3] = L
    pts[:, :, 4] = y
    pts[:, :, 5] = z
    return pts


def helix_pts(W: int, H: int, n_views: int, nz: int, sad: float = 1000.0, turns: float = 2.0,
              pitch: float = 1.0, seed: int = 0, jitter: float = 0.05, views=None):
    """Cone-beam helix as per-view general3D points [W,H,6,nP] plus the view angles.

    The source sits at radius ``sad`` and advances ``pitch*nz`` voxels in z per turn; the
    flat detector sits ``sad`` behind the axis with unit pixels magnified by 2; the points
    are given in the un-rotated frame (the kernels rotate them by each view angle about z).
    Seeded jitter of the end points avoids perfectly regular rays.  ``views`` (sorted
    indices) returns only those views of the ``n_views`` helix, with the same values."""
    rng = np.random.default_rng(seed)
    ang = angles_full(n_views, turns)
    zsrc = (np.arange(n_views) / max(n_views - 1, 1) - 0.5) * turns * pitch * nz
    u = (np.arange(W) - (W - 1) / 2.0)[:, None] * 2.0
    v = (np.arange(H) - (H - 1) / 2.0)[None, :] * 2.0
    keep = list(range(n_views)) if views is None else [int(j) for j in views]
    slot = {j: i for i, j in enumerate(keep)}
    pts = np.zeros((W, H, 6, len(keep)), dtype=np.float32, order="F")
    for j in range(n_views):
        ju = rng.uniform(-jitter, jitter, size=(W, H))
        jv = rng.uniform(-jitter, jitter, size=(W, H))
        if j not in slot:
            continue
        i = slot[j]
        pts[:, :, 0, i] = sad
        pts[:, :, 1, i] = 0.0
        pts[:, :, 2, i] = zsrc[j]
        pts[:, :, 3, i] = -sad
        pts[:, :, 4, i] = u + ju
        pts[:, :, 5, i] = zsrc[j] + v + jv
    return pts, ang[keep]


def poisson_counts(fp: np.ndarray, i0: float = 1e5, seed: int = 0):
    """pre = I0, post = Poisson(I0 * exp(-fp)) as float32 (counts, not log)."""
    rng = np.random.default_rng(seed)
    pre = np.full(fp.shape, np.float32(i0), dtype=np.float32, order="F")
    lam = i0 * np.exp(-np.asarray(fp, dtype=np.float64))
    post = np.asfortranarray(rng.poisson(lam).astype(np.float32))
    return pre, post
