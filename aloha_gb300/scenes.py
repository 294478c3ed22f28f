"""Seeded synthetic scenes for the volume path: blob fields, transfer functions, cameras.

Inputs stand in for the reference's raw volumes (``volume.h`` reader,
``chopSuey.cpp`` bricks): no dataset ships with the reference, so every
workload is a seeded Gaussian-blob field with the documented shape.

Camera convention follows the viewer (``viewer.cpp:147-158``): the renderer
gets ``org``, ``dir_00`` (ray direction through the lower-left image corner),
and the per-pixel steps ``dir_du`` / ``dir_dv``; pixel (x, y) shoots through
``dir_00 + (x+.5) dir_du + (y+.5) dir_dv`` (``deviceCode.cpp:94-107``).
"""
from __future__ import annotations

import math

import numpy as np

# --------------------------------------------------------------- volumes


def blob_factors(dims, n_blobs: int, sigma_range, seed: int, centre_range=(0.2, 0.8)):
    """Per-axis Gaussian factors of `n_blobs` isotropic blobs (separable)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nx, ny, nz = (int(d) for d in dims)
    centres = rng.uniform(centre_range[0], centre_range[1], size=(n_blobs, 3))
    sigmas = rng.uniform(sigma_range[0], sigma_range[1], size=n_blobs)
    facs = []
    for a, n in enumerate((nx, ny, nz)):
        coord = np.arange(n, dtype=np.float64)[None, :]
        c = (centres[:, a] * (n - 1))[:, None]
        facs.append(np.exp(-((coord - c) ** 2) / (2.0 * sigmas[:, None] ** 2)))
    return facs  # [gx (b,nx), gy (b,ny), gz (b,nz)]


def blob_field(dims, n_blobs: int, sigma_range, seed: int, normalize: bool = True, device=None):
    """Sum of seeded Gaussian blobs, float32, shape (nz, ny, nx), x fastest.

    With ``normalize`` the field is divided by its maximum, so values lie in
    [0, 1] (the transfer function is indexed by the raw value,
    ``deviceCode.cpp:289``).  ``device`` = a torch device builds the field with
    a matmul on that device (used for the 512^3 and 1024^3 workloads).
    """
    gx, gy, gz = blob_factors(dims, n_blobs, sigma_range, seed)
    nx, ny, nz = gx.shape[1], gy.shape[1], gz.shape[1]
    if device is not None:
        import torch
        tgx = torch.from_numpy(gx.astype(np.float32)).to(device)
        tgy = torch.from_numpy(gy.astype(np.float32)).to(device)
        tgz = torch.from_numpy(gz.astype(np.float32)).to(device)
        zy = (tgz[:, :, None] * tgy[:, None, :]).reshape(n_blobs, nz * ny)  # (b, nz*ny)
        f = (zy.t() @ tgx).reshape(nz, ny, nx)
        if normalize:
            f = f / f.max()
        return f.contiguous()
    zy = (gz[:, :, None] * gy[:, None, :]).reshape(n_blobs, nz * ny).astype(np.float32)
    f = (zy.T @ gx.astype(np.float32)).reshape(nz, ny, nx)
    if normalize:
        f = f / f.max()
    return np.ascontiguousarray(f, dtype=np.float32)


def value_noise(dims, amplitude: float, seed: int, cell: int = 4):
    """Seeded lattice value noise (random values every `cell` voxels, trilinear in between)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nx, ny, nz = (int(d) for d in dims)
    lat = rng.uniform(-1.0, 1.0, size=(nz // cell + 2, ny // cell + 2, nx // cell + 2))

    def axis(n):
        p = np.arange(n) / cell
        i = np.floor(p).astype(np.int64)
        return i, p - i

    iz, fz = axis(nz)
    iy, fy = axis(ny)
    ix, fx = axis(nx)
    out = np.zeros((nz, ny, nx))
    for dz in (0, 1):
        wz = fz if dz else 1 - fz
        for dy in (0, 1):
            wy = fy if dy else 1 - fy
            for dx in (0, 1):
                wx = fx if dx else 1 - fx
                out += (wz[:, None, None] * wy[None, :, None] * wx[None, None, :] *
                        lat[(iz + dz)[:, None, None], (iy + dy)[None, :, None], (ix + dx)[None, None, :]])
    return (amplitude * out).astype(np.float32)


def quantize_u8(field: np.ndarray) -> np.ndarray:
    """Clamp to [0,1] and quantise to 0..255 (a raw uint8 volume)."""
    return np.round(np.clip(field, 0.0, 1.0) * 255.0).astype(np.uint8)


def normalize_raw(raw: np.ndarray) -> np.ndarray:
    """Volume::get's conversion (volume.h:75-88): uint8 /255, uint16 /65535, float as is."""
    from .volfile import normalize_raw as _normalize
    return _normalize(raw)


def plain_c1_volume(seed: int = 1):
    """64^3 uint8 volume: 8 blobs (sigma 4-10 voxels) + 0.05 value noise, quantised."""
    dims = (64, 64, 64)
    f = blob_field(dims, 8, (4.0, 10.0), seed, normalize=False)
    f = f + value_noise(dims, 0.05, seed + 1)
    return quantize_u8(f)


# ------------------------------------------------------ transfer functions


def ramp_tf(n: int = 256, alpha_lo: float = 0.2, alpha_max: float = 0.6, rgb_knots=None) -> np.ndarray:
    """Piecewise-linear RGBA table at x_i = i/(n-1): alpha 0 below `alpha_lo`,
    rising linearly to `alpha_max` at 1.0; RGB interpolated between knots."""
    x = np.arange(n, dtype=np.float64) / (n - 1)
    if rgb_knots is None:
        rgb_knots = [(0.0, (0.10, 0.20, 0.90)), (0.2, (0.20, 0.40, 0.95)), (0.5, (0.30, 0.90, 0.40)),
                     (0.8, (1.00, 0.70, 0.10)), (1.0, (1.00, 0.25, 0.10))]
    kx = np.array([k[0] for k in rgb_knots])
    rgb = np.stack([np.interp(x, kx, np.array([k[1][c] for k in rgb_knots])) for c in range(3)], axis=1)
    a = np.where(x < alpha_lo, 0.0, (x - alpha_lo) / (1.0 - alpha_lo) * alpha_max)
    return np.ascontiguousarray(np.concatenate([rgb, a[:, None]], axis=1), dtype=np.float32)


def seeded_tf(seed: int, n: int = 256) -> np.ndarray:
    """A second, seeded transfer function (random knots, different alpha ramp)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    knots = [(float(k), tuple(rng.uniform(0.05, 1.0, 3))) for k in (0.0, 0.25, 0.5, 0.75, 1.0)]
    return ramp_tf(n, alpha_lo=float(rng.uniform(0.15, 0.3)), alpha_max=float(rng.uniform(0.4, 0.7)),
                   rgb_knots=knots)


# ---------------------------------------------------------------- cameras


def look_at_camera(org, target, up, fovy_deg: float, W: int, H: int):
    """Pinhole camera -> (org, dir_00, dir_du, dir_dv) as float32 triples."""
    org = np.asarray(org, dtype=np.float64)
    f = np.asarray(target, dtype=np.float64) - org
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, dtype=np.float64))
    if np.linalg.norm(r) < 1e-12:
        r = np.cross(f, np.array([1.0, 0.0, 0.0]))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    h = 2.0 * math.tan(math.radians(fovy_deg) * 0.5)
    vertical = h * u
    horizontal = h * (W / H) * r
    lower_left = f - 0.5 * horizontal - 0.5 * vertical
    f32 = lambda v: np.asarray(v, dtype=np.float32)
    return f32(org), f32(lower_left), f32(horizontal / W), f32(vertical / H)


def axis_camera(dims, W: int, H: int, distance: float = 2.0, fovy: float = 45.0):
    """Camera on the +z axis at `distance` x extent from the centre, looking at it."""
    c = np.asarray(dims, dtype=np.float64) * 0.5
    ext = float(max(dims))
    return look_at_camera(c + np.array([0.0, 0.0, distance * ext]), c, (0.0, 1.0, 0.0), fovy, W, H)


def orbit_cameras(dims, n: int, W: int, H: int, seed: int, distance: float = 2.0, fovy: float = 45.0,
                  elevation_deg=(-60.0, 60.0)):
    """`n` seeded orbit cameras: azimuth U[0, 2pi), elevation U[-60, 60] deg, radius distance x extent."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = np.asarray(dims, dtype=np.float64) * 0.5
    ext = float(max(dims))
    cams = []
    for _ in range(n):
        az = rng.uniform(0.0, 2.0 * math.pi)
        el = math.radians(rng.uniform(*elevation_deg))
        d = np.array([math.cos(el) * math.sin(az), math.sin(el), math.cos(el) * math.cos(az)])
        cams.append(look_at_camera(c + distance * ext * d, c, (0.0, 1.0, 0.0), fovy, W, H))
    return cams


# ----------------------------------------------------------------- bricks


def grid_split(dims, cuts) -> list[dict]:
    """Bricks of an axis-aligned grid split with chopSuey's ghost rule
    (voxelRange = [cell.lo, min(cell.hi+1, dims)), chopSuey.cpp:302-313).
    `cuts` = interior cut positions per axis, e.g. ([200, 380], [256], [300])."""
    from .volfile import grid_split as _grid
    return _grid(dims, cuts)


def single_brick(dims) -> list[dict]:
    """One brick covering the whole volume (no ghost layer needed)."""
    return grid_split(dims, ([], [], []))


def extract_bricks(volume, descs):
    """Slice each brick's voxel range out of a (nz, ny, nx) volume and fill its value range."""
    out = []
    for d in descs:
        lo, hi = d["voxel_lo"], d["voxel_hi"]
        v = volume[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
        if hasattr(v, "contiguous"):
            v = v.contiguous()
            d["value_range"] = [float(v.min()), float(v.max())]
        else:
            v = np.ascontiguousarray(v, dtype=np.float32)
            d["value_range"] = [float(v.min()), float(v.max())]
        out.append(v)
    return out
