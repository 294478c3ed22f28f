"""CPU model of the padded yz-quad brick layout and of the stencil's seven
loads (aloha_gb300/csrc/render.cu pad_brick_kernel, aloha_gb300/csrc/march.cuh
stencil / stencil_quads / axis_coord*): for coordinates across and beyond the
brick, every element the stencil addresses lies inside the padded array, and
the regrouped x rows hold exactly the clamped voxels the 20-voxel cross needs
(cudaAddressModeClamp, waikikiRenderer.cpp:753-755).  The GPU parity tests pin
the kernels themselves; this pins the index algebra without a GPU."""
import numpy as np
import pytest

APRON = 2


def padded_dims(n):
    nx, ny, nz = n
    px = ((nx + 2 * APRON) + 1) & ~1  # rows padded to an even number of quads
    return px, ny + 2 * APRON, nz + 2 * APRON


def pad_yz_quads(vol):
    """Element (x, y, z) of the padded array = V(x, y, z), V(x, y+1, z),
    V(x, y, z+1), V(x, y+1, z+1), indices clamped, apron of 2."""
    nz, ny, nx = vol.shape
    px, py, pz = padded_dims((nx, ny, nz))
    xs = np.clip(np.arange(px) - APRON, 0, nx - 1)
    ys = np.clip(np.arange(py) - APRON, 0, ny - 1)
    ys1 = np.clip(np.arange(py) + 1 - APRON, 0, ny - 1)
    zs = np.clip(np.arange(pz) - APRON, 0, nz - 1)
    zs1 = np.clip(np.arange(pz) + 1 - APRON, 0, nz - 1)
    out = np.empty((pz, py, px, 4), np.float32)
    out[..., 0] = vol[zs[:, None, None], ys[None, :, None], xs[None, None, :]]
    out[..., 1] = vol[zs[:, None, None], ys1[None, :, None], xs[None, None, :]]
    out[..., 2] = vol[zs1[:, None, None], ys[None, :, None], xs[None, None, :]]
    out[..., 3] = vol[zs1[:, None, None], ys1[None, :, None], xs[None, None, :]]
    return out


def axis(u, n, round_down):
    """axis_coord / axis_coord_floors: (i, c, h) in float32 arithmetic."""
    u = np.float32(u)
    m = np.float32(u - np.float32(0.5))
    if round_down:
        k = int(np.floor(u))
        fc = np.float32(k)
        h = bool(m < fc)
        c = min(max(k, -APRON), n)
        i = min(max(c - (1 if h else 0), -APRON), n - 1)
    else:
        fm, fc = np.floor(m), np.floor(u)
        h = bool(fc != fm)
        c = min(max(int(fc), -APRON), n)
        i = min(max(int(fm), -APRON), n - 1)
    return i, c, h


def clamped(vol, x, y, z):
    nz, ny, nx = vol.shape
    return vol[min(max(z, 0), nz - 1), min(max(y, 0), ny - 1), min(max(x, 0), nx - 1)]


@pytest.mark.parametrize("dims", [(5, 3, 4), (1, 1, 1), (2, 7, 1), (9, 8, 10)])
@pytest.mark.parametrize("round_down", [False, True])
def test_stencil_loads_stay_inside_and_fetch_the_cross(dims, round_down):
    nx, ny, nz = dims
    rng = np.random.default_rng(nx * 100 + ny * 10 + nz)
    vol = rng.random((nz, ny, nx), dtype=np.float32)
    q = pad_yz_quads(vol)
    px, py, pz = padded_dims(dims)
    edge = [-2.5, -1.0, -0.5, -1e-7, 0.0, 0.25, 0.5, 1e-7]
    coords = [(ux, uy, uz) for ux in edge + [nx - 0.5, nx + 1.5, nx + 40.0]
              for uy in edge[:4] + [ny - 0.25, ny + 3.0] for uz in edge[4:] + [nz - 1e-6, nz + 2.0]]
    coords += [tuple(rng.uniform(-3, np.array(dims) + 3)) for _ in range(300)]

    def elem(x, y, z):
        assert 0 <= x + APRON < px and 0 <= y + APRON < py and 0 <= z + APRON < pz, (x, y, z)
        return q[z + APRON, y + APRON, x + APRON]

    for ux, uy, uz in coords:
        ix, cx, hx = axis(ux, nx, round_down)
        iy, cy, hy = axis(uy, ny, round_down)
        iz, cz, hz = axis(uz, nz, round_down)
        ye = iy if hy else iy + 2
        ze = iz if hz else iz + 2
        q0, q1, q2 = elem(ix, cy, cz), elem(ix + 1, cy, cz), elem(ix + 2, cy, cz)
        e0, e1 = elem(cx, ye, cz), elem(cx + 1, ye, cz)
        f0, f1 = elem(cx, cy, ze)[:2], elem(cx + 1, cy, ze)[:2]
        # stencil_quads' regrouping into the x rows of stencil_rows
        rows = {(0, 0): (q0[0], q1[0], q2[0]), (1, 0): (q0[1], q1[1], q2[1]),
                (0, 1): (q0[2], q1[2], q2[2]), (1, 1): (q0[3], q1[3], q2[3])}
        for (j, l), got in rows.items():
            want = [clamped(vol, ix + k, cy + j, cz + l) for k in range(3)]
            assert list(got) == want
        assert [e0[0], e1[0], e0[2], e1[2]] == [clamped(vol, cx + k, ye, cz + l) for l in (0, 1) for k in (0, 1)]
        assert [f0[0], f1[0], f0[1], f1[1]] == [clamped(vol, cx + k, cy + j, ze) for j in (0, 1) for k in (0, 1)]


def test_round_down_coordinates_equal_the_floors():
    """axis_coord (one round-down conversion) and axis_coord_floors give the
    same indices, and the same weights, for every coordinate a sample inside
    a brick can have."""
    rng = np.random.default_rng(7)
    us = np.concatenate([rng.uniform(-3, 600, 20000).astype(np.float32),
                         np.float32([-2.5, -0.5, -1e-7, 0, 0.5, 1 - 2**-24, 1, 1.5, 255.5, 511.999])])
    for u in us:
        for n in (1, 7, 512):
            assert axis(u, n, True) == axis(u, n, False)
        m = np.float32(u - np.float32(0.5))
        k = int(np.floor(u))
        fc = np.float32(k)
        f_round = np.float32(m - (np.float32(fc - np.float32(1)) if m < fc else fc))
        assert f_round == np.float32(m - np.floor(m))
        assert np.float32(u - fc) == np.float32(u - np.floor(u))
