"""Seeded synthetic tilt series for the HAADF workloads (no dataset is shipped or needed).

Phantoms are unions of spheres / ellipsoids in the reconstruction frame (nm, origin at the
volume centre, x across the detector, y along the tilt axis, z along the beam at 0 deg).
Projections are exact parallel-beam line integrals of those shapes at detector pixel centres,
computed analytically, so the data are independent of the engine's own discrete A matrix.
Geometry conventions follow the reference: detector coordinate r = x cos(theta) - z sin(theta)
(Code/MBIRLib/Common/AMatrixCol.cpp:148), detector row t = y, pixel centres at
R0 + (j + 1/2) delta_r with R0 = -n_r delta_r / 2 (MRCSinogramInitializer.cpp:302-305).
"""
import struct

import numpy as np


def tilt_angles(max_deg, step_deg):
    n = int(round(2 * max_deg / step_deg)) + 1
    return np.linspace(-max_deg, max_deg, n).astype(np.float64)


def ellipsoid_projection(angles_deg, n_r, n_t, shapes, delta_r=1.0, delta_t=1.0):
    """Line integrals [theta][r][t] of ellipsoids.

    shapes: iterable of (cx, cy, cz, ax, ay, az, value); semi-axes aligned with x, y, z.
    """
    th = np.deg2rad(np.asarray(angles_deg, np.float64))
    r = -n_r * delta_r / 2 + (np.arange(n_r) + 0.5) * delta_r
    t = -n_t * delta_t / 2 + (np.arange(n_t) + 0.5) * delta_t
    out = np.zeros((len(th), n_r, n_t), np.float64)
    c, s = np.cos(th)[:, None, None], np.sin(th)[:, None, None]
    R = r[None, :, None]
    T = t[None, None, :]
    for (cx, cy, cz, ax, ay, az, val) in shapes:
        # ray: points p = (x, y, z) with x cos - z sin = r, y = t; direction d = (sin, 0, cos);
        # base point p0 = (r cos, t, -r sin).  Solve |M(p0 + s d - c0)|^2 = 1, M = diag(1/a).
        px, py, pz = R * c - cx, T - cy, -R * s - cz
        dx, dz = s, c
        A = (dx / ax) ** 2 + (dz / az) ** 2
        B = 2 * (px * dx / ax ** 2 + pz * dz / az ** 2)
        Cq = (px / ax) ** 2 + (py / ay) ** 2 + (pz / az) ** 2 - 1
        disc = B * B - 4 * A * Cq
        chord = np.where(disc > 0, np.sqrt(np.maximum(disc, 0)) / A, 0.0)
        out += val * chord
    return out


def two_sphere_shapes():
    """Two spheres of radius 20 and 12 voxels, values 1.0 and 0.5 (1 nm voxels)."""
    return [(-25.0, 0.0, 0.0, 20.0, 20.0, 20.0, 1.0), (30.0, 2.0, 6.0, 12.0, 12.0, 12.0, 0.5)]


def haadf_measurements(proj, seed=0, gain_jitter=0.05, offset=0.1, var_scale=0.05,
                       var_floor=1e-3):
    """y = g_k * proj + d_k + N(0, var_scale*|signal| + var_floor), g_k = 1 +- U(gain_jitter)."""
    rng = np.random.default_rng(seed)
    n_theta = proj.shape[0]
    g = 1.0 + rng.uniform(-gain_jitter, gain_jitter, n_theta)
    sig = g[:, None, None] * proj
    noise = rng.standard_normal(proj.shape) * np.sqrt(var_scale * np.abs(sig) + var_floor)
    return (sig + offset + noise).astype(np.float32), g


def haadf_two_spheres(n_r=128, n_t=32, max_deg=70.0, step_deg=2.0, seed=0):
    """The small HAADF case: 128 x 32 detector, +-70 deg in 2 deg steps (71 views)."""
    ang = tilt_angles(max_deg, step_deg)
    proj = ellipsoid_projection(ang, n_r, n_t, two_sphere_shapes())
    y, g = haadf_measurements(proj, seed=seed)
    return y, ang.astype(np.float32), g


def particles_on_slab(n_r=512, n_t=256, thickness=64.0, max_deg=60.0, step_deg=2.0,
                      n_particles=200, slab=(-0.75, -0.5), slab_value=0.1, seed=0):
    """Nanoparticles on a substrate: `n_particles` random ellipsoids (semi-axes 3-15 voxels,
    values U(0.5, 2.0)) above a slab of value `slab_value` spanning x and y.  The sample is
    `thickness` nm thick (the engine's volume is 2x that along z).  Returns (y, angles, gains).
    The slab's 1% texture of the workload description is not modelled by the analytic
    projection."""
    ang = tilt_angles(max_deg, step_deg)
    lz = 2 * thickness
    z0, z1 = slab[0] * lz / 2, slab[1] * lz / 2
    shapes = random_ellipsoids(n_particles, n_r, n_t, lz, seed=seed, z_range=(z1, lz / 2))
    proj = np.zeros((len(ang), n_r, n_t), np.float64)
    t = -n_t / 2 + np.arange(n_t) + 0.5
    for s in shapes:
        rows = np.nonzero(np.abs(t - s[1]) < s[4])[0]
        if len(rows) == 0:
            continue
        lo, hi = rows[0], rows[-1] + 1
        # project onto the detector rows the particle covers only: a sub-detector of hi-lo rows
        # centred at offset in the full frame
        offset = -n_t / 2 + lo + (hi - lo) / 2
        sub = (s[0], s[1] - offset, s[2], s[3], s[4], s[5], s[6])
        proj[:, :, lo:hi] += ellipsoid_projection(ang, n_r, hi - lo, [sub])
    proj += slab_value * (z1 - z0) / np.cos(np.deg2rad(ang))[:, None, None]
    y, g = haadf_measurements(proj, seed=seed + 1)
    return y, ang.astype(np.float32), g


def bf_counts(proj, dose=1.0e4, drift=0.03, atten=0.02, seed=0):
    """Bright-field raw counts: Poisson(dose * d_k * exp(-atten * proj)) with a per-view dose
    drift d_k = 1 +- U(drift).  `proj` holds line integrals of the phantom's values; `atten`
    turns them into attenuation (the phantom values U(0.5, 2.0) per voxel times 0.02 keep the
    thickest particle stacks at a few percent transmission).  Returns (counts float32, d)."""
    rng = np.random.default_rng(seed)
    d = 1.0 + rng.uniform(-drift, drift, proj.shape[0])
    lam = dose * d[:, None, None] * np.exp(-atten * proj)
    counts = rng.poisson(lam).astype(np.float32)
    return np.maximum(counts, 1.0), d


def bf_particles_on_slab(n_r=512, n_t=256, thickness=64.0, max_deg=60.0, step_deg=2.0,
                         n_particles=200, slab=(-0.75, -0.5), slab_value=0.1, seed=0,
                         dose=1.0e4):
    """The bright-field workload: the particles-on-slab phantom of particles_on_slab seen as
    Poisson counts at `dose` electrons with +-3% per-view drift.  Returns (counts, angles)."""
    ang = tilt_angles(max_deg, step_deg)
    lz = 2 * thickness
    z0, z1 = slab[0] * lz / 2, slab[1] * lz / 2
    shapes = random_ellipsoids(n_particles, n_r, n_t, lz, seed=seed, z_range=(z1, lz / 2))
    proj = np.zeros((len(ang), n_r, n_t), np.float64)
    t = -n_t / 2 + np.arange(n_t) + 0.5
    for s in shapes:
        rows = np.nonzero(np.abs(t - s[1]) < s[4])[0]
        if len(rows) == 0:
            continue
        lo, hi = rows[0], rows[-1] + 1
        offset = -n_t / 2 + lo + (hi - lo) / 2
        sub = (s[0], s[1] - offset, s[2], s[3], s[4], s[5], s[6])
        proj[:, :, lo:hi] += ellipsoid_projection(ang, n_r, hi - lo, [sub])
    proj += slab_value * (z1 - z0) / np.cos(np.deg2rad(ang))[:, None, None]
    counts, _ = bf_counts(proj, dose=dose, seed=seed + 1)
    return counts, ang.astype(np.float32)


def particles_on_slab_volume(n_x, n_y, n_z, thickness, n_particles, slab=(-0.75, -0.5),
                             slab_value=0.1, seed=0):
    """The particles-on-slab phantom of particles_on_slab voxelised on the engine's grid (1 nm
    voxels; the volume is 2 x thickness along z, centred): float32 [z][x][y].  Each voxel whose
    centre lies inside an ellipsoid takes the ellipsoid's value (summed where they overlap)."""
    lz = 2 * thickness
    vol = np.zeros((n_z, n_x, n_y), np.float32)
    zc = -n_z / 2 + np.arange(n_z) + 0.5
    xc = -n_x / 2 + np.arange(n_x) + 0.5
    yc = -n_y / 2 + np.arange(n_y) + 0.5
    z0, z1 = slab[0] * lz / 2, slab[1] * lz / 2
    vol[(zc >= z0) & (zc < z1)] = slab_value
    shapes = random_ellipsoids(n_particles, n_x, n_y, lz, seed=seed, z_range=(z1, lz / 2))
    for cx, cy, cz, ax, ay, az, val in shapes:
        iz = np.nonzero(np.abs(zc - cz) <= az)[0]
        ix = np.nonzero(np.abs(xc - cx) <= ax)[0]
        iy = np.nonzero(np.abs(yc - cy) <= ay)[0]
        if len(iz) == 0 or len(ix) == 0 or len(iy) == 0:
            continue
        Z, X, Y = np.ix_(zc[iz], xc[ix], yc[iy])
        m = ((X - cx) / ax) ** 2 + ((Y - cy) / ay) ** 2 + ((Z - cz) / az) ** 2 <= 1.0
        sub = vol[iz[0]:iz[-1] + 1, ix[0]:ix[-1] + 1, iy[0]:iy[-1] + 1]
        sub[m] += np.float32(val)
    return vol


def random_ellipsoids(n, extent_x, extent_y, extent_z, seed=0, axes=(3.0, 15.0),
                      values=(0.5, 2.0), z_range=None):
    rng = np.random.default_rng(seed)
    zlo, zhi = z_range if z_range is not None else (-extent_z / 2, extent_z / 2)
    shapes = []
    for _ in range(n):
        a = rng.uniform(axes[0], axes[1], 3)
        a[2] = min(a[2], (zhi - zlo) / 2 - 0.5)
        cx = rng.uniform(-extent_x / 2 + a[0], extent_x / 2 - a[0])
        cy = rng.uniform(-extent_y / 2, extent_y / 2)
        cz = rng.uniform(zlo + a[2], zhi - a[2])
        shapes.append((cx, cy, cz, a[0], a[1], a[2], rng.uniform(*values)))
    return shapes


def write_tilt_series_mrc(path, counts_trt, tilts_deg, pixel_size_nm=1.0, mode=2,
                          label="Fei Company (C) Copyright 2003"):
    """Write counts[theta][r][t] as an MRC stack (sections = views, x = r, y = t) with an FEI
    extended header carrying a_tilt, b_tilt = -a_tilt and the pixel size (metres)."""
    n_theta, n_r, n_t = counts_trt.shape
    h = bytearray(1024)
    struct.pack_into("<4i", h, 0, n_r, n_t, n_theta, mode)
    struct.pack_into("<3i", h, 28, n_r, n_t, n_theta)
    struct.pack_into("<3f", h, 40, float(n_r), float(n_t), float(n_theta))
    struct.pack_into("<3f", h, 52, 90.0, 90.0, 90.0)
    struct.pack_into("<3i", h, 64, 1, 2, 3)
    struct.pack_into("<i", h, 92, 128 * n_theta)
    h[208:212] = b"MAP "
    h[212:214] = bytes([68, 65])
    struct.pack_into("<i", h, 220, 1)
    lab = label.encode()[:80]
    h[224:224 + len(lab)] = lab
    ext = bytearray(128 * n_theta)
    for k in range(n_theta):
        struct.pack_into("<2f", ext, 128 * k, float(tilts_deg[k]), -float(tilts_deg[k]))
        struct.pack_into("<f", ext, 128 * k + 44, float(pixel_size_nm) * 1e-9)
    data = np.ascontiguousarray(np.transpose(counts_trt, (0, 2, 1)))  # [z][y][x]
    if mode == 2:
        data = data.astype("<f4")
    elif mode == 1:
        data = np.round(data).astype("<i2")
    elif mode == 6:
        data = np.round(data).astype("<u2")
    else:
        raise ValueError("mode must be 1, 2 or 6")
    with open(path, "wb") as f:
        f.write(bytes(h))
        f.write(bytes(ext))
        f.write(data.tobytes())


def read_mrc_volume(path):
    """Read a float32 MRC volume written by the engine: returns (header ints, data [z][y][x])."""
    with open(path, "rb") as f:
        h = f.read(1024)
        nx, ny, nz, mode = struct.unpack_from("<4i", h, 0)
        nxt = struct.unpack_from("<i", h, 92)[0]
        f.read(nxt)
        data = np.frombuffer(f.read(4 * nx * ny * nz), "<f4").reshape(nz, ny, nx)
    amin, amax, amean = struct.unpack_from("<3f", h, 76)
    return dict(nx=nx, ny=ny, nz=nz, mode=mode, next=nxt, amin=amin, amax=amax, amean=amean,
                label0=h[224:304].split(b"\0")[0].decode()), data
