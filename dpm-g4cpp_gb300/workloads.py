"""Synthetic workloads (phantoms, sources, job lists) of the benchmark and test
configurations. Material ids refer to data sets whose materials are
[0] water, [1] lung, [2] compact bone (data/water_lung_bone) unless noted.
255 is vacuum.
"""
import math

import numpy as np

from . import Job, Phantom, Source

WATER, LUNG, BONE = 0, 1, 2
AIR = 3          # data/water_lung_bone_air only
VACUUM = 255
MEV_TO_J = 1.602176634e-13


def voxel_centres(n, v, origin):
    return origin + (np.arange(n) + 0.5) * v


def precision_phantom(nx=128, ny=128, nz=256, v=2.0, lung=(60.0, 120.0), bone_r=15.0, bone_xz=(0.0, 180.0)):
    """Water body, a lung slab z in [60,120) mm and a compact-bone cylinder of
    radius 15 mm along y with its axis at x = 0, z = 180 mm (128x128x256 x 2 mm).
    Axes: x in [-nx v/2, nx v/2], y likewise, z in [0, nz v]."""
    x = voxel_centres(nx, v, -0.5 * nx * v)
    z = voxel_centres(nz, v, 0.0)
    m = np.full((nz, ny, nx), WATER, dtype=np.uint8)
    m[(z >= lung[0]) & (z < lung[1]), :, :] = LUNG
    zz, xx = np.meshgrid(z, x, indexing="ij")
    cyl = (xx - bone_xz[0]) ** 2 + (zz - bone_xz[1]) ** 2 < bone_r ** 2
    m[:, :, :][np.broadcast_to(cyl[:, None, :], m.shape)] = BONE
    return m


def precision_source(e0=1.0, e1=20.0, field=100.0):
    """10x10 cm2 broad photon beam, energy uniform on [1, 20] MeV."""
    return Source(particle=0, spectrum=1, e0=e0, e1=e1, shape=1, cx=0.0, cy=0.0, fx=field, fy=field)


def _ellipsoid(shape, v, centre, semi):
    nz, ny, nx = shape
    x = voxel_centres(nx, v, -0.5 * nx * v)
    y = voxel_centres(ny, v, -0.5 * ny * v)
    z = voxel_centres(nz, v, 0.0)
    zz, yy, xx = np.meshgrid(z, y, x, indexing="ij")
    return ((xx - centre[0]) / semi[0]) ** 2 + ((yy - centre[1]) / semi[1]) ** 2 + ((zz - centre[2]) / semi[2]) ** 2 < 1


def batching_job_spec(i, v=2.0, hist_range=(1e5, 1e7), scale=1.0):
    """Job i of the batching workload, drawn from seed i: a cubic phantom with
    edge in {32,64,96,128,192} voxels of v mm (water base), 3 ellipsoidal
    inserts of a random material (water/lung/bone), an electron or photon beam
    (p = 0.5) of a monoenergetic energy uniform in [4, 20] MeV covering the
    central half of the entry face, and a history count log-uniform in
    hist_range (times `scale`). Returns (mat[nz,ny,nx], Source, histories)."""
    rng = np.random.default_rng(i)
    edge = int(rng.choice([32, 64, 96, 128, 192]))
    shape = (edge, edge, edge)
    m = np.full(shape, WATER, dtype=np.uint8)
    L = edge * v
    for _ in range(3):
        mat = int(rng.integers(0, 3))
        centre = (rng.uniform(-0.3, 0.3) * L, rng.uniform(-0.3, 0.3) * L, rng.uniform(0.2, 0.8) * L)
        semi = tuple(rng.uniform(0.05, 0.25) * L for _ in range(3))
        m[_ellipsoid(shape, v, centre, semi)] = mat
    particle = -1 if rng.random() < 0.5 else 0
    energy = float(rng.uniform(4.0, 20.0))
    hist = int(round(math.exp(rng.uniform(math.log(hist_range[0]), math.log(hist_range[1]))) * scale))
    src = Source(particle=particle, spectrum=0, e0=energy, e1=energy, shape=1, fx=0.5 * L, fy=0.5 * L)
    return m, src, max(1, hist)


def batching_jobs(tables, njobs=64, v=2.0, hist_range=(1e5, 1e7), scale=1.0):
    """The 64 independent jobs of the batching workload (batching_job_spec),
    job i with seed i. Returns (jobs, phantoms)."""
    jobs, phantoms = [], []
    for i in range(njobs):
        m, src, hist = batching_job_spec(i, v, hist_range, scale)
        ph = Phantom.voxels(tables, m, v)
        phantoms.append(ph)
        jobs.append(Job(ph, src, hist, seed=i))
    return jobs, phantoms


def differentiation_setup(seed=4, n=128, v=2.0):
    """128^3 x 2 mm water phantom with a bone block and a lung block at seeded
    positions, a 20x20 grid of 5x5 mm2 6 MeV photon beamlets, and the target
    dose (2 Gy in a central 30 mm sphere, 0 elsewhere). Returns
    (mat, source, target[nz,ny,nx])."""
    rng = np.random.default_rng(seed)
    m = np.full((n, n, n), WATER, dtype=np.uint8)
    for mat in (BONE, LUNG):
        size = rng.integers(max(2, n // 13), max(3, n // 5), size=3)   # 10-25 voxels at n = 128
        lo = [int(rng.integers(n // 25, n - n // 25 - s)) for s in size]
        m[lo[2]:lo[2] + size[2], lo[1]:lo[1] + size[1], lo[0]:lo[0] + size[0]] = mat
    src = Source(particle=0, spectrum=0, e0=6.0, e1=6.0, shape=2, cx=0.0, cy=0.0, fx=5.0, fy=5.0, nbx=20, nby=20)
    x = voxel_centres(n, v, -0.5 * n * v)
    z = voxel_centres(n, v, 0.0)
    zz, yy, xx = np.meshgrid(z, x, x, indexing="ij")
    target = np.where(xx ** 2 + yy ** 2 + (zz - 0.5 * n * v) ** 2 < 15.0 ** 2, 2.0, 0.0)
    return m, src, target


def full_scale_phantom(seed=99, nx=512, ny=512, nz=256, v=1.0, outside=AIR):
    """Synthetic CT-like phantom (512x512x256 x 1 mm): an elliptical water body
    (semi-axes 180 mm in x and 120 mm in z, long axis along y), two lung
    ellipsoids, a bone spine cylinder along y and a bone rib shell; air (of the
    water/lung/bone/air data set) outside the body. The beam enters along +z
    (anterior face) through the air gap. Vacuum voxels would end every track
    that reaches them, as in the reference's transport, so they are not used
    around the body."""
    rng = np.random.default_rng(seed)
    x = voxel_centres(nx, v, -0.5 * nx * v)
    y = voxel_centres(ny, v, -0.5 * ny * v)
    z = voxel_centres(nz, v, 0.0)
    zc = 0.5 * nz * v
    zz, xx = np.meshgrid(z, x, indexing="ij")
    ell = (xx / 180.0) ** 2 + ((zz - zc) / 120.0) ** 2
    body = ell < 1.0
    ribs = (ell > 0.80) & (ell < 0.86)
    sl = np.where(body, WATER, outside).astype(np.uint8)
    m = np.repeat(sl[:, None, :], ny, axis=1)
    thorax = (y > -120.0 + rng.uniform(-10, 10)) & (y < 120.0 + rng.uniform(-10, 10))
    rib_mask = np.broadcast_to(ribs[:, None, :], m.shape) & thorax[None, :, None]
    m[rib_mask] = BONE
    for sx in (-1.0, 1.0):
        cx = sx * rng.uniform(60.0, 80.0)
        lung = _ellipsoid(m.shape, v, (cx, rng.uniform(-10, 10), zc), (rng.uniform(45, 55), rng.uniform(90, 110),
                                                                      rng.uniform(60, 75)))
        m[lung & (m != outside)] = LUNG
    spine = (xx ** 2 + (zz - (zc + 85.0)) ** 2) < 15.0 ** 2
    m[np.broadcast_to(spine[:, None, :], m.shape)] = BONE
    return m


def full_scale_source():
    """10x10 cm2 photon beam, p(E) ~ (20 - E) on [0.5, 20] MeV."""
    return Source(particle=0, spectrum=2, e0=0.5, e1=20.0, shape=1, cx=0.0, cy=0.0, fx=100.0, fy=100.0)


def dose_gy(edep_mev, mat, densities, voxel_mm3, histories=1):
    """Energy per voxel [MeV] -> dose per history [Gy] (vacuum voxels: 0)."""
    rho = np.zeros(256)
    rho[:len(densities)] = densities
    mass_kg = rho[mat] * voxel_mm3 * 1.0e-6   # g/cm3 * mm3 -> kg
    with np.errstate(divide="ignore", invalid="ignore"):
        d = np.where(mass_kg > 0, edep_mev * MEV_TO_J / mass_kg, 0.0)
    return d / histories
