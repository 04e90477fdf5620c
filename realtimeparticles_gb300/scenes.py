"""Seeded synthetic scenes for the benchmark and test configurations.

The reference initialises its cases from unseeded lattices (utils/Geometry.cpp:40-69,
Fluids.cpp:273-398, Boids.cpp:277-321); these generators produce the configurations the
GB300 build is measured on, from a seed, with numpy's PCG64:

* fluids dam break: a jittered cubic lattice of spacing d in a unit box (W = 0.5),
  h = 2d, packed against the low corner of the reference's asymmetric wall clamp
  [-W + 0.01, W - 0.1] (fluids.cl:435-439);
* boids: positions uniform in [-W, W]^3, velocities of uniform random direction and
  speed uniform in [0.5, 1.0] x velocityScale;
* clouds: particles uniform in the lower quarter of a 1 x 2 x 1 box (the reference's
  Cumulus case, Clouds.cpp:451-456, scaled to unit width), with a value-noise ground
  temperature field.
"""
import math

import numpy as np

from . import abi

PI_F = np.float32(3.1415927)


def lattice_rest_density(d, h):
    """Interior SPH density (unit mass) of a cubic lattice of spacing d under poly6
    (sph.cl:10-14): sum over lattice points within h, in double precision."""
    coeff = 315.0 / (64.0 * math.pi * h ** 9)
    m = int(math.ceil(h / d)) + 1
    rho = 0.0
    for i in range(-m, m + 1):
        for j in range(-m, m + 1):
            for k in range(-m, m + 1):
                r2 = (i * i + j * j + k * k) * d * d
                if r2 < h * h:
                    rho += coeff * (h * h - r2) ** 3
    return rho


def fluid_params(rest_density, dt=1.0 / 240.0, eps=600.0, k=0.1, n=4, dq=0.2, xsph=0.01, vort=0.0005):
    """FluidKernelInputs (physics/ocl/Fluids.hpp:17-32) of the dam-break configurations;
    dt is one substep (1/120 s frame, 2 substeps).

    k (s_corr), xsph (c) and vort (epsilon) are given as in Macklin & Mueller 2013, whose
    neighbour sums carry the mass/density factor m / rho_j ~ 1 / rho0.  The reference
    kernels sum with unit mass and no density factor (fluids.cl:240, 317, 369, 422), so the
    coefficients passed to them are divided by rho0.  Taken literally (k = 0.1, c = 0.01
    at rho0 ~ 5e5), the dam break diverges within one step."""
    p = abi.FluidParams()
    p.restDensity = float(rest_density)
    p.relaxCFM = float(eps)
    p.timeStep = float(dt)
    p.dim = 3
    p.isArtPressureEnabled = 1
    p.artPressureRadius = float(dq)
    p.artPressureCoeff = float(k) / float(rest_density)
    p.artPressureExp = int(n)
    p.isVorticityConfEnabled = 1
    p.vorticityConfCoeff = float(vort) / float(rest_density)
    p.xsphViscosityCoeff = float(xsph) / float(rest_density)
    return p


def dam_break(lattice=(16, 32, 32), d=0.0125, box=1.0, jitter=0.01, seed=0, max_n=None):
    """Jittered dam-break lattice: returns dict(pos, vel, model_params, fluid_params).

    lattice = (nx, ny, nz) particles along x, y, z; spacing d; the box is `box` wide in
    every axis with grid cell h = 2d.  Positions start half a spacing above the clamp
    floor -W + 0.01."""
    nx, ny, nz = lattice
    n = nx * ny * nz
    h = 2.0 * d
    W = box / 2.0
    res = int(round(box / h))
    lo = -W + 0.01
    rng = np.random.default_rng(seed)
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    pos = np.zeros((n, 4), np.float32)
    base = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    xyz = lo + (base + 0.5) * d + rng.uniform(-jitter * d, jitter * d, size=(n, 3))
    pos[:, :3] = xyz.astype(np.float32)
    vel = np.zeros((n, 4), np.float32)
    mp = abi.model_params(n, max_n or n, (box, box, box), (res, res, res), 3, abi.CASE_FLUIDS_DAM)
    fp = fluid_params(lattice_rest_density(d, h))
    return {"pos": pos, "vel": vel, "model_params": mp, "fluid_params": fp, "h": h, "d": d}


def boids_params(velocity=1.0, align=1.0, coh=0.8, sep=1.5):
    p = abi.BoidsParams()
    p.velocityScale = float(velocity)
    p.alignmentScale = float(align)
    p.separationScale = float(sep)
    p.cohesionScale = float(coh)
    return p


def boids_cloud(n=131072, box=2.0, radius=0.05, speed=(0.5, 1.0), seed=0, max_n=None, velocity=1.0):
    """Boids: uniform positions in [-W, W]^3, uniform random directions, speeds uniform
    in `speed` (times velocityScale); grid cell = neighbour radius."""
    rng = np.random.default_rng(seed)
    W = box / 2.0
    res = int(round(box / radius))
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(-W, W, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    s = rng.uniform(speed[0], speed[1], size=(n, 1)) * velocity
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = (d * s).astype(np.float32)
    mp = abi.model_params(n, max_n or n, (box, box, box), (res, res, res), 3, abi.CASE_BOIDS_XLARGE,
                          velocity=velocity)
    return {"pos": pos, "vel": vel, "model_params": mp, "boids_params": boids_params(velocity)}


def value_noise_2d(nx, nz, octaves=8, amplitude=3.0, base=300.0, seed=0):
    """Seeded 2D value noise on an nx x nz table: octave o samples a random lattice of
    2^(o+1) cells per side, smoothstep-interpolated, weight 2^-o; the sum is scaled to
    +-amplitude around base."""
    rng = np.random.default_rng(seed)
    u = np.linspace(0.0, 1.0, nx)
    v = np.linspace(0.0, 1.0, nz)
    total = np.zeros((nx, nz))
    for o in range(octaves):
        cells = 2 ** (o + 1)
        lat = rng.uniform(-1.0, 1.0, size=(cells + 1, cells + 1))
        fu = u * cells
        fv = v * cells
        i0 = np.minimum(np.floor(fu).astype(int), cells - 1)
        k0 = np.minimum(np.floor(fv).astype(int), cells - 1)
        tu = fu - i0
        tv = fv - k0
        su = tu * tu * (3 - 2 * tu)
        sv = tv * tv * (3 - 2 * tv)
        a = lat[np.ix_(i0, k0)]
        b = lat[np.ix_(i0, k0 + 1)]
        c = lat[np.ix_(i0 + 1, k0)]
        dd = lat[np.ix_(i0 + 1, k0 + 1)]
        ab = a + (b - a) * sv[None, :]
        cd = c + (dd - c) * sv[None, :]
        total += (ab + (cd - ab) * su[:, None]) * 0.5 ** o
    total /= np.max(np.abs(total))
    return (base + amplitude * total).astype(np.float32)


def cloud_params(dt=0.01, rest_density=450.0, buoyancy=0.10, lapse=5.0):
    """CloudKernelInputs with the reference defaults (Clouds.cpp:67-102)."""
    p = abi.CloudParams()
    p.dim = 3
    p.timeStep = float(dt)
    p.restDensity = float(rest_density)
    p.groundHeatCoeff = 10.0
    p.buoyancyCoeff = float(buoyancy)
    p.gravCoeff = 0.0005
    p.adiabaticLapseRate = float(lapse)
    p.phaseTransitionRate = 0.3485
    p.latentHeatCoeff = 0.07
    p.isTempSmoothingEnabled = 1
    p.relaxCFM = 600.0
    p.initVaporDensityCoeff = 0.75
    p.windCoeff = 1.0
    return p


def cloud_env_reference():
    e = abi.CloudEnv()
    e.groundTemp0 = 293.0
    e.lapseRate = 3.5
    e.heatDecay = 3.0
    e.windDecayX = 0.2
    e.windDecayZ = 0.3
    e.groundNx = 0
    e.groundNz = 0
    return e


def clouds_cumulus(n=131072, res=(30, 60, 30), width=1.0, seed=0, noise=True, noise_res=64, max_n=None,
                   dt=0.01):
    """Clouds scene: the reference's Cumulus case (Clouds.cpp:451-456, box 10 x 20 x 10,
    grid 30 x 60 x 30, ParticleSystemApp.cpp:303-304) scaled to `width`, particles uniform
    in the lower quarter of the box.

    The reference's box height (20 units) stands for 10 km: its environment lapse is
    3.5 K/unit (7 K/km) and its adiabatic cooling 5 K/unit (10 K/km).  Scaled to the
    box: environment lapse 6.5 K/km (the standard atmosphere), adiabatic cooling
    10 K/km, heat-source decay, wind profile decays and wind drift scaled by the box
    ratio; buoyancy 0.5; condensation and latent-heat constants as in the reference.
    The ground temperature is seeded 8-octave value noise of +-3 K around 300 K.

    rho0 is the expected density of the uniform random start, W(0) + n / V (unit mass,
    poly6 integrates to 1).  The reference's unit-mass PBF coefficients (k, c, epsilon
    of Fluids.cpp:52-74, tuned at rho0 = 450) are rescaled by 450 / rho0."""
    rng = np.random.default_rng(seed)
    box = (width, 2.0 * width, width)
    W = [b / 2.0 for b in box]
    pos = np.zeros((n, 4), np.float32)
    pos[:, 0] = rng.uniform(-W[0], W[0], n)
    pos[:, 1] = rng.uniform(-W[1], -W[1] / 2.0, n)
    pos[:, 2] = rng.uniform(-W[2], W[2], n)
    vel = np.zeros((n, 4), np.float32)
    mp = abi.model_params(n, max_n or n, box, res, 3, abi.CASE_CLOUDS_CUMULUS)
    scale = box[1] / 20.0                # box units per reference unit
    km_per_unit = 10.0 / box[1]
    env = cloud_env_reference()
    env.lapseRate = 6.5 * km_per_unit    # K per box unit
    env.heatDecay = 3.0 * scale
    env.windDecayX = 0.2 / scale
    env.windDecayZ = 0.3 / scale
    ground = None
    if noise:
        ground = value_noise_2d(noise_res, noise_res, seed=seed + 1)
        env.groundTemp0 = 300.0
        env.groundNx = noise_res
        env.groundNz = noise_res
    h = width / res[0]
    volume = box[0] * box[1] * 0.25 * box[2]
    rho0 = 315.0 / (64.0 * math.pi * h ** 3) + n / volume
    r = 450.0 / rho0
    fp = abi.FluidParams()
    fp.restDensity = rho0
    fp.relaxCFM = 600.0
    fp.timeStep = dt
    fp.dim = 3
    fp.isArtPressureEnabled = 1
    fp.artPressureRadius = 0.006
    fp.artPressureCoeff = 0.001 * r
    fp.artPressureExp = 4
    fp.isVorticityConfEnabled = 1
    fp.vorticityConfCoeff = 0.0004 * r
    fp.xsphViscosityCoeff = 0.0001 * r
    cp = cloud_params(dt=dt, rest_density=rho0, buoyancy=0.5, lapse=10.0 * km_per_unit)
    cp.windCoeff = 1.0 * scale
    return {"pos": pos, "vel": vel, "model_params": mp, "fluid_params": fp, "cloud_params": cp,
            "env": env, "ground": ground}


def batched_dam_breaks(count=48, seed=0, n_range=(4096, 65536), aspect_range=(0.5, 2.0), d=0.0125, jitter=0.01):
    """Independent dam-break scenes for one batch: particle counts log-uniform in n_range,
    box aspect ratios (x extent over the unit y, z extents) uniform in aspect_range, seeded.

    Scene box = (round(40 a) h, 40 h, 40 h) with h = 2d; its fluid is a jittered lattice of
    spacing d filling x in [lo, lo + 0.4 L_x), z in [lo, lo + 0.8 L_z), layer by layer from
    the floor until the scene's count is reached (lo = -W + 0.01, the clamp floor).  Returns
    dict(scenes=[(n, (bx, by, bz))], pos, vel (concatenated in scene order), offsets,
    fluid_params, h, d)."""
    rng = np.random.default_rng(seed)
    h = 2.0 * d
    lo_n, hi_n = n_range
    ns = np.round(np.exp(rng.uniform(np.log(lo_n), np.log(hi_n), count))).astype(np.int64)
    aspects = rng.uniform(aspect_range[0], aspect_range[1], count)
    descs, poss, offs = [], [], []
    off = 0
    for n, a in zip(ns, aspects):
        rx = max(3, int(round(40 * a)))
        box = (rx * h, 40 * h, 40 * h)
        W = [b / 2.0 for b in box]
        nx = int(np.floor(0.4 * box[0] / d))
        nz = int(np.floor(0.8 * box[2] / d))
        ny = int(np.ceil(n / (nx * nz)))
        iy, ix, iz = np.meshgrid(np.arange(ny), np.arange(nx), np.arange(nz), indexing="ij")
        idx = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1)[:n].astype(np.float64)
        lo = np.array([-W[0] + 0.01, -W[1] + 0.01, -W[2] + 0.01])
        xyz = lo + (idx + 0.5) * d + rng.uniform(-jitter * d, jitter * d, size=(n, 3))
        p = np.zeros((n, 4), np.float32)
        p[:, :3] = xyz.astype(np.float32)
        descs.append((int(n), tuple(float(b) for b in box)))
        poss.append(p)
        offs.append(off)
        off += int(n)
    pos = np.concatenate(poss)
    return {"scenes": descs, "pos": pos, "vel": np.zeros_like(pos), "offsets": offs,
            "fluid_params": fluid_params(lattice_rest_density(d, h)), "h": h, "d": d}


def boids_plane(n=4096, box=2.0, res2=None):
    """The reference's 2D boids start (Boids.cpp:291-299): a circular grid in the x = 0 plane
    (Geometry::GenerateCircularGrid, utils/Geometry.cpp:128-185) between (0, -box/6, -box/6)
    and (0, box/6, box/6), velocities = positions (Boids.cpp:317-318).  res2 = (angles, radii)
    defaults to the reference's subdivision of n."""
    sub = {512: (32, 16), 1024: (32, 32), 4096: (64, 64), 8192: (128, 64), 16384: (128, 128),
           32768: (128, 256), 65536: (256, 256), 131072: (256, 512)}
    na, nr = res2 or sub[n]
    s = np.array([0.0, -box / 6.0, -box / 6.0], np.float32)
    e = np.array([0.0, box / 6.0, box / 6.0], np.float32)
    v = e - s
    c = s + v / np.float32(2.0)
    radius = np.float32(np.sqrt(np.float32(v @ v))) / np.float32(2.0)
    da = np.float32(2.0 * np.pi) / np.float32(na)
    dr = radius / np.float32(nr)
    io, ir = np.meshgrid(np.arange(na), np.arange(nr), indexing="ij")
    ang = (io.ravel().astype(np.float32) * da).astype(np.float32)
    rad = ((ir.ravel() + 1).astype(np.float32) * dr).astype(np.float32)
    pos = np.zeros((na * nr, 4), np.float32)
    pos[:, 0] = c[0]
    pos[:, 1] = c[1] + rad * np.cos(ang)
    pos[:, 2] = c[2] + rad * np.sin(ang)
    res = int(round(box / 0.05))
    mp = abi.model_params(na * nr, na * nr, (box, box, box), (res, res, res), 2, abi.CASE_INVALID)
    return {"pos": pos, "vel": pos.copy(), "model_params": mp, "boids_params": boids_params()}
