"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset of the reference is available (its data files are Git-LFS stubs),
so every input is generated here from a recorded seed:

  plain      : conv_imaging, 1024^2, theta 0.08, 200k vis, w = 0, S 8, Q 8
  wproj      : w_cache_imaging, 4096^2, theta 0.1, 2M vis, |w| <= 500, S 15, Q 8,
               wstep 10, NpixFF 64
  diff       : predict/invert of a 2048^2 image, 1M vis, w = 0, S 8, Q 8
  wstack     : 4096^2, 32 w-planes over +-800, 4M vis, power-law plane counts
  aw         : 8192^2, theta 0.05, 64 antennas, 2016 baselines x 125 times x 64
               channels of Earth-rotation uvw, AW kernels S 16, Q 16

Visibilities are point-source sums exp(-2 pi i (u l + v m + w (n - 1)))
(the formula of crocodile/simulate.py:210-230) computed in numpy.
"""

import dataclasses

import numpy


@dataclasses.dataclass
class Workload:
    name: str
    N: int
    theta: float
    lam: float
    uvw: numpy.ndarray
    vis: numpy.ndarray
    S: int
    Q: int
    params: dict


def radial_uv(rng, n, lam, rmax=0.45):
    """(u, v) with radial density proportional to 1/r inside |uv| <= rmax * lam."""
    r = rng.uniform(0, rmax * lam, n)
    phi = rng.uniform(0, 2 * numpy.pi, n)
    return r * numpy.cos(phi), r * numpy.sin(phi)


def point_sources(rng, uvw, nsrc, half_width, chunk=1 << 20):
    l = rng.uniform(-half_width, half_width, nsrc)
    m = rng.uniform(-half_width, half_width, nsrc)
    f = rng.normal(size=nsrc)
    nm1 = numpy.sqrt(1 - l ** 2 - m ** 2) - 1.0
    s = numpy.stack([l, m, nm1])  # [3, nsrc]
    vis = numpy.empty(len(uvw), dtype=numpy.complex128)
    for a in range(0, len(uvw), chunk):
        ph = uvw[a:a + chunk] @ s
        vis[a:a + chunk] = numpy.exp(-2j * numpy.pi * ph) @ f
    return vis


def plain(seed=20261203, n=200_000):
    rng = numpy.random.default_rng(seed)
    N, theta = 1024, 0.08
    lam = N / theta
    u, v = radial_uv(rng, n, lam)
    uvw = numpy.column_stack([u, v, numpy.zeros(n)])
    vis = point_sources(rng, uvw, 20, theta / 2)
    return Workload("conv_imaging 1024^2 S8 Q8 200k vis", N, theta, lam, uvw, vis, 8, 8,
                    {"seed": seed, "aa_c": 8})


def wproj(seed=20261204, n=2_000_000):
    rng = numpy.random.default_rng(seed)
    N, theta = 4096, 0.1
    lam = N / theta
    u, v = radial_uv(rng, n, lam)
    w = rng.uniform(-500, 500, n)
    uvw = numpy.column_stack([u, v, w])
    vis = point_sources(rng, uvw, 20, theta / 2)
    return Workload("w_cache_imaging+predict 4096^2 S15 Q8 2M vis", N, theta, lam, uvw, vis, 15, 8,
                    {"seed": seed, "wstep": 10.0, "NpixFF": 64, "w_range": 500.0})


def diff(seed=20261205, n=1_000_000):
    rng = numpy.random.default_rng(seed)
    N, theta = 2048, 0.08
    lam = N / theta
    u, v = radial_uv(rng, n, lam)
    uvw = numpy.column_stack([u, v, numpy.zeros(n)])
    image = numpy.zeros((N, N), dtype=numpy.float32)
    ix = rng.integers(N // 4, 3 * N // 4, (50, 2))
    image[ix[:, 1], ix[:, 0]] = rng.normal(size=50)
    return Workload("predict/invert 2048^2 S8 Q8 1M vis", N, theta, lam, uvw, None, 8, 8,
                    {"seed": seed, "image": image, "sources": ix})


def wstack(seed=20261206, n=4_000_000, planes=32, wmax=800.0, alpha=1.5):
    rng = numpy.random.default_rng(seed)
    N, theta = 4096, 0.1
    lam = N / theta
    step = 2 * wmax / (planes - 1)
    centres = -wmax + step * numpy.arange(planes)
    weights = (1.0 + numpy.arange(planes)) ** (-alpha)
    weights = weights[rng.permutation(planes)]
    counts = numpy.floor(weights / weights.sum() * n).astype(int)
    counts[numpy.argmax(counts)] += n - counts.sum()
    plane = numpy.repeat(numpy.arange(planes), counts)
    rng.shuffle(plane)
    w = centres[plane] + rng.uniform(-0.5 * step, 0.5 * step, n)
    u, v = radial_uv(rng, n, lam)
    uvw = numpy.column_stack([u, v, w])
    vis = point_sources(rng, uvw, 20, theta / 2)
    return Workload("w-stacking 4096^2 32 planes S8 Q8 4M vis", N, theta, lam, uvw, vis, 8, 8,
                    {"seed": seed, "plane": plane.astype(numpy.int32), "centres": centres,
                     "step": step})


def _local_to_celestial(xyz, lat):
    """Local (east, north, up) to celestial XYZ at latitude lat (simulate.py:50-69)."""
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    c = numpy.pi / 2 - lat
    return numpy.column_stack([x, -z * numpy.sin(c) + y * numpy.cos(c),
                               z * numpy.cos(c) + y * numpy.sin(c)])


def _xyz_to_uvw(xyz, ha, dec):
    """Rotation by hour angle and declination (simulate.py:74-100)."""
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    u = x * numpy.cos(ha) - y * numpy.sin(ha)
    v0 = x * numpy.sin(ha) + y * numpy.cos(ha)
    return numpy.column_stack([u, z * numpy.cos(dec) + v0 * numpy.sin(dec),
                               z * numpy.sin(dec) - v0 * numpy.cos(dec)])


def a_beams(rng, nant, npix, theta):
    """Per-antenna smooth complex beams on an npix far field: a Gaussian amplitude of
    random width times a low-order random phase screen (complex128 [nant, npix, npix])."""
    c = numpy.arange(-(npix // 2), -(npix // 2) + npix) / npix * theta
    m, l = numpy.meshgrid(c, c, indexing="ij")
    out = numpy.empty((nant, npix, npix), dtype=complex)
    for a in range(nant):
        sig = theta / 3 * (1 + 0.1 * rng.normal())
        amp = numpy.exp(-(l ** 2 + m ** 2) / (2 * sig ** 2))
        k = rng.normal(size=5)
        ph = (k[0] * l + k[1] * m) / theta * 0.2 + (k[2] * l * l + k[3] * m * m + k[4] * l * m) \
            / theta ** 2 * 0.3
        out[a] = amp * numpy.exp(2j * numpy.pi * ph)
    return out


def aw(seed=20261207, nant=64, ntime=125, nchan=64, nsrc=8, sigma_m=1500.0,
       lat_deg=-27.0, dec_deg=-45.0, ha_deg=60.0, bandwidth=0.3, wbins=64):
    """AW-projection at scale: 8192^2, theta 0.05, 64 antennas (Gaussian ENU positions,
    sigma 1.5 km), 2016 baselines x 125 hour angles x 64 channels of Earth-rotation uvw,
    channel frequencies scaled so that max |uv| = 0.45 lam (16,128,000 visibilities).
    Per-visibility antennas a1 < a2; per-antenna A-beams (32^2 far fields) for
    kernel_oversample(., 1, 16); w bins of width wstep = max|w| / (wbins / 2)."""
    rng = numpy.random.default_rng(seed)
    N, theta = 8192, 0.05
    lam = N / theta
    enu = numpy.column_stack([rng.normal(0, sigma_m, nant), rng.normal(0, sigma_m, nant),
                              rng.normal(0, 5.0, nant)])
    xyz = _local_to_celestial(enu, numpy.radians(lat_deg))
    i1, i2 = numpy.triu_indices(nant, 1)
    ha = numpy.radians(numpy.linspace(-ha_deg, ha_deg, ntime))
    dec = numpy.radians(dec_deg)
    bl = numpy.concatenate([(lambda a: a[i2] - a[i1])(_xyz_to_uvw(xyz, h, dec)) for h in ha])
    freq = 1 + bandwidth * numpy.arange(nchan) / max(nchan - 1, 1)  # relative frequencies
    scale = 0.45 * lam / (numpy.max(numpy.hypot(bl[:, 0], bl[:, 1])) * freq.max()) * (1 - 1e-9)
    uvw = (bl[:, None, :] * (freq[None, :, None] * scale)).reshape(-1, 3)
    nbl = len(i1)
    a1 = numpy.repeat(numpy.tile(i1, ntime), nchan).astype(numpy.int32)
    a2 = numpy.repeat(numpy.tile(i2, ntime), nchan).astype(numpy.int32)
    vis = point_sources(rng, uvw, nsrc, theta / 2)
    wstep = float(numpy.ceil(numpy.max(numpy.abs(uvw[:, 2])) / (wbins / 2)))
    beams = a_beams(rng, nant, 32, theta)
    return Workload("AW 8192^2 S16 Q16 %d vis" % len(uvw), N, theta, lam, uvw, vis, 16, 16,
                    {"seed": seed, "a1": a1, "a2": a2, "nbl": nbl, "nant": nant, "beams": beams,
                     "wstep": wstep, "NpixFF": 32, "dec_deg": dec_deg, "lat_deg": lat_deg,
                     "scale": scale})


def wproj_subset(w, n):
    """The first n visibilities of a workload (parity-test sized)."""
    return dataclasses.replace(w, uvw=w.uvw[:n].copy(), vis=w.vis[:n].copy())
