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


def wproj_subset(w, n):
    """The first n visibilities of a workload (parity-test sized)."""
    return dataclasses.replace(w, uvw=w.uvw[:n].copy(), vis=w.vis[:n].copy())
