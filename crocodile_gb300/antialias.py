"""Sze-Tan optimal gridding functions: the ``crocodile.antialias`` surface.

Same names, arguments and results as crocodile/antialias.py (Sze Meng Tan's
optimal gridder: a gridding correction h(x) optimised by least squares so that
a support-2R gridding function C(l, nu) minimises the map error up to x0).

Where the work runs:

* the design step stays on the host in FP64, as in the reference: the
  least-squares fit of h (scipy ``leastsq`` over ``func_to_min``), the
  2R x 2R Gram systems, the small evaluation grids of the map error;
* the table- and image-sized evaluations run on the device in FP64:
  ``calc_gridding_fine`` (the gridding function at every oversampled offset;
  ``cg_szetan_gridding``) and ``calc_gridding_correction_fine`` (the grid
  correction at every image coordinate; ``cg_szetan_correction``).  The
  reference evaluates the latter with a Python loop over pixels, one numpy
  sum per (pixel, rp, r): minutes for an 8192-pixel axis.

The kernel cache: the reference reads ``gridder.json`` (json_tricks format)
from the working directory at import and fails without it
(antialias.py:16-20).  Here the file is read at import when present, and
``load_kernel_cache(path)`` reads one explicitly; json_tricks' ndarray
encoding (``{"__ndarray__": [...], "dtype": ..., "shape": [...]}``) is
decoded with the standard json module.  A missing kernel is optimised and
cached as in the reference.

The result of ``sze_tan_gridder(R, x0, over)`` is a real separable kernel
table [over, 2R]; ``conv_imaging(..., kv=table)`` grids with it as with any
[Q, S] table, and the image is divided by ``sze_tan_grid_correction``.
"""

import json
import os

import numpy
from scipy.optimize import leastsq

from . import engine as E
from .synthesis import coordinates

KERNEL_CACHE = {}


def _decode(obj):
    if isinstance(obj, dict) and "__ndarray__" in obj:
        a = numpy.asarray(obj["__ndarray__"], dtype=obj.get("dtype", "float64"))
        return a.reshape(obj.get("shape", a.shape))
    return obj


def load_kernel_cache(path="gridder.json"):
    """Add the optimised kernels of a json_tricks cache file (a list of
    ``[[[R, x0, N, M], []], {"R":, "x0":, "h":}]`` pairs) to KERNEL_CACHE."""
    with open(path) as f:
        entries = json.load(f, object_hook=_decode)
    for key, val in entries:
        KERNEL_CACHE[tuple(key[0])] = val
    return len(entries)


if os.path.exists("gridder.json"):
    load_kernel_cache("gridder.json")


def trap(vec, dx):
    """Trapezoidal integration (antialias.py:22-24)."""
    return dx * (numpy.sum(vec) - 0.5 * (vec[0] + vec[-1]))


def _trap_rows(mat, dx):
    return dx * (numpy.sum(mat, axis=-1) - 0.5 * (mat[..., 0] + mat[..., -1]))


def _offsets(R):
    """l = r - R + 1 for r = 0 .. 2R-1."""
    return numpy.arange(2 * R) - R + 1


def _h_grid(h, x0):
    N = len(h)
    x = x0 * numpy.arange(0, N + 1, dtype=float) / N
    return x, x0 / N, numpy.concatenate(([1.0], h))


def _gram(h_ext, x, dx, R):
    """K[rp, r] = trap(h_ext^2 cos(2 pi (lp - l) x), dx) (antialias.py:150-155)."""
    l = _offsets(R)
    arg = (2 * numpy.pi * (l[:, None] - l[None, :]).astype(float))[:, :, None] * x
    return _trap_rows((h_ext ** 2) * numpy.cos(arg), dx)


def _rhs(h_ext, x, dx, nu, R):
    """rhs[rp, m] = trap(h_ext cos(2 pi (lp - nu_m) x), dx) (antialias.py:158-162)."""
    l = _offsets(R)
    arg = (2 * numpy.pi * (l[:, None] - numpy.asarray(nu, dtype=float)[None, :]))[:, :, None] * x
    return _trap_rows(h_ext * numpy.cos(arg), dx)


def func_to_min(h, x0, M, R):
    """Residuals of the map-error fit (antialias.py:26-44): for each x_n and
    offset nu_m, 1 - Re and Im of h_ext[n] sum_r C[r, m] e^{2 pi i (l - nu_m) x_n},
    the end points weighted by 1/sqrt(2)."""
    N = len(h)
    nu = (numpy.arange(M, dtype=float) + 0.5) / (2 * M)
    x = x0 * numpy.arange(N + 1, dtype=float) / N
    C = calc_gridder_as_C(h, x0, nu, R)
    h_ext = numpy.concatenate(([1.0], h))
    one_app = 0
    for r, l in enumerate(_offsets(R)):
        one_app = one_app + h_ext[:, None] * C[r, :][None, :] * numpy.exp(
            (2j * numpy.pi * (l - nu))[None, :] * x[:, None])
    loss = numpy.empty((N + 1, 2, M), dtype=float)
    loss[:, 0, :] = 1.0 - numpy.real(one_app)
    loss[:, 1, :] = numpy.imag(one_app)
    loss[[0, N]] /= numpy.sqrt(2)
    return loss.reshape(2 * M * (N + 1))


def optimal_grid(R, x0, N, M, h_initial=None):
    """Least-squares fit of h at N points (antialias.py:46-49)."""
    if h_initial is None:
        h_initial = numpy.ones(N, dtype=float)
    return leastsq(func_to_min, h_initial, args=(x0, M, R), full_output=True)


def find_cached_kernel(R, x0, N=32, M=64, max_dx0=1 / 16):
    """Key of the cached kernel for (R, x0, N, M), else of the cached kernel with
    the same R and the closest x0 (ties: the later of two with N, M at least as
    large) (antialias.py:51-83)."""
    key = (R, x0, N, M)
    if key in KERNEL_CACHE:
        return key
    best, dx0 = None, 1e15
    for kp in KERNEL_CACHE.keys():
        Rp, x0p, Np, Mp = kp
        if Rp != R or abs(x0p - x0) > dx0:
            continue
        if abs(x0p - x0) == dx0 and (Np < best[2] or Mp < best[3]):
            continue
        best, dx0 = kp, abs(x0p - x0)
    return best


def optimal_grid_cached(R, x0, N=32, M=64, max_dx0=1 / 16, h_initial=None):
    """A cached optimal gridder good enough for (R, x0, N, M), else a new fit
    started from the nearest cached one or from smaller supports
    (antialias.py:85-137).  Returns {"R", "x0", "h", "err"}."""
    assert R >= 1
    assert x0 < 0.5
    best = find_cached_kernel(R, x0, N, M, max_dx0)
    if best is not None:
        Rp, x0p, Np, Mp = best
        if x0p >= x0 and x0p - x0 <= max_dx0 and Np >= N and Mp >= M:
            return KERNEL_CACHE[best]
    h_initial = None
    if best is not None:
        Rp, x0p, Np, Mp = best
        if abs(x0p - x0) <= max_dx0:
            x = x0 * (1 + numpy.arange(0, N, dtype=float)) / N
            h_initial = calc_gridding_correction_fine(x, KERNEL_CACHE[best]['h'], x0p, M, Rp)
    if h_initial is None:
        if R == 3:
            h_initial = optimal_grid_cached(R - 1, x0, N, M, max_dx0)['h']
        elif R >= 4:
            h0 = optimal_grid_cached(R - 2, x0, N, M, max_dx0)['h']
            h1 = optimal_grid_cached(R - 1, x0, N, M, max_dx0)['h']
            h_initial = h1 * (h1 / h0)
    key = (R, x0, N, M)
    print("Calculating", key)
    h, cov_h, infodict, mesg, ler = optimal_grid(R, x0, N, M, h_initial)
    if ler == 0:
        return None
    mean_map_err = calc_mean_map_error(x0, N, M, R, h)
    print("Mean map error: %g" % mean_map_err)
    result = {"R": R, "x0": x0, "h": h, "err": mean_map_err}
    KERNEL_CACHE[key] = result
    return result


def calc_gridder_as_C(h, x0, nu, R):
    """Gridding function C[2R, len(nu)] from h by least squares against the
    Gram matrix, rcond 1e-14 (antialias.py:139-164)."""
    x, dx, h_ext = _h_grid(h, x0)
    K = _gram(h_ext, x, dx, R)
    rhs = _rhs(h_ext, x, dx, nu, R)
    return numpy.linalg.lstsq(K, rhs, 1e-14)[0]


def make_evaluation_grids(R, M, N):
    """nu = (k + 0.5) / (2M), k < 2RM, and x = k / (2N), k <= N (antialias.py:166-174)."""
    nu = (numpy.arange(2 * R * M, dtype=float) + 0.5) / (2 * M)
    x = numpy.arange(N + 1, dtype=float) / (2 * N)
    return nu, x


def calc_gridder(h, x0, nu, M, R):
    """The gridder on the nu grid of make_evaluation_grids, folded by symmetry
    from C's first M offsets (antialias.py:176-187)."""
    C = calc_gridder_as_C(h, x0, nu, R)
    gridder = numpy.zeros(2 * M * R, dtype=float)
    m = numpy.arange(M)
    for rp, lp in enumerate(_offsets(R)):
        indx = m - 2 * lp * M
        indx = numpy.where(indx >= 0, indx, -indx - 1)
        gridder[indx] = C[rp, :M]
    return gridder


def calc_gridding_fine(h, x0, nu, R):
    """C[2R, len(nu)] at arbitrary offsets nu (antialias.py:193-213); the Gram
    matrix and its inverse on the host, the offsets on the device."""
    C = _gridding_fine_dev(h, x0, nu, R)
    return C.cpu().numpy()


def _gridding_fine_dev(h, x0, nu, R):
    E.require_cuda()
    x, dx, h_ext = _h_grid(numpy.asarray(h, dtype=float), x0)
    kinv = numpy.linalg.inv(_gram(h_ext, x, dx, R))
    return E.szetan_gridding(h_ext, x0, R, kinv, numpy.asarray(nu, dtype=float))


def gridder_to_C(gridder, R):
    """Sampled C[2R, M] from a gridder on the make_evaluation_grids nu grid
    (antialias.py:215-227)."""
    M = len(gridder) // (2 * R)
    C = numpy.zeros((2 * R, M), dtype=float)
    for r, l in enumerate(_offsets(R)):
        indx = numpy.arange(M) - 2 * M * l
        indx[indx < 0] = -indx[indx < 0] - 1
        C[r, :] = gridder[indx]
    return C


def calc_gridding_correction_fine(x, h, x0, M, R):
    """Grid correction hfine(x) = c(x) / d(x) of the gridder C sampled at M
    offsets (antialias.py:229-246), on the device."""
    nu = (numpy.arange(M, dtype=float) + 0.5) / (2 * M)
    C = _gridding_fine_dev(h, x0, nu, R)
    return E.szetan_correction(C, R, numpy.asarray(x, dtype=float)).cpu().numpy()


def calc_map_error(gridder, grid_correction, nu, x, R):
    """Map error at each x (antialias.py:248-263)."""
    M = len(nu) // (2 * R)
    dnu = nu[1] - nu[0]
    C = gridder_to_C(gridder, R)
    one_app = 0
    for r, l in enumerate(_offsets(R)):
        one_app = one_app + numpy.asarray(grid_correction)[:, None] * C[r, :][None, :] * \
            numpy.exp((2j * numpy.pi * (l - nu[:M]))[None, :] * numpy.asarray(x)[:, None])
    loss = numpy.stack([1.0 - numpy.real(one_app), numpy.imag(one_app)], axis=1)
    return 2 * numpy.sum(loss.reshape(len(x), -1) ** 2, axis=1) * dnu


def calc_mean_map_error(x0, N, M, R, h):
    """RMS map error over [0, x0] (antialias.py:265-271)."""
    nu, x = make_evaluation_grids(R, M, N)
    gridder = calc_gridder(h, x0, nu, M, R)
    grid_correction = calc_gridding_correction_fine(x, h, x0, M, R)
    map_err = calc_map_error(gridder, grid_correction, nu, x, R)
    which = numpy.digitize(x0, x)
    return numpy.sqrt(trap(map_err[:which], 1.0 / (2 * N)) / x[which])


def sze_tan_grid_correction(R, x0, image_size, Nopt=64, Mopt=32, max_dx0=1 / 16):
    """Sze-Tan grid correction on coordinates(image_size) (antialias.py:273-283)."""
    optimal_grid_cached(R, x0, Nopt, Mopt, max_dx0)
    return sze_tan_grid_correction_gen(R, x0, coordinates(image_size), Nopt, Mopt, max_dx0)


def sze_tan_grid_correction_gen(R, x0, x, Nopt=64, Mopt=32, max_dx0=1 / 16):
    """1 / hfine at arbitrary image coordinates x, with the gridder sampled at
    len(x) offsets (antialias.py:285-297)."""
    grid = optimal_grid_cached(R, x0, Nopt, Mopt, max_dx0)
    grid_correction = calc_gridding_correction_fine(numpy.array(x), grid['h'], grid['x0'],
                                                    len(x), R)
    return 1 / grid_correction


def sze_tan_gridder(R, x0, over, Nopt=64, Mopt=32, max_dx0=1 / 16):
    """The gridder as a separable [over, 2R] table in crocodile's kernel
    orientation: row f is C at nu = f / over, taps reversed (antialias.py:299-306)."""
    grid = optimal_grid_cached(R, x0, Nopt, Mopt, max_dx0)
    nu = numpy.arange(over, dtype=float) / over
    gridding = calc_gridding_fine(grid['h'], grid['x0'], nu, R)
    return numpy.transpose(gridding[::-1])


def sze_tan_mean_error(R, x0, Nopt=64, Mopt=32, max_dx0=1 / 16):
    """Mean map error of the cached or fitted gridder (antialias.py:308-316)."""
    grid = optimal_grid_cached(R, x0, Nopt, Mopt, max_dx0)
    return calc_mean_map_error(x0, Nopt, Mopt, R, grid['h'])
