"""Generate golden vectors by running the real crocodile reference (Python).

Run in a container where the reference checkout is importable:

    python tests/golden/make_golden.py /path/to/crocodile

It imports ``crocodile.synthesis`` and ``crocodile.simulate`` from that
checkout.  The two third-party modules they import at top level that are not
installed here (``pylru``, ``astropy``) are replaced by small stand-ins
written into a temporary directory: ``pylru.FunctionCacheManager`` is a
memoising wrapper (the only use on the gridding path, synthesis.py:788,819)
and the astropy names are placeholders that ``simulate_point`` and
``xyz_to_baselines`` never touch.  Outputs go to ``tests/golden/*.npz``;
the GPU machine never runs this script, it only reads the committed fixtures.
"""

import os
import sys
import tempfile
import textwrap

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))

PYLRU_STUB = textwrap.dedent('''
    class FunctionCacheManager:
        def __init__(self, fn, size):
            self.fn = fn
            self.size = size
            self.cache = {}
        def __call__(self, *args, **kw):
            key = (args, tuple(sorted(kw.items())))
            if key not in self.cache:
                if len(self.cache) >= self.size:
                    self.cache.pop(next(iter(self.cache)))
                self.cache[key] = self.fn(*args, **kw)
            return self.cache[key]
''')

ASTROPY_COORD_STUB = textwrap.dedent('''
    class SkyCoord:
        def __init__(self, *a, **k):
            raise NotImplementedError("astropy stand-in")
    class CartesianRepresentation:
        pass
''')


def import_reference(root):
    stub = tempfile.mkdtemp(prefix="crocodile_stubs_")
    with open(os.path.join(stub, "pylru.py"), "w") as f:
        f.write(PYLRU_STUB)
    os.makedirs(os.path.join(stub, "astropy"))
    with open(os.path.join(stub, "astropy", "__init__.py"), "w") as f:
        f.write("")
    with open(os.path.join(stub, "astropy", "coordinates.py"), "w") as f:
        f.write(ASTROPY_COORD_STUB)
    with open(os.path.join(stub, "astropy", "units.py"), "w") as f:
        f.write("")
    sys.path[:0] = [stub, root]
    import crocodile.synthesis as syn
    import crocodile.simulate as sim
    import pylru
    return syn, sim, pylru


def point_vis(sim, uvw, rng, nsrc):
    vis = numpy.zeros(len(uvw), dtype=complex)
    for _ in range(nsrc):
        l, m = rng.uniform(-0.02, 0.02, 2)
        vis += rng.normal() * sim.simulate_point(uvw, l, m)
    return vis


def radial_uv(rng, n, lam, w_range=0.0):
    r = rng.uniform(0, 0.45 * lam, n)
    phi = rng.uniform(0, 2 * numpy.pi, n)
    w = rng.uniform(-w_range, w_range, n) if w_range else numpy.zeros(n)
    return numpy.column_stack([r * numpy.cos(phi), r * numpy.sin(phi), w])


def main(root):
    syn, sim, pylru = import_reference(root)
    rng = numpy.random.default_rng(20261203)
    out = {}

    # frac_coord: the C known-answer grid (N=4, Q=4, coordinates -2..1.9375 cells,
    # examples/grid/test_recombine.c:378-412) evaluated by the Python reference,
    # plus the exhaustive Q sweep of tests/test_synthesis.py:393-409 and random
    # coordinates at several sizes.
    cs = numpy.arange(-32, 32) / 16.0
    out["fc_t05_p"] = cs / 4
    out["fc_t05_x"], out["fc_t05_xf"] = syn.frac_coord(4, 4, cs / 4)
    ps, Ns, Qs, xs, xfs = [], [], [], [], []
    for N in [2, 5, 64, 1024, 4096, 8191, 8192]:
        for Q in [1, 3, 4, 8, 16]:
            p = rng.uniform(-0.5, 0.5, 257)
            p[:4] = [-0.5, 0.0, 0.5 - 2 ** -40, 0.25]
            p[4:8] = (numpy.arange(4) - 2) / (2 * N * Q)  # exact half-steps
            x, xf = syn.frac_coord(N, Q, p)
            ps.append(p); Ns.append(numpy.full(257, N)); Qs.append(numpy.full(257, Q))
            xs.append(x); xfs.append(xf)
    out["fc_p"] = numpy.concatenate(ps)
    out["fc_N"] = numpy.concatenate(Ns)
    out["fc_Q"] = numpy.concatenate(Qs)
    out["fc_x"] = numpy.concatenate(xs)
    out["fc_xf"] = numpy.concatenate(xfs)

    # kernels
    aa = syn.anti_aliasing_function(32, 0, 8)
    out["aa32"] = aa
    out["ko_1d"] = syn.kernel_oversample(aa, 4, 8)
    ff2 = rng.normal(size=(12, 12)) + 1j * rng.normal(size=(12, 12))
    out["ko_2d_ff"] = ff2
    out["ko_2d"] = syn.kernel_oversample(ff2, 3, 7)
    out["ko_2d_even"] = syn.kernel_oversample(ff2, 4, 8)
    out["wk_inv"] = syn.w_kernel(0.1, 37.5, 32, 7, 4)
    out["wk_fwd"] = syn.w_kernel(0.1, -120.0, 32, 7, 4, invert=False)
    T = numpy.array([[1.0, 0.05], [-0.02, 0.97]])
    out["wk_T"] = T
    out["wk_shift"] = syn.w_kernel(0.05, 80.0, 24, 9, 2, dl=0.003, dm=-0.002, T=T)

    # convolutional gridding on a small grid: 4-D kernel, separable kernel, src groups
    N, n, lam = 96, 600, 96 / 0.08
    uvw = radial_uv(rng, n, lam)
    vis = point_vis(sim, uvw, rng, 5)
    out["cg_uvw"], out["cg_vis"], out["cg_lam"] = uvw, vis, lam
    k4 = syn.kernel_oversample(numpy.outer(syn.anti_aliasing_function(N, 0, 6),
                                            syn.anti_aliasing_function(N, 0, 6)), 4, 6)
    k1 = syn.kernel_oversample(syn.anti_aliasing_function(N, 0, 6), 4, 6)
    out["cg_k4"], out["cg_k1"] = k4, k1
    a = numpy.zeros((N, N), dtype=complex)
    syn.convgrid(k4, a, uvw / lam, None, vis)
    out["cg_grid4"] = a
    a = numpy.zeros((N, N), dtype=complex)
    syn.convgrid(k1, a, uvw / lam, None, vis)
    out["cg_grid1"] = a
    src = rng.integers(0, 3, (n, 1))
    kg = numpy.array([k4 * (1 + 0.5 * j) * numpy.exp(0.3j * j) for j in range(3)])
    out["cg_src"], out["cg_kg"] = src, kg
    a = numpy.zeros((N, N), dtype=complex)
    syn.convgrid(kg, a, uvw / lam, src, vis)
    out["cg_gridsrc"] = a
    model = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    out["cg_model"] = model
    out["cd_vis4"] = syn.convdegrid(k4, model, uvw / lam)
    out["cd_vis1"] = syn.convdegrid(k1, model, uvw / lam)
    out["cd_vissrc"] = syn.convdegrid(kg, model, uvw / lam, src)

    # drivers
    theta = 0.08
    out["di_theta"] = theta
    d, psf, pmax = syn.do_imaging(theta, lam, uvw, None, vis, syn.conv_imaging, kv=k4)
    out["di_dirty"], out["di_psf"], out["di_pmax"] = d, psf, pmax
    img = numpy.zeros((N, N))
    img[rng.integers(10, N - 10, 8), rng.integers(10, N - 10, 8)] = rng.normal(size=8)
    out["dp_image"] = img
    out["dp_vis"] = syn.do_predict(theta, lam, uvw, None, img, syn.conv_predict, kv=k4)
    out["wt"] = syn.doweight(theta, lam, uvw, numpy.ones(n))
    mu, mv = syn.mirror_uvw(uvw, vis)
    out["mirror_uvw"], out["mirror_vis"] = mu, mv
    for Nh in (8, 9):
        g = rng.normal(size=(Nh, Nh)) + 1j * rng.normal(size=(Nh, Nh))
        out["herm_in_%d" % Nh] = g.copy()
        out["herm_out_%d" % Nh] = syn.make_grid_hermitian(g)
    g = rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16))
    out["fft_in"] = g
    out["fft_out"] = syn.fft(g)
    out["ifft_out"] = syn.ifft(g)
    g = rng.normal(size=(15, 15)) + 1j * rng.normal(size=(15, 15))
    out["fft_in_odd"] = g
    out["fft_out_odd"] = syn.fft(g)
    out["ifft_out_odd"] = syn.ifft(g)

    # boxcar gridding
    a = numpy.zeros((N, N), dtype=complex)
    syn.grid(a, uvw / lam, vis)
    out["box_grid"] = a
    out["box_degrid"] = syn.degrid(model, uvw / lam)

    # w-projection through the w-cache (the reference's own loop)
    Nw, nw, thw = 128, 400, 0.1
    lamw = Nw / thw
    uvww = radial_uv(rng, nw, lamw, w_range=60.0)
    visw = point_vis(sim, uvww, rng, 4)
    out["wc_uvw"], out["wc_vis"], out["wc_lam"], out["wc_theta"] = uvww, visw, lamw, thw
    kw = dict(NpixFF=16, NpixKern=7, Qpx=4)
    cache = pylru.FunctionCacheManager(syn.w_kernel, 64)
    out["wc_grid"] = syn.w_cache_imaging(thw, lamw, uvww, numpy.zeros((nw, 0)), visw,
                                         wstep=10.0, kernel_cache=cache, **kw)

    # AW kernels: scipy convolve2d semantics pinned by the reference's aw_kernel_fn
    akerns = rng.normal(size=(3, 6, 6)) + 1j * rng.normal(size=(3, 6, 6))
    out["aw_akerns"] = akerns
    awfn = syn.aw_kernel_fn(lambda theta, a: akerns[a],
                            lambda theta, w: syn.w_kernel(theta, w, 16, 6, 2))
    out["aw_k01"] = awfn(0.1, 25.0, 0, 1)
    out["aw_k12"] = awfn(0.1, -40.0, 1, 2)

    # simulate_point
    out["sp_vis"] = sim.simulate_point(uvww, 0.013, -0.007)

    path = os.path.join(HERE, "reference_golden.npz")
    numpy.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
