"""Golden vectors of AW-towers imaging from the real reference notebook.

    python tests/golden/make_awtowers.py /path/to/crocodile

Executes code cells 7, 17, 19, 21 and 22 of
``examples/notebooks/awtowers.ipynb`` (read from that checkout at run time)
with ``crocodile.synthesis`` and ``crocodile.simulate`` imported from the
same checkout (stand-ins for pylru and astropy as make_golden.py), plotting
replaced by a no-op object, and this script's own inputs in place of the
notebook's VLA configuration and ionosphere (cells 3-5, 11-15): a few
antennas, seeded visibilities, per-antenna A-images given through the
notebook's ``ion_sample(antenna, l, m)`` hook, no phase-centre shift
(dl = dm = 0).  The notebook's ``grid_towers(vis)`` returns the image
real(ifft(grid_sum)) / aa x aa / sum(wt); its grid_sum is kept too.

The notebook moves a uv chunk's image between w-planes by multiplying with
wkern**(wp - last_wp), but skips that step after the chunk's first plane
when that plane is the data set's lowest (``if last_wp != wplanes[0]``).
The data here keeps the lowest plane in a chunk of its own, where the skip
changes nothing.  Writes ``tests/golden/awtowers_golden.npz``.
"""

import itertools
import json
import math
import os
import sys
import time

import numpy
import scipy.special

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import import_reference  # noqa: E402


class _NoPlot:
    def __getattr__(self, k):
        return self

    def __call__(self, *a, **k):
        return self

    def __iter__(self):
        return iter([self, self])

    def __setitem__(self, k, v):
        pass


def make_inputs(rng, nant=5, theta=0.1, lam=1280.0, subgrid=32, margin=8, wstep=20.0):
    C = subgrid - margin
    i1, i2 = numpy.triu_indices(nant, 1)
    rows = []
    for b in range(len(i1)):
        # a short track per baseline: a few samples within 0.4 of the grid
        u0, v0 = rng.uniform(-0.35, 0.35, 2) * lam
        v0 = abs(v0)
        w0 = rng.uniform(-40.0, 40.0)
        for t in range(12):
            rows.append((u0 + 3.0 * t, v0 + 1.5 * t, w0 + 1.2 * t, i1[b], i2[b]))
    r = numpy.array(rows)
    uvw = r[:, :3]
    # the lowest w plane alone in a chunk of its own: one visibility far out
    wmin_plane = numpy.floor(numpy.min(uvw[:, 2]) / wstep) - 1
    lone = numpy.array([[-0.4 * lam, 0.4 * lam, wmin_plane * wstep]])
    uvw = numpy.vstack([uvw, lone])
    src = numpy.vstack([r[:, 3:].astype(int), [[0, 1]]])
    vis = rng.normal(size=len(uvw)) + 1j * rng.normal(size=len(uvw))
    antennas = rng.normal(0, 100.0, (nant, 3))
    return dict(theta=theta, lam=lam, subgrid=subgrid, margin=margin, wstep=wstep, C=C,
                uvw=uvw, src=src, vis=vis, antennas=antennas)


def main(root):
    syn, sim, pylru = import_reference(root)
    nb = json.load(open(os.path.join(root, "examples", "notebooks", "awtowers.ipynb")))
    cells = ["".join(c["source"]) for c in nb["cells"]]
    rng = numpy.random.default_rng(21)
    inp = make_inputs(rng)
    g = {"numpy": numpy, "itertools": itertools, "math": math, "time": time, "scipy": scipy}
    for k in ("plt", "pylab", "show_image", "show_grid", "interact"):
        g[k] = _NoPlot()
    for mod in (sim, syn):  # the notebook's "from crocodile.simulate/synthesis import *"
        for n in dir(mod):
            if not n.startswith("_"):
                g[n] = getattr(mod, n)
    theta, lam = inp["theta"], inp["lam"]
    # per-antenna A-images through the notebook's ion_sample hook: a smooth
    # random phase screen and amplitude per antenna
    coef = rng.normal(0, 1.0, (len(inp["antennas"]), 5))

    def ion_sample(ant, l, m):
        a = int(numpy.argmin(numpy.sum((inp["antennas"][:, :2] - numpy.asarray(ant)) ** 2, 1)))
        k = coef[a]
        ph = (k[0] * l + k[1] * m) / theta + (k[2] * l * m) / theta ** 2
        return (1 + 0.1 * k[3] * (l / theta) ** 2) * numpy.exp(2j * numpy.pi * (0.3 * ph + 0.1 * k[4]))

    uvw, src, vis = inp["uvw"], inp["src"], inp["vis"]
    wt = numpy.ones(len(vis))
    wstep = inp["wstep"]
    wplane = numpy.around(uvw[:, 2] / wstep).astype(int)
    g.update(dict(theta=theta, lam=lam, wstep=wstep, margin=inp["margin"],
                  subgrid_size=inp["subgrid"], scaleByDet=False, approxKernel=False,
                  grid_size=int(numpy.ceil(theta * lam)), dl=0, dm=0, antennas=inp["antennas"],
                  ion_sample=ion_sample, uvw=uvw.copy(), vis=vis.copy(), src=src.copy(), wt=wt,
                  wplane=wplane, wplanes=numpy.arange(numpy.min(wplane), numpy.max(wplane) + 1)))
    exec(cells[7], g)
    for i in (17, 19, 21):
        exec(cells[i], g)
    # the bug case: a chunk holding the lowest plane and another plane
    C = inp["C"]
    ub = numpy.floor(uvw[:, 0] * theta / C + 0.5).astype(int)
    vb = numpy.floor(uvw[:, 1] * theta / C + 0.5).astype(int)
    low = wplane == numpy.min(wplane)
    for cu, cv in set(zip(ub[low], vb[low])):
        sel = (ub == cu) & (vb == cv)
        assert len(set(wplane[sel])) == 1, "the lowest plane shares its chunk"
    exec(cells[22], g)
    out = {k: numpy.asarray(v) for k, v in inp.items()}
    out["aimage"] = numpy.asarray(g["aimage"])
    out["image"] = numpy.asarray(g["image"])
    out["grid_sum"] = numpy.asarray(g["grid_sum"])
    out["aa_support"] = numpy.array(g["aa_support"])
    out["aa_over"] = numpy.array(g["aa_over"])
    numpy.savez_compressed(os.path.join(HERE, "awtowers_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "awtowers_golden.npz"), out["image"].shape,
          len(uvw), "visibilities")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
