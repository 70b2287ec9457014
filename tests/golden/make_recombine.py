"""Golden vectors of facet <-> subgrid recombination from the real reference.

    python tests/golden/make_recombine.py /path/to/crocodile

Executes the code cells of the reference notebook
``examples/notebooks/facet-subgrid-impl.ipynb`` (read from that checkout at
run time) with ``crocodile.synthesis`` imported from the same checkout (the
notebook's "Crocodile mode"), plotting replaced by a no-op object and
``numpy.random.seed(0)`` before the random test data.  The notebook's
parameter search at N = 512 selects the sizes of the C test set T05
(examples/grid/bench_recombine.c: 512, yB 128, yN 140, yP 216, xA 128,
xM 256, xMxN_yP 136).  Two loops are given one extra statement each to keep
their per-subgrid / per-facet results.  Writes
``tests/golden/recombine_golden.npz``.
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


def _patch(src, anchor, extra):
    assert anchor in src, anchor
    return src.replace(anchor, anchor + "\n" + extra)


def main(root):
    syn, sim, pylru = import_reference(root)
    nb = json.load(open(os.path.join(root, "examples", "notebooks",
                                     "facet-subgrid-impl.ipynb")))
    cells = ["".join(c["source"]) for c in nb["cells"]]
    g = {"numpy": numpy, "itertools": itertools, "math": math, "time": time, "scipy": scipy}
    for k in ("pylab", "mark_range", "show_image", "show_grid", "patches"):
        g[k] = _NoPlot()
    for n in dir(syn):
        if not n.startswith("_"):
            g[n] = getattr(syn, n)
    g["_cap_sub"], g["_cap_fac"] = [], []
    numpy.random.seed(0)
    for i in (2, 4, 6, 8, 11, 12, 14):
        exec(cells[i], g)
    exec(_patch(cells[16], "    approx = subgrid_A[i] * extract_mid(ifft(approx), xA_size)",
                "    _cap_sub.append(approx.copy())"), g)
    exec(_patch(cells[18], "    approx *= Fb * facet_B[j]", "    _cap_fac.append(approx.copy())"), g)
    for i in (20, 22, 24):
        exec(cells[i], g)
    ns, nf, n = g["nsubgrid"], g["nfacet"], g["xM_yN_size"]
    g["NMBF_NMBF"] = numpy.empty((ns, ns, nf, nf, n, n), dtype=complex)
    exec(cells[29], g)
    exec(cells[30], g)

    out = {}
    for k in ("N", "xA_size", "yB_size", "xM_size", "yN_size", "xM_yN_size", "yP_size",
              "xM_yP_size", "xMxN_yP_size", "nsubgrid", "nfacet", "subgrid_off", "facet_off",
              "pswf", "Fb", "Fn", "facet_m0_trunc", "G", "facet", "subgrid", "subgrid_A",
              "facet_B", "RNjMiBjFj", "FNjSi"):
        out[k] = numpy.asarray(g[k])
    out["approx_subgrid_1d"] = numpy.array(g["_cap_sub"])
    out["approx_facet_1d"] = numpy.array(g["_cap_fac"])
    facets = [(0, 0), (2, 1)]
    subgrids = [(0, 0), (1, 3), (3, 2)]
    out["facet2_idx"] = numpy.array(facets)
    out["subgrid2_idx"] = numpy.array(subgrids)
    out["facet2"] = numpy.array([g["facet_2"][j] for j in facets])
    out["nmbf2"] = numpy.array([[g["NMBF_NMBF"][i + j] for i in subgrids] for j in facets])
    out["rmse2"] = numpy.array(float(numpy.sqrt(numpy.mean(g["err_sum"]))))
    numpy.savez_compressed(os.path.join(HERE, "recombine_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "recombine_golden.npz"),
          os.path.getsize(os.path.join(HERE, "recombine_golden.npz")), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
