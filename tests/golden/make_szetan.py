"""Golden vectors of the Sze-Tan gridder from the real crocodile reference.

    python tests/golden/make_szetan.py /path/to/crocodile

Imports ``crocodile.antialias`` from that checkout.  It needs ``json_tricks``
(not installed here) only for ``json_tricks.np.load`` of the kernel cache
``examples/notebooks/gridder.json``; a stand-in decoding json_tricks'
ndarray encoding is written to a temporary directory.  The reference reads
the cache from the working directory at import, so the script runs there.
Writes ``tests/golden/szetan_golden.npz``: the cache keys, for three cached
(R, x0) the optimised h and the reference's outputs, kernel-cache lookups,
and one small least-squares fit.
"""

import os
import sys
import tempfile
import textwrap

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import import_reference  # noqa: E402

JSON_TRICKS_STUB = textwrap.dedent('''
    import json
    import numpy
    def _decode(obj):
        if isinstance(obj, dict) and "__ndarray__" in obj:
            a = numpy.asarray(obj["__ndarray__"], dtype=obj.get("dtype", "float64"))
            return a.reshape(obj.get("shape", a.shape))
        return obj
    def load(f):
        return json.load(f, object_hook=_decode)
''')

CASES = [(2, 0.25), (4, 0.375), (5, 0.4375)]
QUERIES = [(3, 0.25, 64, 32), (3, 0.26, 64, 32), (2, 0.3, 32, 64), (4, 0.1, 32, 64),
           (1, 0.49, 64, 32), (6, 0.25, 64, 32)]


def main(root):
    import_reference(root)
    stub = tempfile.mkdtemp(prefix="json_tricks_stub_")
    os.makedirs(os.path.join(stub, "json_tricks"))
    open(os.path.join(stub, "json_tricks", "__init__.py"), "w").close()
    with open(os.path.join(stub, "json_tricks", "np.py"), "w") as f:
        f.write(JSON_TRICKS_STUB)
    sys.path.insert(0, stub)
    cwd = os.getcwd()
    os.chdir(os.path.join(root, "examples", "notebooks"))
    try:
        import crocodile.antialias as A
    finally:
        os.chdir(cwd)

    out = {}
    keys = sorted(A.KERNEL_CACHE.keys())
    out["cache_keys"] = numpy.array(keys, dtype=float)
    for i, (R, x0) in enumerate(CASES):
        key = (R, x0, 64, 32)
        h = numpy.asarray(A.KERNEL_CACHE[key]["h"], dtype=float)
        out["case_%d" % i] = numpy.array([R, x0])
        out["h_%d" % i] = h
        out["gridder_%d" % i] = A.sze_tan_gridder(R, x0, 16)
        out["corr_%d" % i] = A.sze_tan_grid_correction(R, x0, 64)
        out["mean_err_%d" % i] = numpy.array(A.sze_tan_mean_error(R, x0))
        out["ftm_%d" % i] = A.func_to_min(h, x0, 32, R)
        nu = (numpy.arange(32, dtype=float) + 0.5) / 64
        out["gac_%d" % i] = A.calc_gridder_as_C(h, x0, nu, R)
        xs = numpy.linspace(0, 0.5, 37)
        out["fine_corr_%d" % i] = A.calc_gridding_correction_fine(xs, h, x0, 48, R)
    res = []
    for q in QUERIES:
        b = A.find_cached_kernel(*q)
        res.append([numpy.nan] * 4 if b is None else list(b))
    out["queries"] = numpy.array(QUERIES, dtype=float)
    out["query_results"] = numpy.array(res, dtype=float)
    h, cov, info, mesg, ler = A.optimal_grid(2, 0.25, 8, 8)
    out["fit_h"] = numpy.asarray(h)
    out["fit_mean_err"] = numpy.array(A.calc_mean_map_error(0.25, 8, 8, 2, h))
    numpy.savez_compressed(os.path.join(HERE, "szetan_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "szetan_golden.npz"), sorted(out))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
