"""Golden vectors of visibility ingest from the real reference.

    python tests/golden/make_ingest.py /path/to/crocodile

Builds seeded per-baseline visibility blocks as ``arl.data_models.Visibility``
objects (imported from that checkout) and flattens them with the
``collect_blocks`` function of ``scripts/image_dataset.py:75-82``, taken from
the script's source with ``ast`` and executed here, exactly as the script
does for uvw (``Visibility.uvw_lambda``, data_models.py:198-202), the src
columns and the first polarisation.  ``arl.data_models`` imports astropy,
which is not installed: the stand-ins give ``astropy.table.Table`` as a
column dictionary (the only use: ``self.data[col]``) and
``astropy.constants.c.value`` as the SI value 299792458.0 m/s.  Writes
``tests/golden/ingest_golden.npz``.
"""

import ast
import os
import sys
import tempfile
import textwrap

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))

ASTROPY_TABLE = textwrap.dedent('''
    class Table(dict):
        def __init__(self, cols=None, names=None, **kw):
            super().__init__()
            if isinstance(cols, dict):
                self.update(cols)
            elif cols is not None:
                self.update(zip(names, cols))
''')

ASTROPY_CONSTANTS = textwrap.dedent('''
    class _C:
        value = 299792458.0
    c = _C()
''')


def main(root):
    stub = tempfile.mkdtemp(prefix="arl_stubs_")
    os.makedirs(os.path.join(stub, "astropy"))
    open(os.path.join(stub, "astropy", "__init__.py"), "w").close()
    with open(os.path.join(stub, "astropy", "table.py"), "w") as f:
        f.write(ASTROPY_TABLE)
    with open(os.path.join(stub, "astropy", "constants.py"), "w") as f:
        f.write(ASTROPY_CONSTANTS)
    sys.path[:0] = [stub, root]
    from arl.data_models import Visibility

    rng = numpy.random.default_rng(12)
    viss, blocks = [], []
    for b, (a1, a2) in enumerate([(0, 1), (0, 5), (3, 4), (2, 7), (1, 6), (5, 6)]):
        nrow = int(rng.integers(1, 7))
        nchan = int(rng.integers(1, 5))
        npol = 4  # collect_blocks stacks the polarisation axis: one npol per data set
        freq = 1e8 + 1e6 * numpy.sort(rng.random(nchan)) * 50 + rng.random() * 1e3
        time = 58000.0 + numpy.sort(rng.random(nrow))
        uvw = rng.normal(0, 3000.0, (nrow, 3))
        vis = rng.normal(size=(nrow, nchan, npol)) + 1j * rng.normal(size=(nrow, nchan, npol))
        ant1 = numpy.full(nrow, a1, dtype=numpy.int64)
        ant2 = numpy.full(nrow, a2, dtype=numpy.int64)
        v = Visibility(frequency=freq, uvw=uvw, time=time, antenna1=ant1, antenna2=ant2,
                       vis=vis, weight=numpy.ones(vis.shape))
        viss.append(v)
        blocks.append(dict(frequency=freq, time=time, uvw=uvw, antenna1=ant1, antenna2=ant2,
                           vis=vis))

    src = open(os.path.join(root, "scripts", "image_dataset.py")).read()
    fn = [n for n in ast.walk(ast.parse(src))
          if isinstance(n, ast.FunctionDef) and n.name == "collect_blocks"][0]
    g = {"numpy": numpy, "viss": viss}
    exec(compile(ast.Module(body=[fn], type_ignores=[]), "image_dataset.py", "exec"), g)
    collect_blocks = g["collect_blocks"]
    uvw = collect_blocks(lambda vis, chan: vis.uvw_lambda(chan))
    srcc = collect_blocks(lambda vis, chan: numpy.transpose([
        vis.antenna1, vis.antenna2, vis.time,
        vis.frequency[chan] * numpy.ones(vis.time.shape)]))
    visc = collect_blocks(lambda vis, chan: vis.vis[:, chan, :])[:, 0]

    out = {"uvw_lambda": uvw, "src": srcc, "vis": visc, "nblocks": numpy.array(len(blocks))}
    for b, blk in enumerate(blocks):
        for k, v in blk.items():
            out["b%d_%s" % (b, k)] = v
    numpy.savez_compressed(os.path.join(HERE, "ingest_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "ingest_golden.npz"), uvw.shape, srcc.shape, visc.shape)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
