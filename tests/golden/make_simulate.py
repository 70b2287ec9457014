"""Golden vectors of the reference's visibility helpers used by its own tests
(crocodile/simulate.py: simulate_point :210-230, visibility_shift :259-274,
uvw_transform :278-298), by running the real reference:

    python tests/golden/make_simulate.py /path/to/crocodile

Writes tests/golden/simulate_golden.npz; tests/test_oracle_golden.py pins the
oracle's restatements against it.  The GPU machine never runs this script.
"""

import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import import_reference  # noqa: E402  (stand-ins for pylru / astropy)


def main(root):
    _, simulate, _ = import_reference(root)
    rng = numpy.random.default_rng(2027)
    uvw = rng.uniform(-300, 300, (64, 3))
    vis = rng.normal(size=64) + 1j * rng.normal(size=64)
    s = 1 / numpy.sqrt(2)
    Ts = [numpy.array([[s, -s], [s, s]]), numpy.array([[1e5, -5e3], [6e4, -1e6]]),
          numpy.array([[0, .05], [-.05, 0]])]
    out = {"uvw": uvw, "vis": vis,
           "point": simulate.simulate_point(uvw, 0.013, -0.021),
           "shift": simulate.visibility_shift(uvw, vis, 0.01, -0.03),
           "Ts": numpy.array(Ts),
           "transformed": numpy.array([simulate.uvw_transform(uvw, T) for T in Ts])}
    numpy.savez_compressed(os.path.join(HERE, "simulate_golden.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
