"""The plan's counting sort (cg_plan_export): the permutation is a bijection,
every sorted record is the bit-exact cell assignment of its input visibility
(frac_coords, synthesis.py:438-449, and the kernel rows of make_gcf,
synthesis.py:451-461), and bucket keys never decrease — for the lane
layout's tile buckets, the warp layout's Morton sub-tiles, w-bin plans and
the plain form's kernel groups."""

import numpy
import pytest

from test_tile_order_cpu import tile_index, tiles_per_layer  # the plans' tile numbering
from numpy.testing import assert_array_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import _lib as L
    from crocodile_gb300 import autotune, engine
    from oracle import crocodile_oracle
    yield torch, L, engine, autotune, crocodile_oracle
    autotune.set_tuning()


def _morton(x, y):
    def spread(a):
        a = a & 0xFF
        a = (a | (a << 4)) & 0x0F0F
        a = (a | (a << 2)) & 0x3333
        return (a | (a << 1)) & 0x5555
    return spread(x) | (spread(y) << 1)


def _case(n=60000, N=384, seed=41, wmax=0.0):
    rng = numpy.random.default_rng(seed)
    theta = 0.1
    lam = N / theta
    r = rng.uniform(0, 0.45 * lam, n)
    ph = rng.uniform(0, 2 * numpy.pi, n)
    uvw = numpy.column_stack([r * numpy.cos(ph), r * numpy.sin(ph), rng.uniform(-wmax, wmax, n)])
    return lam, N, uvw


def _expected(O, uvw, lam, N, Q, S, sep, g):
    x, xf, y, yf = O.frac_coords((N, N), Q, uvw[:, :2] / lam)
    x0, y0 = x - S // 2, y - S // 2
    if sep:
        return numpy.column_stack([x0, y0, g * Q + yf, g * Q + xf]).astype(numpy.int32)
    return numpy.column_stack([x0, y0, g, yf * Q + xf]).astype(numpy.int32)


def _check(plan, exp, key_of):
    recs, perm, counts = (t.cpu().numpy() for t in plan.export())
    n = len(exp)
    assert counts.sum() == n
    assert_array_equal(numpy.sort(perm), numpy.arange(n))   # a bijection
    assert_array_equal(recs, exp[perm])                      # bit-exact records
    keys = key_of(recs)
    assert (numpy.diff(keys) >= 0).all()                     # sorted by bucket
    assert_array_equal(numpy.bincount(keys, minlength=len(counts))[:len(counts)], counts)


@pytest.mark.parametrize("layout,S_,sep", [(0, 8, False), (1, 8, False), (1, 7, True),
                                           (2, 5, False), (3, 16, False)])
def test_tiled_plan_sort(env, layout, S_, sep):
    torch, L, E, A, O = env
    lam, N, uvw = _case()
    Q, G = 4, 3
    rng = numpy.random.default_rng(S_)
    g = rng.integers(0, G, len(uvw))
    shape = (G, Q, S_) if sep else (G, Q, Q, S_, S_)
    table = torch.zeros(int(numpy.prod(shape)), dtype=E.CF, device="cuda")
    kt = E.KernelTable(table, sep, Q, S_)
    A.set_tuning(layout=layout)
    try:
        plan = E.Plan(uvw, lam, (N, N), kt, kidx=g)
        info = plan.info()
        eff = A.effective_layout(kt)
    finally:
        A.set_tuning()
    plan.check()
    T = info["tile"]
    ntx = (N + T - 1) // T
    full = 0
    while (4 << full) < T:
        full += 1
    sublog = 0 if eff == L.CG_LAYOUT_LANE else full
    subshift = 2 + full - sublog
    assert info["buckets"] == tiles_per_layer(ntx, ntx) << (2 * sublog)

    def key_of(r):
        tile = tile_index(r[:, 0] // T, r[:, 1] // T, ntx, ntx)
        lx, ly = r[:, 0] - (r[:, 0] // T) * T, r[:, 1] - (r[:, 1] // T) * T
        return (tile << (2 * sublog)) | _morton(lx >> subshift, ly >> subshift)

    _check(plan, _expected(O, uvw, lam, N, Q, S_, sep, g), key_of)


def test_wbin_plan_sort(env):
    torch, L, E, A, O = env
    lam, N, uvw = _case(wmax=300.0, seed=42)
    Q, S_, wstep = 4, 8, 25.0
    k = numpy.round(uvw[:, 2] / wstep).astype(int)
    kmin = int(k.min())
    G = int(k.max()) - kmin + 1
    kt = E.KernelTable(torch.zeros(G * Q * Q * S_ * S_, dtype=E.CF, device="cuda"), False, Q, S_)
    plan = E.Plan(uvw, lam, (N, N), kt, wbins=(wstep, kmin))
    plan.check()
    T = plan.info()["tile"]
    ntx = (N + T - 1) // T
    _check(plan, _expected(O, uvw, lam, N, Q, S_, False, k - kmin),
           lambda r: tile_index(r[:, 0] // T, r[:, 1] // T, ntx, ntx))


def test_group_plan_sort(env):
    torch, L, E, A, O = env
    lam, N, uvw = _case(seed=43)
    Q, S_, G = 4, 6, 5
    g = numpy.random.default_rng(3).integers(0, G, len(uvw))
    kt = E.KernelTable(torch.zeros(G * Q * Q * S_ * S_, dtype=E.CD, device="cuda"), False, Q, S_)
    plan = E.Plan(uvw, lam, (N, N), kt, kidx=g, mode=L.CG_PLAN_GROUPS)
    plan.check()
    _check(plan, _expected(O, uvw, lam, N, Q, S_, False, g), lambda r: r[:, 2])
