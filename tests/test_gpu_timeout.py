"""A bounded wait of the lane gridder runs out on the GPU, and the call says so.

The lane gridder waits for every kernel slice's bulk copy for at most the
process-wide limit of cg_set_wait_limit (about two seconds by default).  With
the limit at 0 a warp whose copy has not landed when it first polls gives up:
the call counts CG_ERR_TIMEOUT in the status block, the warp lets its copies in
flight land (waiting at most the default limit) and returns.  Nothing hangs,
and the context stays usable: the next call with the default limit grids the
same visibilities to the oracle's result.
"""

import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import _lib as L
    from crocodile_gb300 import autotune
    from crocodile_gb300 import build
    from crocodile_gb300 import engine as E
    from oracle import crocodile_oracle as O
    build.build()
    return torch, L, E, O, autotune


def test_lane_wait_runs_out_and_context_survives(env):
    torch, L, E, O, autotune = env
    lib = L.lib()
    rng = numpy.random.default_rng(31)
    N, S, Q, G, n = 512, 16, 4, 2, 20_000
    r = rng.uniform(0, 0.4, n)
    ph = rng.uniform(0, 2 * numpy.pi, n)
    uvw = numpy.column_stack([r * numpy.cos(ph), r * numpy.sin(ph), numpy.zeros(n)])
    vis = rng.normal(size=n) + 1j * rng.normal(size=n)
    gcf = rng.normal(size=(G, Q, Q, S, S)) + 1j * rng.normal(size=(G, Q, Q, S, S))
    kidx = rng.integers(0, G, n).astype(numpy.int32)
    kt = E.KernelTable.from_gcf(gcf, 1, E.CF)
    assert autotune.effective_layout(kt) == L.CG_LAYOUT_LANE  # the gridder with the waits
    st = E.Status()
    st.reset()
    plan = E.Plan(uvw, 1.0, (N, N), kt, kidx, status=st)
    plan.check()
    v = E.cuda_tensor(vis, E.CF)

    default = lib.cg_get_wait_limit()
    assert default > 0
    try:
        assert lib.cg_set_wait_limit(0) == L.CG_OK
        grid = torch.zeros((N, N), dtype=E.CF, device="cuda")
        plan.grid(kt, v, grid)  # returns: every wait is bounded
        torch.cuda.synchronize()
        assert st.counts()[3] > 0  # timeouts counted
        with pytest.raises(RuntimeError, match="code -7"):
            st.check()
    finally:
        lib.cg_set_wait_limit(default)
    assert lib.cg_get_wait_limit() == default

    # the same plan and context, default limit: the oracle's grid
    st.reset()
    grid = torch.zeros((N, N), dtype=E.CF, device="cuda")
    plan.grid(kt, v, grid)
    plan.check()
    ref = numpy.zeros((N, N), dtype=complex)
    O.convgrid(gcf, ref, uvw[:, :2], kidx[:, None], vis)
    got = grid.cpu().numpy()
    assert numpy.linalg.norm(got - ref) / numpy.linalg.norm(ref) < 1e-5


def test_fft_tile_wait_runs_out_and_next_transform_is_exact(env):
    """The FP32 FFT's column passes (tensor copies of their tiles, from 2048
    rows) wait under the same limit: at 0 the first poll of a copy not yet
    landed gives up, the timeout is counted, and the call returns; with the
    default limit the next transform matches numpy."""
    torch, L, E, O, autotune = env
    lib = L.lib()
    rng = numpy.random.default_rng(32)
    a = rng.normal(size=(4096, 4096)) + 1j * rng.normal(size=(4096, 4096))
    E.fft_timeouts(reset=True)
    default = lib.cg_get_wait_limit()
    try:
        assert lib.cg_set_wait_limit(0) == L.CG_OK
        t = E.cuda_tensor(a, E.CF)
        E.fft_(t, True)
        torch.cuda.synchronize()
        assert E.fft_timeouts(reset=True) > 0
    finally:
        lib.cg_set_wait_limit(default)
    t = E.cuda_tensor(a, E.CF)
    E.fft_(t, True)
    assert E.fft_timeouts(reset=True) == 0
    ref = O.ifft(a)
    got = t.cpu().numpy()
    assert numpy.linalg.norm(got - ref) / numpy.linalg.norm(ref) < 2e-6


def test_ring_degrid_polls_under_zero_limit_and_next_call_is_exact(env):
    """The ring degridder (tuning dvis 3) waits for its slices' bulk copies under
    the same limit.  Its first copies fly while the CTA stages the grid window,
    so at a limit of 0 a poll may or may not find its copy landed: the call
    returns either way, and either counts timeouts (code -7) or gives the
    oracle's visibilities; with the default limit the same plan degrids to the
    oracle's visibilities."""
    torch, L, E, O, autotune = env
    lib = L.lib()
    rng = numpy.random.default_rng(33)
    N, S, Q, G, n = 512, 16, 4, 2, 20_000
    r = rng.uniform(0, 0.4, n)
    ph = rng.uniform(0, 2 * numpy.pi, n)
    uvw = numpy.column_stack([r * numpy.cos(ph), r * numpy.sin(ph), numpy.zeros(n)])
    gcf = rng.normal(size=(G, Q, Q, S, S)) + 1j * rng.normal(size=(G, Q, Q, S, S))
    kidx = rng.integers(0, G, n).astype(numpy.int32)
    a = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    kt = E.KernelTable.from_gcf(gcf, 1, E.CF)
    assert autotune.effective_layout(kt) == L.CG_LAYOUT_LANE
    st = E.Status()
    st.reset()
    plan = E.Plan(uvw, 1.0, (N, N), kt, kidx, status=st)
    plan.check()
    g = E.cuda_tensor(a, E.CF)
    default = lib.cg_get_wait_limit()
    autotune.set_tuning(dvis=3)
    try:
        try:
            assert lib.cg_set_wait_limit(0) == L.CG_OK
            first = plan.degrid(kt, g).cpu().numpy()  # returns: every wait is bounded
            timed_out = st.counts()[3] > 0
            if timed_out:
                with pytest.raises(RuntimeError, match="code -7"):
                    st.check()
        finally:
            lib.cg_set_wait_limit(default)
        st.reset()
        got = plan.degrid(kt, g).cpu().numpy()
        plan.check()
    finally:
        autotune.set_tuning()
    ref = O.convdegrid(gcf, a, uvw[:, :2], kidx[:, None])
    assert numpy.linalg.norm(got - ref) / numpy.linalg.norm(ref) < 1e-5
    if not timed_out:
        assert numpy.linalg.norm(first - ref) / numpy.linalg.norm(ref) < 1e-5
