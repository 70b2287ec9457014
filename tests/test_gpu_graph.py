"""A step captured in a CUDA graph (plan + grid + degrid, and plan + fused
degrid/grid) replays to the same results as eager launches."""

import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import engine
    from oracle import crocodile_oracle
    return torch, engine, crocodile_oracle


def _case(O, S_, sep, n=40000, N=256, seed=31):
    rng = numpy.random.default_rng(seed)
    theta = 0.1
    lam = N / theta
    r = rng.uniform(0, 0.45 * lam, n)
    ph = rng.uniform(0, 2 * numpy.pi, n)
    uvw = numpy.column_stack([r * numpy.cos(ph), r * numpy.sin(ph), numpy.zeros(n)])
    vis = rng.normal(size=n) + 1j * rng.normal(size=n)
    aa = O.anti_aliasing_function(N, 0, 7)
    kv = O.kernel_oversample(aa, 4, S_) if sep else O.kernel_oversample(numpy.outer(aa, aa), 4, S_)
    return lam, N, uvw, vis, kv


def _rel(torch, a, b):
    return float(torch.linalg.vector_norm((a - b).to(torch.complex128)) /
                 torch.linalg.vector_norm(b.to(torch.complex128)))


@pytest.mark.parametrize("S_,sep", [(8, False), (16, False), (7, True)])
def test_captured_step_matches_eager(env, S_, sep):
    torch, E, O = env
    lam, N, uvw, vis, kv = _case(O, S_, sep)
    kt = E.KernelTable.from_gcf(kv, 0, E.CF)
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    v = E.cuda_tensor(vis, E.CF)
    grid = torch.zeros((N, N), dtype=E.CF, device="cuda")
    out = torch.empty(len(vis), dtype=E.CF, device="cuda")
    st = E.Status()

    def step():
        plan = E.Plan(uvw_t, lam, (N, N), kt, status=st)
        grid.zero_()
        plan.grid(kt, v, grid)
        plan.degrid(kt, grid, out)

    step()
    torch.cuda.synchronize()
    st.check()
    g_ref, o_ref = grid.clone(), out.clone()
    cap = E.CapturedStep(step)
    for _ in range(3):
        grid.fill_(1.0)
        out.zero_()
        cap.replay()
    torch.cuda.synchronize()
    st.check()
    assert _rel(torch, grid, g_ref) < 1e-6
    assert _rel(torch, out, o_ref) < 1e-6


def test_captured_major_cycle(env):
    """plan + residual fused pass (predict the model, grid vis - predicted) in a graph."""
    torch, E, O = env
    lam, N, uvw, vis, kv = _case(O, 16, False, seed=32)
    kt = E.KernelTable.from_gcf(kv, 0, E.CF)
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    v = E.cuda_tensor(vis, E.CF)
    rng = numpy.random.default_rng(5)
    model = E.cuda_tensor(rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N)), E.CF)
    res = torch.zeros((N, N), dtype=E.CF, device="cuda")
    pred = torch.empty(len(vis), dtype=E.CF, device="cuda")

    def cycle():
        plan = E.Plan(uvw_t, lam, (N, N), kt)
        res.zero_()
        plan.degrid_grid(kt, model, v, res, residual=True, vis_out=pred)

    cycle()
    torch.cuda.synchronize()
    r_ref, p_ref = res.clone(), pred.clone()
    cap = E.CapturedStep(cycle)
    res.fill_(2.0)
    cap.replay()
    torch.cuda.synchronize()
    assert _rel(torch, res, r_ref) < 1e-6
    assert _rel(torch, pred, p_ref) < 1e-6
