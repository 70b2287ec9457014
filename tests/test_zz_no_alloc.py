"""cg_grid_noalloc: gridding for callers that cannot allocate device memory.

Such callers (a pipeline that owns all GPU memory in its own pool and may not
call cudaMalloc while it runs, or an FFI host that only passes its input and
output buffers) get the plan's scratch from a static device array inside the
library.  This test calls the entry point through the C ABI twice in a row
and checks each result against the existing cg_plan_create + cg_grid path on
the same inputs, within the FP32 tolerance of the other gridding tests; it
also checks that a request beyond the static scratch is refused without
writing.  It sits in a file of its own, collected last.
"""

import ctypes

import numpy
import pytest

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import _lib as L
    from crocodile_gb300 import build
    build.build()
    return torch, L


def _inputs(torch, seed, n, N, S, Q, G):
    rng = numpy.random.default_rng(seed)
    r = rng.uniform(0, 0.4, n)
    ph = rng.uniform(0, 2 * numpy.pi, n)
    uvw = numpy.column_stack([r * numpy.cos(ph), r * numpy.sin(ph), rng.uniform(-1, 1, n)])
    vis = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(numpy.complex64)
    ktab = (rng.normal(size=(G, Q, Q, S, S)) + 1j * rng.normal(size=(G, Q, Q, S, S)))
    kidx = rng.integers(0, G, n).astype(numpy.int32)
    dev = torch.device("cuda")
    return (torch.from_numpy(uvw).to(dev), torch.from_numpy(vis).to(dev),
            torch.from_numpy(ktab.astype(numpy.complex64)).to(dev),
            torch.from_numpy(kidx).to(dev))


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


# (S, Q, G, n): odd S runs the warp/owner gridders with 4 x 4-cell sub-tile
# buckets; even S <= 16 with a 4-D table runs the lane gridder (tile buckets,
# bulk-copy ring of kernel slices) with its scratch in the static array too
CASES = [(7, 4, 3, 100_000), (16, 4, 2, 60_000)]


@pytest.mark.parametrize("S,Q,G,n", CASES, ids=["warp-S7", "lane-S16"])
def test_noalloc_matches_workspace_path_twice(env, S, Q, G, n):
    torch, L = env
    lib = L.lib()
    N = 512
    kd = L.KernelDesc(0, Q, S, G)
    from types import SimpleNamespace
    from crocodile_gb300 import autotune
    lane = autotune.effective_layout(SimpleNamespace(S=S, sep=False)) == L.CG_LAYOUT_LANE
    assert lane == (S == 16)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call, seed in enumerate((11, 12)):
        uvw, vis, ktab, kidx = _inputs(torch, seed, n, N, S, Q, G)
        status = torch.zeros(L.CG_STATUS_WORDS, dtype=torch.int32, device="cuda")

        # existing entry points with a caller workspace
        ws_bytes = lib.cg_plan_workspace_bytes(L.CG_PLAN_TILED, n, N, N, ctypes.byref(kd))
        assert ws_bytes <= L.CG_NOALLOC_SCRATCH_BYTES
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
        ref = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
        plan = ctypes.c_void_p()
        L.call("cg_plan_create", ctypes.byref(plan), L.CG_PLAN_TILED, ctypes.byref(kd), N, N,
               _ptr(uvw), 3, 1.0, _ptr(kidx), n, _ptr(ws), ws_bytes, _ptr(status), stream)
        L.call("cg_grid", plan, _ptr(ktab), _ptr(vis), _ptr(ref), stream)
        lib.cg_plan_destroy(plan)

        # the static-scratch entry point on the same inputs
        got = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
        rc = lib.cg_grid_noalloc(ctypes.byref(kd), N, N, _ptr(uvw), 3, 1.0, _ptr(kidx), n,
                                 _ptr(ktab), _ptr(vis), _ptr(got), _ptr(status), stream)
        assert rc == L.CG_OK, lib.cg_last_error()
        assert lib.cg_status_check(_ptr(status), None, stream) == L.CG_OK
        err = float(torch.linalg.vector_norm((got - ref).to(torch.complex128)) /
                    torch.linalg.vector_norm(ref.to(torch.complex128)))
        assert err < FP32_TOL, "call %d: rel err %g" % (call, err)
        assert float(torch.linalg.vector_norm(ref)) > 0


def test_noalloc_refuses_more_than_its_scratch(env):
    torch, L = env
    lib = L.lib()
    N, S, Q, n = 512, 7, 4, 1_000_000
    kd = L.KernelDesc(0, Q, S, 1)
    need = lib.cg_plan_workspace_bytes(L.CG_PLAN_TILED, n, N, N, ctypes.byref(kd))
    assert need > L.CG_NOALLOC_SCRATCH_BYTES
    uvw = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    vis = torch.zeros(n, dtype=torch.complex64, device="cuda")
    ktab = torch.zeros((Q, Q, S, S), dtype=torch.complex64, device="cuda")
    grid = torch.full((N, N), 5 + 0j, dtype=torch.complex64, device="cuda")
    status = torch.zeros(L.CG_STATUS_WORDS, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.cg_grid_noalloc(ctypes.byref(kd), N, N, _ptr(uvw), 3, 1.0, None, n, _ptr(ktab),
                             _ptr(vis), _ptr(grid), _ptr(status), stream)
    assert rc == L.CG_ERR_WORKSPACE
    assert b"static scratch" in lib.cg_last_error()
    torch.cuda.synchronize()
    assert bool((grid == 5).all())
