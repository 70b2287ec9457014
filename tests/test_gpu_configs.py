"""The measured configurations at their full sizes against the complex128
oracle (relative L2 <= 1e-5, bit-exact cell assignment):

* conv_imaging 1024^2, 200,000 visibilities, S 8, Q 8 (separable and 4-D
  anti-aliasing kernels): the grid, do_imaging's dirty image, PSF and PSF
  maximum, and do_predict's visibilities (synthesis.py:583-613, 883-927);
* w_cache_imaging / w_cache_predict 4096^2, 2,000,000 visibilities, S 15,
  Q 8, 101 w-kernels (synthesis.py:757-828): the grid and the predicted
  visibilities, and the w bin of every visibility.
The AW and w-stacking configurations are checked in test_gpu_aw.py and
test_gpu_wstack.py."""

import numpy
import pytest
from numpy.testing import assert_array_equal

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import configs, synthesis
    from oracle import crocodile_oracle
    return configs, synthesis, crocodile_oracle


def rel(a, b):
    return numpy.linalg.norm(numpy.asarray(a) - numpy.asarray(b)) / numpy.linalg.norm(b)


@pytest.mark.parametrize("four_d", [False, True])
def test_conv_imaging_config(env, four_d):
    C, S, O = env
    w = C.plain()
    assert (w.N, len(w.uvw)) == (1024, 200_000)
    aa = O.anti_aliasing_function(w.N, 0, w.params["aa_c"])
    kv = O.kernel_oversample(numpy.outer(aa, aa) if four_d else aa, 8, 8)
    p = w.uvw / w.lam
    for g, e in zip(S.frac_coords((w.N, w.N), 8, p), O.frac_coords((w.N, w.N), 8, p)):
        assert_array_equal(numpy.asarray(g), e)
    grid = S.conv_imaging(w.theta, w.lam, w.uvw, None, w.vis, kv)
    grid_ref = O.conv_imaging(w.theta, w.lam, w.uvw, None, w.vis, kv)
    assert rel(grid, grid_ref) < TOL
    dirty, psf, pmax = S.do_imaging(w.theta, w.lam, w.uvw, None, w.vis, S.conv_imaging, kv=kv)
    d_ref, p_ref, m_ref = O.do_imaging(w.theta, w.lam, w.uvw, None, w.vis, O.conv_imaging, kv=kv)
    assert rel(dirty, d_ref) < TOL
    assert rel(psf, p_ref) < TOL
    assert abs(pmax - m_ref) <= TOL * abs(m_ref)
    pv = S.do_predict(w.theta, w.lam, w.uvw, None, d_ref, S.conv_predict, kv=kv)
    pv_ref = O.do_predict(w.theta, w.lam, w.uvw, None, d_ref, O.conv_predict, kv=kv)
    assert rel(pv, pv_ref) < TOL


def test_w_projection_config(env):
    C, S, O = env
    w = C.wproj()
    assert (w.N, len(w.uvw)) == (4096, 2_000_000)
    kw = dict(wstep=w.params["wstep"], NpixFF=w.params["NpixFF"], NpixKern=w.S, Qpx=w.Q)
    grid = S.w_cache_imaging(w.theta, w.lam, w.uvw, None, w.vis, **kw)
    grid_ref = O.w_cache_imaging(w.theta, w.lam, w.uvw, None, w.vis, **kw)
    assert rel(grid, grid_ref) < TOL
    vis = S.w_cache_predict(w.theta, w.lam, w.uvw, None, grid_ref, **kw)
    vis_ref = O.w_cache_predict(w.theta, w.lam, w.uvw, None, grid_ref, **kw)
    assert rel(vis, vis_ref) < TOL
    # the w bin of every visibility (synthesis.py:793), bit-exact
    from crocodile_gb300 import engine as E
    st = E.Status()
    kidx, kmin, kmax = E.w_bins(w.uvw, kw["wstep"], st)
    st.check()
    k = numpy.round(w.uvw[:, 2] / kw["wstep"]).astype(numpy.int64)
    assert (kmin, kmax) == (k.min(), k.max())
    assert_array_equal(kidx.cpu().numpy(), k - k.min())
