"""AW-projection on the device: per-baseline A-kernels convolved with w-kernels.

The reference's AW path is w_cache_imaging (crocodile/synthesis.py:757-796)
with kernel_cache = aw_kernel_fn(a_kernel_fn, w_kernel_fn) (:701-734) keyed by
(theta, wbin, a1, a2) (scripts/image_dataset.py:142-171): one kernel per
distinct (w bin, antenna pair), generated on a cache miss, and one
convgrid call per visibility.  Here the distinct keys of all visibilities are
found on the device (cg_aw_keys + cg_compact_keys), every AW kernel they need
is generated in one batch (cg_aw_kernels) into a table resident in HBM, and
all visibilities grid and degrid through one plan.
"""

import time

import numpy
import torch

from . import _lib as L
from . import engine as E


class AWProjection:
    """Grid/degrid operator with AW kernels for fixed uvw and antenna pairs.

    uvw [n, 3] (wavelengths), a1, a2 [n] antenna indices, beams [nant, F, F]
    complex far fields of the antennas (A-kernel = kernel_oversample(beam, 1,
    SA)), wstep: w-bin width, w-kernels w_kernel(theta, wbin, NpixFF, S, Q).
    fp64=True also prepares the plain FP64 form (one launch per w-plane).
    phase_ms: a dict that receives the host time of each set-up phase (the
    device synchronised at every phase boundary), for profiling."""

    def __init__(self, theta, lam, uvw, a1, a2, beams, wstep, NpixFF=32, Q=16, S=16, SA=16,
                 N=None, fp64=False, phase_ms=None):
        t_last = [time.perf_counter()]

        def phase(name):
            if phase_ms is not None:
                torch.cuda.synchronize()
                now = time.perf_counter()
                phase_ms[name] = 1e3 * (now - t_last[0])
                t_last[0] = now

        self.status = st = E.Status()
        self.theta, self.lam = float(theta), float(lam)
        self.N = int(round(theta * lam)) if N is None else int(N)
        self.uvw = E.cuda_tensor(uvw, torch.float64)
        nant = int(beams.shape[0])
        wbin, kmin, kmax = E.w_bins(self.uvw, wstep, st)
        st.check()
        nb = kmax - kmin + 1
        keys = E.aw_keys(self.uvw, a1, a2, nant, wstep, kmin, nb, st)
        rows, kor = E.compact_keys(keys, nant * nant * nb, st)
        st.check()
        kor = kor.cpu().numpy().astype(numpy.int64)
        wi, pair = kor % nb, kor // nb
        self.rows, self.wbin, self.nbins, self.kmin = rows, wbin, nb, kmin
        self.nkernels = len(kor)
        phase("bins_and_keys")
        A = E.kernel_oversample(beams, 1, SA, dtype=E.CD, ndim=2).reshape(nant, SA, SA)
        phase("a_kernels")
        Wk = E.w_kernels(theta, wstep * numpy.arange(kmin, kmax + 1).astype(numpy.float64),
                         NpixFF, S, Q, dtype=E.CD, status=st)
        phase("w_kernels")
        self.A, self.Wk = A, Wk
        args = (A, Wk, (pair // nant).astype(numpy.int32), (pair % nant).astype(numpy.int32),
                wi.astype(numpy.int32))
        self._aw_args = args
        self.ktab = E.KernelTable(E.aw_kernels(*args, dtype=E.CF, status=st).reshape(-1), False,
                                  Q, SA)
        phase("aw_table")
        self.replan()
        phase("plan")
        self.ktab64 = self.plan64 = None
        if fp64:
            self.enable_fp64()
        st.check()

    def enable_fp64(self):
        """Prepare the plain FP64 form: the same AW kernels held as complex128 and a
        groups plan with one launch per w-plane."""
        st = self.status
        Q, SA = self.ktab.Q, self.ktab.S
        self.ktab64 = E.KernelTable(E.aw_kernels(*self._aw_args, dtype=E.CD,
                                                 status=st).reshape(-1), False, Q, SA)
        self.plan64 = E.Plan(self.uvw, self.lam, (self.N, self.N), self.ktab64, self.rows,
                             mode=L.CG_PLAN_GROUPS, status=st, groups=(self.nbins, self.wbin))
        st.check()

    def disable_fp64(self):
        self.ktab64 = self.plan64 = None

    def replan(self):
        """(Re)build the tiled plan, e.g. after the launch-shape tuning changed."""
        self.plan = E.Plan(self.uvw, self.lam, (self.N, self.N), self.ktab, self.rows,
                           status=self.status)

    def tune(self, vis, quick=True):
        """Autotune the tiled kernels on these visibilities and rebuild the plan."""
        from . import autotune
        best, table = autotune.tune(self.uvw, self.lam, (self.N, self.N), self.ktab, self.rows,
                                    E.cuda_tensor(vis, E.CF),
                                    cands=autotune.candidates(self.ktab.S, quick=quick),
                                    use_cache=False)
        self.replan()
        return best

    def grid(self, vis, out=None):
        g = out if out is not None else torch.zeros((self.N, self.N), dtype=E.CF, device="cuda")
        return self.plan.grid(self.ktab, E.cuda_tensor(vis, E.CF), g)

    def degrid(self, grid):
        return self.plan.degrid(self.ktab, E.cuda_tensor(grid, E.CF))

    def degrid_grid(self, grid_in, vis_in, grid_out, residual=False, vis_out=None):
        """Fused pass: each AW kernel slice is read once for both directions."""
        return self.plan.degrid_grid(self.ktab, E.cuda_tensor(grid_in, E.CF),
                                     None if vis_in is None else E.cuda_tensor(vis_in, E.CF),
                                     grid_out, residual, vis_out)

    def grid_fp64(self, vis, out=None):
        g = out if out is not None else torch.zeros((self.N, self.N), dtype=E.CD, device="cuda")
        return self.plan64.grid_fp64(self.ktab64, E.cuda_tensor(vis, E.CD), g)

    def degrid_fp64(self, grid):
        return self.plan64.degrid_fp64(self.ktab64, E.cuda_tensor(grid, E.CD))
