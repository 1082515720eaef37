"""The allocation-free operator apply, checked against the context's apply.

``scf_apply_operator_noalloc`` serves callers that cannot allocate device
memory mid-step (hosts that hand out all device memory from their own arena,
or jobs at a fixed memory budget on a shared GPU).  It keeps its only scratch,
the per-block partial sums of x.Ax, in a static device array.  This test feeds
it the operator that ``scf_debug_operator`` reports, in device buffers the
test owns, and compares y = A x with ``scf_debug_apply`` on two calls in a row
(the second call reuses the scratch the first one left behind).
"""
import ctypes as C

import numpy as np
import pytest

from simcoflow3d_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu


def test_apply_operator_noalloc_matches_context_apply(gpu_lib):
    import torch
    from simcoflow3d_gb300.projection import Projection

    w = W.config("c1", n=20)
    I, J, K = w.imax, w.jmax, w.kmax
    proj = Projection.for_workload(w)
    proj.stage(w, correction=False)
    op = proj.debug_operator()

    def ghosted(a):
        g = np.zeros(w.shape_g, order="F")
        g[1:-1, 1:-1, 1:-1] = a
        return g

    dev = torch.device("cuda", 0)

    def to_dev(a):
        return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).to(dev)

    ops = [to_dev(ghosted(op[k])) for k in ("diag", "cpl_e", "cpl_n", "cpl_t")]
    rng = np.random.default_rng(11)
    solid = w.arrays["cell_type"] == 2
    for call in range(2):
        x = np.zeros(w.shape_g, order="F")
        x[1:-1, 1:-1, 1:-1] = rng.normal(size=(I, J, K))
        x[1:-1, 1:-1, 1:-1][solid] = 0.0
        y_ref = proj.debug_apply(x)

        xd = to_dev(x)
        yd = torch.zeros_like(xd)
        ed = torch.zeros(1, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = gpu_lib.scf_apply_operator_noalloc(I, J, K, *(o.data_ptr() for o in ops), xd.data_ptr(),
                                                yd.data_ptr(), ed.data_ptr(), None)
        assert rc == capi.SCF_OK
        torch.cuda.synchronize()
        y = yd.cpu().numpy().reshape(w.shape_g, order="F")
        yi, ri = y[1:-1, 1:-1, 1:-1], y_ref[1:-1, 1:-1, 1:-1]
        assert np.linalg.norm(yi - ri) <= 1e-14 * np.linalg.norm(ri), f"call {call}"
        energy = float(np.dot(x[1:-1, 1:-1, 1:-1].ravel(), ri.ravel()))
        assert abs(ed.item() - energy) <= 1e-12 * abs(energy), f"call {call}"


def test_apply_operator_noalloc_rejects_oversized_grids(gpu_lib):
    big = 1 << 11
    rc = gpu_lib.scf_apply_operator_noalloc(big, big, big, *([C.c_void_p(8)] * 6), None, None)
    assert rc == capi.SCF_ERR_BAD_ARG
