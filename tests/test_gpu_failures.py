"""Failure paths of the device contexts, each made on the host: no kernel is
broken, no device memory is exhausted and no wait is cut short on the GPU.

The reference ignores the solver's ``ierr`` and stops in ``pause`` on a bad
matrix (``ProjectionP.f90:102-106,463-474``); here every failure is a status
code and the context stays usable afterwards.

* The wall-clock cap of a solve (``scf_opts.time_limit_s``) ends it with
  ``SCF_ERR_NOT_CONVERGED`` after the iteration in which it expires; the next
  call with a normal cap gives the same pressure as a fresh context.
* An allocation failure injected at every device allocation of every
  context's create (``scf_debug_fail_device_alloc``: the n-th allocation
  returns what ``cudaMalloc`` returns on a full GPU, and no ``cudaMalloc`` is
  made for it) gives ``SCF_ERR_OUT_OF_MEMORY`` and leaves no device buffer
  behind (``scf_debug_device_buffers``).  The adjoint's buffers, allocated on
  first use, fail all or none, and a later call succeeds.
"""
import ctypes as C

import numpy as np
import pytest

from simcoflow3d_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L(gpu_lib):
    gpu_lib.scf_debug_fail_device_alloc.argtypes = [C.c_int64]
    gpu_lib.scf_debug_fail_device_alloc.restype = C.c_int
    gpu_lib.scf_debug_device_buffers.argtypes = []
    gpu_lib.scf_debug_device_buffers.restype = C.c_int64
    for name in ("scf_geo_create", "scf_mom_create", "scf_clsvof_create"):
        getattr(gpu_lib, name).argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    for name in ("scf_geo_destroy", "scf_mom_destroy", "scf_clsvof_destroy"):
        getattr(gpu_lib, name).argtypes = [C.c_void_p]
    yield gpu_lib
    gpu_lib.scf_debug_fail_device_alloc(0)


def _proj(w, **kw):
    from simcoflow3d_gb300.projection import Projection
    return Projection.for_workload(w, **kw)


@pytest.mark.parametrize("precision", [capi.SCF_PREC_FP64, capi.SCF_PREC_MIXED])
def test_time_limit_expiry_is_not_converged_and_the_context_stays_usable(L, precision):
    from simcoflow3d_gb300.projection import ScfError
    w = W.config("c1", n=32)
    p = _proj(w, rel_tol=1e-12, precision=precision, time_limit_s=0.0)
    with pytest.raises(ScfError) as e:
        p.poisson_solve(w, want_pocoef=False)
    assert e.value.status == capi.SCF_ERR_NOT_CONVERGED
    _, pp0, st0 = p.poisson_solve(w, want_pocoef=False, allow_not_converged=True)
    assert st0["converged"] == 0 and 1 <= st0["iterations"] <= 2
    assert np.isfinite(pp0).all()
    p.set_opts(time_limit_s=3600.0)
    _, pp, st = p.poisson_solve(w, want_pocoef=False)
    assert st["converged"] == 1 and st["rel_residual"] <= 1e-12
    q = _proj(w, rel_tol=1e-12, precision=precision)
    _, pq, sq = q.poisson_solve(w, want_pocoef=False)
    assert sq["iterations"] == st["iterations"]
    assert np.array_equal(pp, pq)
    # the drop-in call hits the cap the same way and still writes finite fields
    p.set_opts(time_limit_s=0.0)
    u, v, ww, pr, _, su = p.update_puvw(w, allow_not_converged=True)
    assert su["converged"] == 0
    assert all(np.isfinite(a).all() for a in (u, v, ww, pr))
    p.close()
    q.close()


def _sweep_create_failures(L, create, destroy):
    """Creates once to count the context's device allocations, then fails
    each of them in turn; returns how many there were."""
    base = L.scf_debug_device_buffers()
    h, rc = create()
    assert rc == 0
    n = L.scf_debug_device_buffers() - base
    assert n > 0
    destroy(h)
    assert L.scf_debug_device_buffers() == base
    for nth in range(1, n + 1):
        assert L.scf_debug_fail_device_alloc(nth) == 0
        h, rc = create()
        L.scf_debug_fail_device_alloc(0)
        assert rc == capi.SCF_ERR_OUT_OF_MEMORY, (nth, rc)
        assert not h.value
        assert L.scf_debug_device_buffers() == base, nth
    h, rc = create()     # and a normal create works afterwards
    assert rc == 0
    destroy(h)
    assert L.scf_debug_device_buffers() == base
    return n


@pytest.mark.parametrize("precision", [capi.SCF_PREC_FP64, capi.SCF_PREC_MIXED])
def test_projection_create_fails_cleanly_at_every_allocation(L, precision):
    from simcoflow3d_gb300.projection import default_opts

    def create():
        h = C.c_void_p()
        o = default_opts(precision=precision)
        return h, L.scf_ctx_create(C.byref(h), 12, 10, 9, C.byref(o))

    n = _sweep_create_failures(L, create, L.scf_ctx_destroy)
    assert n >= 60


@pytest.mark.parametrize("name", ["scf_geo", "scf_mom", "scf_clsvof"])
def test_other_contexts_fail_cleanly_at_every_allocation(L, name):
    cr, de = getattr(L, name + "_create"), getattr(L, name + "_destroy")

    def create():
        h = C.c_void_p()
        return h, cr(C.byref(h), 10, 9, 8, 0)

    assert _sweep_create_failures(L, create, de) >= 10


def test_adjoint_buffers_fail_all_or_none(L):
    from simcoflow3d_gb300.projection import ScfError
    w = W.config("c1", n=12)
    p = _proj(w, rel_tol=1e-12)
    g = W.pressure_force_weights(w)
    base = L.scf_debug_device_buffers()
    for nth in (1, 4, 8):
        L.scf_debug_fail_device_alloc(nth)
        with pytest.raises(ScfError) as e:
            p.loss_forward(w, g)
        L.scf_debug_fail_device_alloc(0)
        assert e.value.status == capi.SCF_ERR_OUT_OF_MEMORY
        assert L.scf_debug_device_buffers() == base
    jp, jd = p.loss_forward(w, g)[:2]
    assert np.isfinite(jp) and np.isfinite(jd)
    assert L.scf_debug_device_buffers() == base + 8
    q = _proj(w, rel_tol=1e-12)
    assert q.loss_forward(w, g)[:2] == (jp, jd)
    p.close()
    q.close()
