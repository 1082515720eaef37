"""Parity at the full sizes of the named configurations, through the C ABI.

Each case solves one projection on the device and compares it with the
oracle's literal restatement of the reference path at the same size:

* ``PoCoef`` (``ProjectionP.f90:123-265``) bit for bit;
* the relative residual of the device pressure in the reference's own matrix
  (the oracle's literal CSR system, ``ProjectionP.f90:301-576``) within the
  stated tolerance (the reference's HYPRE solve is asked for the same);
* the pressure against the oracle's FP64 solve to 1e-13 (relative L2,
  mean-aligned for the all-Neumann systems), within the bound in CASES;
* u, v, w, p bit for bit with the oracle's correction and boundary
  conditions given the device pressure (``ComputePUVW.f90:179-384``), and
  the corrected velocity against the oracle's own (its 1e-13 pressure).

Cases: c0 64^3 and c1 128^3 in FP64 to 1e-10; c2 256^3 in FP64 to 1e-10 and
mixed precision to 1e-8; c4 512x256x256 mixed to 1e-8.  The error bounds are
the errors measured on GB300 with a margin of about ten (c0 FP64: p 1.5e-10,
u 6.6e-11; c1: 1.5e-10, 3.1e-11; c2 FP64: 5.8e-10, 5.4e-11; c2 mixed:
8.9e-8, 1.1e-8; c4 mixed: 3.9e-9, 5.9e-9): they pin the accuracy the solve
reaches at each size rather than a size-independent rule.
"""
import numpy as np
import pytest

from simcoflow3d_gb300 import capi, workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64, MIXED = capi.SCF_PREC_FP64, capi.SCF_PREC_MIXED

# (config, precision, tolerance, bound on the pressure error, bound on the velocity error)
CASES = [
    ("c0", FP64, 1e-10, 2e-9, 1e-9),
    ("c1", FP64, 1e-10, 2e-9, 5e-10),
    ("c2", FP64, 1e-10, 6e-9, 6e-10),
    ("c2", MIXED, 1e-8, 1e-6, 1.2e-7),
    ("c4", MIXED, 1e-8, 4e-8, 6e-8),
]

_REF = {}


def _reference(name):
    """Workload and oracle projection (FP64 GMG-PCG to 1e-13), computed
    once per configuration."""
    if name not in _REF:
        _REF.clear()     # keep one full-size configuration in host memory
        w = W.config(name)
        _REF[name] = (w, O.project(w, rel_tol=1e-13))
    return _REF[name]


@pytest.mark.parametrize("name,precision,tol,p_bound,u_bound", CASES,
                         ids=[f"{c[0]}-{'fp64' if c[1] == FP64 else 'mixed'}" for c in CASES])
def test_full_size_projection_against_the_oracle(gpu_lib, name, precision, tol, p_bound, u_bound):
    from simcoflow3d_gb300.projection import Projection
    w, ref = _reference(name)
    assert ref["stats"]["csr_relres"] <= 2e-13
    p = Projection.for_workload(w, rel_tol=tol, precision=precision)
    try:
        pc, pp, st = p.poisson_solve(w)
        assert st["converged"] == 1 and st["rel_residual"] <= tol
        assert np.array_equal(pc, ref["pocoef"], equal_nan=True), "PoCoef differs from the oracle"
        act = w.arrays["posnu"] >= 0
        x = np.zeros(w.ext_cell + 1)
        x[w.arrays["posnu"][act]] = pp[1:-1, 1:-1, 1:-1][act]
        rr = O.csr_relres(ref["A"], ref["b"], x, ref["singular"])
        assert rr <= 1.05 * tol + 1e-14, rr
        err_p = O.pressure_error(w, pp, ref["pp"], ref["singular"])
        assert err_p <= p_bound, err_p
        # the drop-in call: correction + BCs + mass fix, bit-exact given the
        # device pressure (the solve is deterministic, so it is the same p)
        u, v, ww, pr, bc, su = p.update_puvw(w)
        assert su["iterations"] == st["iterations"]
        ru, rv, rw, rp_, rbc, rc = O.correct(w, pc, pp)
        assert rc == 0
        for a, b in ((u, ru), (v, rv), (ww, rw), (pr, rp_)):
            assert np.array_equal(a, b, equal_nan=True)
        for f in range(4):
            for q in range(6):
                assert np.array_equal(bc[f][q], rbc[f][q], equal_nan=True)
        err_u = O.velocity_error((u, v, ww), (ref["u"], ref["v"], ref["w"]))
        assert err_u <= u_bound, err_u
        print(f"{name} prec={precision}: {st['iterations']} iterations, residual {rr:.2e} in the reference's "
              f"matrix, err_p {err_p:.2e}, err_u {err_u:.2e}")
    finally:
        p.close()
