"""The CLSVOF interface transport on the GPU (scf_clsvof_step) against the
oracle's Clsvof_Scheme, bit for bit.  The kernels' bodies match the oracle
bit for bit on the CPU (test_transport_host.py); the device runs the same
expressions with -fmad=false, IEEE division and square root, and x**3 and
x**(1/3) correctly rounded by the same compensated code, whose result does
not depend on the ulp the device's cbrt and log return
(test_results_do_not_depend_on_the_cbrt_and_log_ulps)."""
import numpy as np
import pytest

from oracle import oracle as O

from test_transport_host import _case, _copy, _deformation_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from simcoflow3d_gb300.projection import load_library
    return load_library()


def _run_gpu(lib, case, steps=1):
    from simcoflow3d_gb300.transport import ClsvofScheme
    centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags, vflags = case
    I, J, K = spacings[0].shape
    sch = ClsvofScheme(I, J, K, lib=lib)
    try:
        vof_bc = None
        for _ in range(steps):
            vof_bc, st = sch(centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, lvs_flag=flags[0],
                             lvs_const=flags[1], vof_flag=vflags[0], vof_const=vflags[1])
        return vof_bc, st
    finally:
        sch.close()


@pytest.mark.parametrize("kind", ["plane", "rest", "shear", "random", "pow2", "deformation"])
def test_gpu_step_matches_the_oracle(lib, kind):
    case = _deformation_case() if kind == "deformation" else _case(kind)
    centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags, vflags = case
    s_ref, p_ref = _copy(state, lvs_bc)
    v_ref = O.clsvof_scheme(centres, spacings, s_ref, vel, fn, bc_vel, p_ref, dt, lvs_flag=flags[0],
                            lvs_const=flags[1], vof_flag=vflags[0], vof_const=vflags[1])
    s_got, p_got = _copy(state, lvs_bc)
    v_got, st = _run_gpu(lib, (centres, spacings, s_got, vel, fn, bc_vel, p_got, dt, flags, vflags))
    assert st["gpu_launches"] == 66 and st["steps"] == 1
    for key in ("vofl", "phil", "nxl", "nyl", "nzl"):
        np.testing.assert_array_equal(s_got[key], s_ref[key], err_msg=key)
    for q in range(6):
        np.testing.assert_array_equal(p_got[q], p_ref[q], err_msg=f"lvs plane {q}")
        np.testing.assert_array_equal(v_got[q], v_ref[q], err_msg=f"vof plane {q}")


def test_gpu_resident_steps_equal_single_calls(lib):
    """stage + run(3) + fetch on the device-resident state gives the same
    bits as three scf_clsvof_step calls (the scatter's 64-bit atomicMin
    makes the redistancing independent of the order of the atomics)."""
    from simcoflow3d_gb300.transport import ClsvofScheme
    case = _case("shear")
    centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags, vflags = case
    s_a, p_a = _copy(state, lvs_bc)
    v_a, _ = _run_gpu(lib, (centres, spacings, s_a, vel, fn, bc_vel, p_a, dt, flags, vflags), steps=3)
    s_b, p_b = _copy(state, lvs_bc)
    I, J, K = spacings[0].shape
    sch = ClsvofScheme(I, J, K, lib=lib)
    try:
        sch.stage(centres, spacings, s_b, vel, fn, bc_vel, p_b, dt)
        st = sch.run(3)
        assert st["gpu_launches"] == 3 * 66
        v_b, _ = sch.fetch(s_b, p_b)
    finally:
        sch.close()
    for key in s_a:
        np.testing.assert_array_equal(s_a[key], s_b[key], err_msg=key)
    for q in range(6):
        np.testing.assert_array_equal(p_a[q], p_b[q])
        np.testing.assert_array_equal(v_a[q], v_b[q])


def test_gpu_shear_keeps_the_liquid_volume(lib):
    """In the shear u(y), v(z), w(x) every sweep is divergence-free along
    its own axis, so the divisions and corrections are exact no-ops and a
    drop keeps its liquid volume over three steps to rounding (no liquid
    reaches a wall)."""
    case = _case("shear")
    centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags, vflags = case
    s, p = _copy(state, lvs_bc)
    before = s["vofl"][1:-1, 1:-1, 1:-1].sum()
    _run_gpu(lib, (centres, spacings, s, vel, fn, bc_vel, p, dt, flags, vflags), steps=3)
    after = s["vofl"][1:-1, 1:-1, 1:-1].sum()
    assert abs(after - before) < 1e-10 * before


@pytest.mark.parametrize("seed", [5, 6])
def test_gpu_uvw_liquid_field_matches_the_oracle(lib, seed):
    """ComputeUVWLiquidField on the device from the staged P cells, against
    the oracle, bit for bit."""
    from simcoflow3d_gb300.transport import ClsvofScheme
    from test_transport_host import _uvw_case
    pgrid, pcell, vgrids, vcells = _uvw_case(seed)
    ref = [{k: v.copy(order="F") for k, v in c.items()} for c in vcells]
    O.uvw_liquid_field(pgrid, pcell, vgrids, ref)
    I, J, K = pgrid[0].shape
    g = (I + 2, J + 2, K + 2)
    zg = np.zeros(g, order="F")
    centres = tuple(np.zeros((I, J, K), order="F") for _ in range(3))
    state = {k: pcell[k].copy(order="F") for k in ("vofl", "phil", "nxl", "nyl", "nzl")}
    planes = [np.zeros(sh, order="F") for sh in [(J, K)] * 2 + [(I, K)] * 2 + [(I, J)] * 2]
    got = [{k: v.copy(order="F") for k, v in c.items()} for c in vcells]
    sch = ClsvofScheme(I, J, K, lib=lib)
    try:
        sch.stage(centres, pgrid, state, [zg] * 3, [zg] * 3,
                  [np.zeros((J, K), order="F"), np.zeros((I, K), order="F"), np.zeros((I, J), order="F")],
                  planes, 0.0)
        st = sch.uvw_liquid_field(vgrids, got)
        assert st["gpu_launches"] == 3
    finally:
        sch.close()
    for f in range(3):
        for k in ("phil", "nxl", "nyl", "nzl", "vofl"):
            np.testing.assert_array_equal(got[f][k], ref[f][k], err_msg=f"family {f} {k}")


def test_gpu_rejects_bad_arguments(lib):
    import ctypes as C
    from simcoflow3d_gb300.projection import ScfError
    from simcoflow3d_gb300.transport import ClsvofScheme
    ctx = C.c_void_p()
    assert lib.scf_clsvof_create(C.byref(ctx), 2, 8, 8, 0) == 1
    sch = ClsvofScheme(4, 4, 4, lib=lib)
    try:
        with pytest.raises(ScfError):
            sch.run(1)   # nothing staged
    finally:
        sch.close()
