"""The CLSVOF transport kernels' bodies (simcoflow3d_gb300/csrc/
transport_body.cuh) compiled for the host with every index range-checked
(tests/transport_host.cpp drives them over the kernels' thread indices),
against the oracle, bit for bit: Clsvof_Scheme on six cases and
ComputeUVWLiquidField on two.  Also on the host build: the same runs under
AddressSanitizer and UBSan; the independence of the results from the ulp
the math library's cbrt and log return (so the device reproduces them);
the Python front end (transport.py) and bench.py's transport leg over a
stand-in library that unpacks the C ABI's structs into the host build.  CPU
only; the device runs are in test_gpu_vof_transport.py."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    out = str(tmp_path_factory.mktemp("transport_host") / "libtransport_host.so")
    cmd = [cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "simcoflow3d_gb300", "csrc"), os.path.join(HERE, "transport_host.cpp"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(out)
    dp = C.POINTER(C.c_double)
    L.host_clsvof_step.argtypes = [C.c_int] * 3 + [dp * 6, dp, dp, dp, dp, dp, dp * 3, dp * 3, dp * 3, dp * 6,
                                                    dp * 6, C.c_int * 6, C.c_double * 6, C.c_int * 6,
                                                    C.c_double * 6, C.c_double]
    L.host_uvw.argtypes = [C.c_int] * 3 + [dp * 3, dp * 5, dp * 9, dp * 15]
    return L


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def host_step(L, centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, lvs=((1,) * 6, (0.0,) * 6),
              vofb=((1,) * 6, (0.0,) * 6)):
    I, J, K = spacings[0].shape
    keep = [np.asfortranarray(a, dtype=np.float64) for a in (*centres, *spacings, *fn, *vel, *bc_vel)]
    dp = C.POINTER(C.c_double)
    shapes = [(J, K), (J, K), (I, K), (I, K), (I, J), (I, J)]
    vof_bc = [np.zeros(sh, order="F") for sh in shapes]
    rc = L.host_clsvof_step(I, J, K, (dp * 6)(*[_p(a) for a in keep[:6]]), _p(state["vofl"]), _p(state["phil"]),
                            _p(state["nxl"]), _p(state["nyl"]), _p(state["nzl"]),
                            (dp * 3)(*[_p(a) for a in keep[6:9]]), (dp * 3)(*[_p(a) for a in keep[9:12]]),
                            (dp * 3)(*[_p(a) for a in keep[12:15]]), (dp * 6)(*[_p(a) for a in lvs_bc]),
                            (dp * 6)(*[_p(a) for a in vof_bc]), (C.c_int * 6)(*lvs[0]), (C.c_double * 6)(*lvs[1]),
                            (C.c_int * 6)(*vofb[0]), (C.c_double * 6)(*vofb[1]), float(dt))
    assert rc == 0
    return vof_bc


def _case(kind):
    """Inputs of one Clsvof_Scheme call: a tilted plane in a uniform
    stream, a drop in a shear, a plane at rest with Dirichlet planes, or a
    drop in a random (divergent) velocity field, on grids whose spacings are
    not powers of two -- or ("pow2") the random case on a 16x8x16 grid whose
    spacings are, so that every division by a spacing takes the exact
    reciprocal product."""
    I, J, K = {"plane": (12, 9, 10), "rest": (12, 9, 10), "pow2": (16, 8, 16)}.get(kind, (13, 12, 11))
    h = np.array([1.0 / I, 1.0 / J, 1.0 / K])
    cs = [(np.arange(m) + 0.5) * hq for m, hq in zip((I, J, K), h)]
    cg = [(np.arange(m + 2) - 0.5) * hq for m, hq in zip((I, J, K), h)]
    centres = tuple(np.asfortranarray(a) for a in np.meshgrid(*cs, indexing="ij"))
    spacings = tuple(np.full((I, J, K), hq, order="F") for hq in h)
    Xg, Yg, Zg = np.meshgrid(*cg, indexing="ij")
    g = Xg.shape
    rng = np.random.default_rng({"plane": 1, "rest": 2, "shear": 3, "random": 4, "pow2": 7}[kind])
    if kind in ("plane", "rest"):
        n = np.array([1.0, 0.15, -0.1]) if kind == "rest" else np.array([1.0, 0.0, 0.15])
        n /= np.linalg.norm(n)
        phi = n[0] * (Xg - 0.5) + n[1] * (Yg - 0.5) + n[2] * (Zg - 0.5)
        from simcoflow3d_gb300 import workloads as W
        s = phi + 0.5 * (np.abs(n) * h).sum()
        vof = 1.0 - W.volume_fraction_calc(h[0], h[1], h[2], n[0], n[1], n[2], s) / h.prod()
        fn = [np.full(g, n[q]) for q in range(3)]
    else:
        r = np.sqrt((Xg - 0.48) ** 2 + (Yg - 0.52) ** 2 + (Zg - 0.5) ** 2)
        phi = r - 0.24
        sub = (np.arange(4) + 0.5) / 4 - 0.5
        vof = np.zeros(g)
        for a in sub:
            for b in sub:
                for d in sub:
                    vof += np.sqrt((Xg + a * h[0] - 0.48) ** 2 + (Yg + b * h[1] - 0.52) ** 2 +
                                   (Zg + d * h[2] - 0.5) ** 2) < 0.24
        vof /= 64.0
        fn = [rng.normal(size=g) for _ in range(3)]
    vof = np.where(vof <= 1e-14, 0.0, np.where(vof >= 1 - 1e-14, 1.0, vof))
    if kind == "plane":
        vel = [np.full(g, 0.9), np.zeros(g), np.zeros(g)]
    elif kind == "rest":
        vel = [np.zeros(g) for _ in range(3)]
    elif kind == "shear":
        vel = [0.6 * np.sin(2 * np.pi * Yg), 0.3 * np.cos(2 * np.pi * Zg), 0.2 * np.sin(2 * np.pi * Xg)]
    else:
        vel = [rng.uniform(-0.8, 0.8, g) for _ in range(3)]
    vel = [np.asfortranarray(v) for v in vel]
    state = {"vofl": np.asfortranarray(vof), "phil": np.asfortranarray(phi)}
    for key in ("nxl", "nyl", "nzl"):
        state[key] = np.asfortranarray(rng.normal(size=g) * 0.1)
    shapes = [(J, K), (J, K), (I, K), (I, K), (I, J), (I, J)]
    lvs_bc = [np.asfortranarray(rng.normal(size=sh) * 0.1) for sh in shapes]
    bc_vel = [np.asfortranarray(vel[0][0, 1:-1, 1:-1]), np.asfortranarray(vel[1][1:-1, 0, 1:-1]),
              np.asfortranarray(vel[2][1:-1, 1:-1, 0])]
    fn = [np.asfortranarray(a) for a in fn]
    dt = 0.4 * h.min()
    flags = ((1, 1, 0, 1, 1, 1), (0.0, 0.0, 0.7, 0.3, 0.0, 0.0)) if kind == "rest" else ((1,) * 6, (0.0,) * 6)
    vflags = ((1, 1, 1, 1, 0, 1), (0.0, 0.0, 0.0, 0.0, 0.25, 0.1)) if kind == "rest" else ((1,) * 6, (0.0,) * 6)
    return centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags, vflags


def _deformation_case(n=24):
    """bench.py's transport workload (the reference AdvectionTest's 3-D
    deformation test, Dirichlet walls on every face) at n^3, in _case's
    order."""
    import sys
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, fl = bench.clsvof_workload(n)
    return (centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, (fl["lvs_flag"], fl["lvs_const"]),
            (fl["vof_flag"], fl["vof_const"]))


def _copy(state, planes):
    return {k: v.copy(order="F") for k, v in state.items()}, [p.copy(order="F") for p in planes]


@pytest.mark.parametrize("kind", ["plane", "rest", "shear", "random", "pow2", "deformation"])
def test_kernel_bodies_match_the_oracle(host_lib, kind):
    centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags, vflags = (
        _deformation_case() if kind == "deformation" else _case(kind))
    s_ref, p_ref = _copy(state, lvs_bc)
    s_got, p_got = _copy(state, lvs_bc)
    v_ref = O.clsvof_scheme(centres, spacings, s_ref, vel, fn, bc_vel, p_ref, dt, lvs_flag=flags[0],
                            lvs_const=flags[1], vof_flag=vflags[0], vof_const=vflags[1])
    v_got = host_step(host_lib, centres, spacings, s_got, vel, fn, bc_vel, p_got, dt, flags, vflags)
    for key in ("vofl", "phil", "nxl", "nyl", "nzl"):
        np.testing.assert_array_equal(s_got[key], s_ref[key], err_msg=key)
    for q in range(6):
        np.testing.assert_array_equal(p_got[q], p_ref[q], err_msg=f"lvs plane {q}")
        np.testing.assert_array_equal(v_got[q], v_ref[q], err_msg=f"vof plane {q}")
    inner = s_ref["vofl"][1:-1, 1:-1, 1:-1]
    assert ((inner > 0) & (inner < 1)).sum() > 30


def _uvw_case(seed):
    """A drop on a stretched grid: P cells' liquid fields and three
    families of velocity cells with their own spacings and prior fields."""
    from test_clsvof_oracle import _fields
    rng = np.random.default_rng(seed)
    I, J, K = 11, 9, 10
    gx = np.cumsum(rng.uniform(0.8, 1.2, I)); gx /= gx[-1]
    dx1 = np.diff(np.concatenate([[0.0], gx]))
    pgrid = (np.asfortranarray(np.broadcast_to(dx1[:, None, None], (I, J, K)).copy()),
             np.full((I, J, K), 1.0 / J, order="F"), np.full((I, J, K), 1.0 / K, order="F"))
    g = (I + 2, J + 2, K + 2)
    n = rng.normal(size=(3,) + g)
    n /= np.linalg.norm(n, axis=0)
    pcell = {"phil": np.asfortranarray(rng.normal(size=g) * 0.1), "nxl": np.asfortranarray(n[0]),
             "nyl": np.asfortranarray(n[1]), "nzl": np.asfortranarray(n[2]),
             "vofl": np.asfortranarray(rng.uniform(0, 1, g))}
    vgrids = [tuple(np.asfortranarray(a * rng.uniform(0.9, 1.1, a.shape)) for a in pgrid) for _ in range(3)]
    vcells = [{k: np.asfortranarray(rng.normal(size=g)) for k in ("phil", "nxl", "nyl", "nzl")} for _ in range(3)]
    for c in vcells:
        c["vofl"] = np.asfortranarray(rng.uniform(0.0, 1.0, size=g))
        c["vof"] = np.asfortranarray(rng.uniform(0.0, 1.0, size=g))
    return pgrid, pcell, vgrids, vcells


@pytest.mark.parametrize("seed", [5, 6])
def test_uvw_bodies_match_the_oracle(host_lib, seed):
    """k_uvw's bodies over its thread indices equal the oracle's
    ComputeUVWLiquidField bit for bit, shifted direction averages and the
    V and W cells' quirks included.  The oracle's clamp of vof + vofL <= 1
    changes nothing the loops do not overwrite, which this checks too: the
    velocity cells' vof is random here and the outputs still agree."""
    pgrid, pcell, vgrids, vcells = _uvw_case(seed)
    ref = [{k: v.copy(order="F") for k, v in c.items()} for c in vcells]
    O.uvw_liquid_field(pgrid, pcell, vgrids, ref)
    got = [{k: v.copy(order="F") for k, v in c.items()} for c in vcells]
    I, J, K = pgrid[0].shape
    dp = C.POINTER(C.c_double)
    outs = [got[f][k] for f in range(3) for k in ("phil", "nxl", "nyl", "nzl", "vofl")]
    vg = [a for f in range(3) for a in vgrids[f]]
    pf = [pcell[k] for k in ("phil", "nxl", "nyl", "nzl", "vofl")]
    assert host_lib.host_uvw(I, J, K, (dp * 3)(*[_p(a) for a in pgrid]), (dp * 5)(*[_p(a) for a in pf]),
                             (dp * 9)(*[_p(a) for a in vg]), (dp * 15)(*[_p(a) for a in outs])) == 0
    for f in range(3):
        for k in ("phil", "nxl", "nyl", "nzl", "vofl"):
            np.testing.assert_array_equal(got[f][k], ref[f][k], err_msg=f"family {f} {k}")


class _HostLib:
    """The scf_clsvof_* entry points the front end calls, served by the host
    build of the kernel bodies: it unpacks the same ctypes structs the real
    library reads, so the CPU checks simcoflow3d_gb300/transport.py's
    marshalling.  (State stays in the caller's arrays: fetch is a no-op.)"""

    def __init__(self, L):
        self.L = L
        self.staged = None

    def scf_clsvof_create(self, pctx, I, J, K, device):
        pctx._obj.value = 1
        self.shape = (I, J, K)
        return 0

    def scf_clsvof_destroy(self, ctx):
        return 0

    def scf_clsvof_last_error(self, ctx, buf, n):
        return 0

    def _step(self, sin, sst):
        from simcoflow3d_gb300 import capi
        I, J, K = self.shape
        dp = C.POINTER(C.c_double)
        geo = (dp * 6)(sin.x, sin.y, sin.z, sin.dx, sin.dy, sin.dz)
        rc = self.L.host_clsvof_step(I, J, K, geo, sst.vofl, sst.phil, sst.nxl, sst.nyl, sst.nzl,
                                     (dp * 3)(sin.nx, sin.ny, sin.nz), (dp * 3)(sin.u, sin.v, sin.w),
                                     (dp * 3)(sin.bc_u_w, sin.bc_v_s, sin.bc_w_b), sst.lvs_bc, sst.vof_bc,
                                     (C.c_int * 6)(*sin.lvs_flag), (C.c_double * 6)(*sin.lvs_const),
                                     (C.c_int * 6)(*sin.vof_flag), (C.c_double * 6)(*sin.vof_const), sin.dt)
        assert isinstance(sin, capi.ScfClsvofIn) and rc == 0

    def scf_clsvof_step(self, ctx, pin, pstate, pstats):
        self._step(pin._obj, pstate._obj)
        pstats._obj.steps, pstats._obj.gpu_launches = 1, 66
        return 0

    def scf_clsvof_stage(self, ctx, pin, pstate):
        from simcoflow3d_gb300 import capi
        self.staged = (capi.ScfClsvofIn.from_buffer_copy(pin._obj), capi.ScfClsvofState.from_buffer_copy(pstate._obj))
        return 0

    def scf_clsvof_run(self, ctx, steps, pstats):
        for _ in range(steps):
            self._step(*self.staged)
        pstats._obj.steps, pstats._obj.gpu_launches = steps, 66 * steps
        return 0

    def scf_clsvof_fetch(self, ctx, pstate, pstats):
        return 0

    def scf_clsvof_uvw_liquid_field(self, ctx, cells, pstats):
        I, J, K = self.shape
        sin, sst = self.staged
        dp = C.POINTER(C.c_double)
        vg = [p for f in range(3) for p in (cells[f].dx, cells[f].dy, cells[f].dz)]
        vf = [p for f in range(3) for p in (cells[f].phil, cells[f].nxl, cells[f].nyl, cells[f].nzl, cells[f].vofl)]
        assert self.L.host_uvw(I, J, K, (dp * 3)(sin.dx, sin.dy, sin.dz),
                               (dp * 5)(sst.phil, sst.nxl, sst.nyl, sst.nzl, sst.vofl), (dp * 9)(*vg),
                               (dp * 15)(*vf)) == 0
        pstats._obj.gpu_launches = 3
        return 0


def test_front_end_marshals_like_the_oracle(host_lib):
    """ClsvofScheme (the Python front end of scf_clsvof.h) over the host
    bodies: one step, then two resident steps, then ComputeUVWLiquidField,
    each equal to the oracle's."""
    from simcoflow3d_gb300.transport import ClsvofScheme
    centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags, vflags = _case("shear")
    kw = dict(lvs_flag=flags[0], lvs_const=flags[1], vof_flag=vflags[0], vof_const=vflags[1])
    I, J, K = spacings[0].shape
    fake = _HostLib(host_lib)
    sch = ClsvofScheme(I, J, K, lib=fake)
    s_got, p_got = _copy(state, lvs_bc)
    v_got, st = sch(centres, spacings, s_got, vel, fn, bc_vel, p_got, dt, **kw)
    assert st["gpu_launches"] == 66
    s_ref, p_ref = _copy(state, lvs_bc)
    v_ref = O.clsvof_scheme(centres, spacings, s_ref, vel, fn, bc_vel, p_ref, dt, **kw)
    for key in s_ref:
        np.testing.assert_array_equal(s_got[key], s_ref[key], err_msg=key)
    for q in range(6):
        np.testing.assert_array_equal(p_got[q], p_ref[q])
        np.testing.assert_array_equal(v_got[q], v_ref[q])
    sch.stage(centres, spacings, s_got, vel, fn, bc_vel, p_got, dt, **kw)
    assert sch.run(2)["gpu_launches"] == 132
    sch.fetch(s_got, p_got)
    for _ in range(2):
        O.clsvof_scheme(centres, spacings, s_ref, vel, fn, bc_vel, p_ref, dt, **kw)
    for key in s_ref:
        np.testing.assert_array_equal(s_got[key], s_ref[key], err_msg=key)
    # the velocity cells from the staged (advanced) P cells
    rng = np.random.default_rng(9)
    g = (I + 2, J + 2, K + 2)
    vgrids = [tuple(np.asfortranarray(a * rng.uniform(0.9, 1.1, a.shape)) for a in spacings) for _ in range(3)]
    vcells = [{k: np.asfortranarray(rng.normal(size=g)) for k in ("phil", "nxl", "nyl", "nzl", "vofl")}
              for _ in range(3)]
    ref = [{k: v.copy(order="F") for k, v in c.items()} for c in vcells]
    for c in ref:
        c["vof"] = np.zeros(g, order="F")
    O.uvw_liquid_field(spacings, {k: s_ref[k] for k in ("phil", "nxl", "nyl", "nzl", "vofl")}, vgrids, ref)
    assert sch.uvw_liquid_field(vgrids, vcells)["gpu_launches"] == 3
    for f in range(3):
        for k in ("phil", "nxl", "nyl", "nzl", "vofl"):
            np.testing.assert_array_equal(vcells[f][k], ref[f][k], err_msg=f"family {f} {k}")
    sch.close()


def test_front_end_rejects_wrong_shapes_before_the_c_side(host_lib):
    """A wrongly sized array raises ValueError (also under ``python -O``)
    before any pointer reaches the library, for the step's inputs, its state
    and the velocity-cell fields."""
    from simcoflow3d_gb300.transport import ClsvofScheme
    centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags, vflags = _case("shear")
    I, J, K = spacings[0].shape
    calls = []

    class Spy(_HostLib):
        def __getattribute__(self, name):
            if name in ("scf_clsvof_step", "scf_clsvof_stage", "scf_clsvof_uvw_liquid_field"):
                calls.append(name)
            return object.__getattribute__(self, name)

    sch = ClsvofScheme(I, J, K, lib=Spy(host_lib))
    short = np.asfortranarray(spacings[0][:-1])
    with pytest.raises(ValueError):
        sch(centres, (short, spacings[1], spacings[2]), *_copy(state, lvs_bc)[:1], vel, fn, bc_vel,
            _copy(state, lvs_bc)[1], dt)
    s_bad, p_bad = _copy(state, lvs_bc)
    s_bad["phil"] = np.asfortranarray(s_bad["phil"][:, :, :-1])
    with pytest.raises(ValueError):
        sch(centres, spacings, s_bad, vel, fn, bc_vel, p_bad, dt)
    vgrids = [tuple(spacings) for _ in range(3)]
    vcells = [{k: np.zeros((I + 1, J + 2, K + 2), order="F") for k in ("phil", "nxl", "nyl", "nzl", "vofl")}
              for _ in range(3)]
    with pytest.raises(ValueError):
        sch.uvw_liquid_field(vgrids, vcells)
    assert not calls, calls
    sch.close()


_SANITIZED_RUN = r"""
import sys, ctypes as C
sys.path[:0] = [sys.argv[2], sys.argv[3]]
import test_transport_host as T
L = C.CDLL(sys.argv[1])
dp = C.POINTER(C.c_double)
L.host_clsvof_step.argtypes = [C.c_int] * 3 + [dp * 6, dp, dp, dp, dp, dp, dp * 3, dp * 3, dp * 3, dp * 6, dp * 6,
                                                C.c_int * 6, C.c_double * 6, C.c_int * 6, C.c_double * 6, C.c_double]
L.host_uvw.argtypes = [C.c_int] * 3 + [dp * 3, dp * 5, dp * 9, dp * 15]
for kind in ("plane", "rest", "shear", "random", "pow2"):
    centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags, vflags = T._case(kind)
    s, p = T._copy(state, lvs_bc)
    T.host_step(L, centres, spacings, s, vel, fn, bc_vel, p, dt, flags, vflags)
pgrid, pcell, vgrids, vcells = T._uvw_case(5)
I, J, K = pgrid[0].shape
outs = [vcells[f][k] for f in range(3) for k in ("phil", "nxl", "nyl", "nzl", "vofl")]
vg = [a for f in range(3) for a in vgrids[f]]
pf = [pcell[k] for k in ("phil", "nxl", "nyl", "nzl", "vofl")]
assert L.host_uvw(I, J, K, (dp * 3)(*[T._p(a) for a in pgrid]), (dp * 5)(*[T._p(a) for a in pf]),
                  (dp * 9)(*[T._p(a) for a in vg]), (dp * 15)(*[T._p(a) for a in outs])) == 0
print("clean")
"""


def test_kernel_bodies_are_memory_clean(tmp_path):
    """The host build under AddressSanitizer and UBSan over every scheme
    case and the velocity cells: no out-of-bounds access, no undefined
    behaviour (the same bodies the kernels run)."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    rt = [subprocess.run([cxx, "-print-file-name=" + n], capture_output=True, text=True).stdout.strip()
          for n in ("libasan.so", "libubsan.so")]
    if not all(os.path.isabs(p) and os.path.exists(p) for p in rt):
        pytest.skip("sanitizer runtimes not installed")
    so = str(tmp_path / "libtransport_host_asan.so")
    r = subprocess.run([cxx, "-O1", "-g", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off",
                        "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer",
                        "-I" + os.path.join(ROOT, "simcoflow3d_gb300", "csrc"),
                        os.path.join(HERE, "transport_host.cpp"), "-o", so], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, LD_PRELOAD=" ".join(rt), ASAN_OPTIONS="detect_leaks=0")
    import sys
    r = subprocess.run([sys.executable, "-c", _SANITIZED_RUN, so, HERE, ROOT], capture_output=True, text=True,
                       env=env, timeout=600)
    assert r.returncode == 0 and "clean" in r.stdout, r.stderr[-3000:]
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr, r.stderr[-3000:]


class _BenchHostLib(_HostLib):
    """_HostLib plus what bench.py's transport leg calls: page-locking (a
    no-op), per-kernel timing and the step statistics, with made-up times
    so the line's arithmetic runs."""

    def __init__(self, L):
        super().__init__(L)
        self.timing = 0

    def scf_host_register(self, ptr, nbytes):
        return 0

    def scf_host_unregister(self, ptr):
        return 0

    def scf_clsvof_set_timing(self, ctx, on):
        self.timing = on
        return 0

    def scf_clsvof_run(self, ctx, steps, pstats):
        super().scf_clsvof_run(ctx, steps, pstats)
        st = pstats._obj
        st.ms_run = 1.5 * steps
        if self.timing:
            st.ms_kernels[:] = [0.4 * steps, 0.8 * steps, 0.01 * steps, 0.2 * steps]
        return 0

    def scf_clsvof_step(self, ctx, pin, pstate, pstats):
        super().scf_clsvof_step(ctx, pin, pstate, pstats)
        st = pstats._obj
        st.ms_h2d, st.ms_run, st.ms_d2h, st.ms_total, st.bytes_h2d, st.bytes_d2h = 0.5, 1.5, 0.4, 2.4, 1 << 20, 1 << 19
        return 0


def test_bench_transport_leg_runs_over_the_host_build(host_lib, monkeypatch, capsys):
    """bench.py --config clsvof at 16^3 over the host build: one JSON line
    with the contract's keys, the live roofline of the heavier kernel kind
    and the oracle's CPU baseline."""
    import json
    import sys
    import types
    sys.path.insert(0, ROOT)
    import bench
    from simcoflow3d_gb300 import projection
    fake = _BenchHostLib(host_lib)
    monkeypatch.setattr(projection, "load_library", lambda: fake)
    args = types.SimpleNamespace(n=16, warmup=3, steps=2, no_cpu=False, seed=1)
    assert bench.run_clsvof(args) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "clocks", "gpu_launches",
                "cpu_baseline"):
        assert key in line, key
    assert line["value"] == 1.5 and line["gpu_launches"] == 2 * 66 and line["unit"] == "ms/step"
    rf = line["roofline"]
    assert rf["kernel"] == "k_sweep" and rf["bytes_per_launch"] == 16 ** 3 * (40 + 2 * 56) // 3
    assert rf["achieved"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 1 << 20
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] > 0


def test_results_do_not_depend_on_the_cbrt_and_log_ulps(tmp_path):
    """x**(1/3) starts from the math library's cbrt and corrects with its
    log; the device's may differ from the host's by an ulp.  A copy of the
    bodies whose cbrt and log results are moved by -1, 0 or +1 ulp at
    random still matches the oracle bit for bit on every case, so the
    device reproduces the oracle whatever its cbrt and log return."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    src = open(os.path.join(ROOT, "simcoflow3d_gb300", "csrc", "transport_body.cuh")).read()
    jitter = ("static unsigned long long jit_state = 88172645463325252ull;\n"
              "inline double jit(double v) { jit_state ^= jit_state << 13; jit_state ^= jit_state >> 7;"
              " jit_state ^= jit_state << 17; const int r = (int)(jit_state % 3ull);"
              " return r == 0 ? v : r == 1 ? nextafter(v, INFINITY) : nextafter(v, -INFINITY); }\n")
    assert src.count("const double c = cbrt(x);") == 1 and src.count("* log(x);") == 1
    src = src.replace("namespace tr {\n", "namespace tr {\n" + jitter, 1)
    src = src.replace("const double c = cbrt(x);", "const double c = jit(cbrt(x));")
    src = src.replace("* log(x);", "* jit(log(x));")
    (tmp_path / "transport_body.cuh").write_text(src)
    so = str(tmp_path / "libjitter.so")
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off", "-I" + str(tmp_path),
                        os.path.join(HERE, "transport_host.cpp"), "-o", so], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(so)
    dp = C.POINTER(C.c_double)
    L.host_clsvof_step.argtypes = [C.c_int] * 3 + [dp * 6, dp, dp, dp, dp, dp, dp * 3, dp * 3, dp * 3, dp * 6,
                                                    dp * 6, C.c_int * 6, C.c_double * 6, C.c_int * 6,
                                                    C.c_double * 6, C.c_double]
    for kind in ("plane", "rest", "shear", "random", "pow2"):
        centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags, vflags = _case(kind)
        s_ref, p_ref = _copy(state, lvs_bc)
        O.clsvof_scheme(centres, spacings, s_ref, vel, fn, bc_vel, p_ref, dt, lvs_flag=flags[0],
                        lvs_const=flags[1], vof_flag=vflags[0], vof_const=vflags[1])
        s_got, p_got = _copy(state, lvs_bc)
        host_step(L, centres, spacings, s_got, vel, fn, bc_vel, p_got, dt, flags, vflags)
        for key in s_ref:
            np.testing.assert_array_equal(s_got[key], s_ref[key], err_msg=f"{kind} {key}")
