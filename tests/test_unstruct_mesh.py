"""Unstructured meshes on the host (no GPU): gmsh 4.1 round trip, the
connectivity and geometry kitgpu builds against the oracle's independent
construction, and the configurations the device solver refuses before any
CUDA call."""
import ctypes
import os

import numpy as np
import pytest

from kitgpu import _native as N
from kitgpu import unstruct as US
import oracle_us as OU


def test_gmsh_round_trip(tmp_path):
    P, T = US.rectangle_mesh(5, 4, jitter=0.2)
    path = str(tmp_path / "m.msh")
    US.write_gmsh(path, P, T)
    P2, T2 = US.read_gmsh(path)
    assert np.array_equal(P2, P) and np.array_equal(T2, T)


@pytest.mark.parametrize("bc", ["fix", "extra"])
def test_connectivity_and_geometry(bc):
    P, T = US.rectangle_mesh(7, 5, x1=2.0, jitter=0.25)
    m = US.build_mesh(P, T, boundary=bc)
    nbf = int((m.face_cells[:, 1] == -1).sum())
    assert nbf == 2 * (7 + 5)
    assert m.nface == (3 * m.ncell + nbf) // 2
    assert abs(m.cell_area.sum() - 2.0) < 1e-12
    for f in range(m.nface):  # normals point from the first to the second cell
        c1, c2 = m.face_cells[f]
        if c2 >= 0:
            assert m.face_n[f] @ (m.cell_center[c2] - m.cell_center[c1]) > 0
    # closed cells: the oriented face normals times lengths sum to ~0 (the
    # normals are (|d| + 1e-6)-scaled, as the reference's unit_normal)
    for c in range(m.ncell):
        s = np.zeros(2)
        for j in range(3):
            f = m.cell_faces[c, j]
            sg = 1.0 if (m.face_cells[f, 0] == c and m.face_cells[f, 1] != -1) else -1.0
            s += sg * m.face_n[f] * m.face_len[f]
        assert np.abs(s).max() < 1e-5
    nn = (m.cell_neighbors != -1).sum(axis=1)
    if bc == "fix":
        assert np.array_equal(m.cell_type, np.where(nn < 3, 1, 0))
    else:  # single-neighbour corners stay fixed: the two-neighbour mean needs two
        assert np.array_equal(m.cell_type, np.select([nn < 2, nn == 2], [1, 3], 0))
    # the oracle's own construction agrees cell by cell
    o = OU.UnstructOracle(P, T, m.cell_type, [0.0], [0.0], [1.0], 1.0, 5 / 3, 1e-3, 0.72, 1.0, "bgk")
    assert np.allclose(o.area, m.cell_area, rtol=1e-15, atol=0)
    assert np.allclose(o.center, m.cell_center, rtol=1e-15, atol=1e-15)
    assert np.allclose(o.dx.min(axis=1), m.cell_dx.min(axis=1), rtol=1e-14)
    for c in range(m.ncell):
        for j in range(3):
            f = m.cell_faces[c, j]
            sg = 1.0 if (m.face_cells[f, 0] == c and m.face_cells[f, 1] != -1) else -1.0
            assert o.dirc[c, j] == sg


def _create(mesh, cell_type=None, **kw):
    lib = US._lib()
    c = N.KbConfig()
    c.dim, c.nx, c.ny, c.nu, c.nv = 2, mesh.ncell, 1, 4, 4
    c.flux, c.collision, c.interp_order, c.precision = 0, 0, 1, 0
    c.K, c.gamma, c.mu_ref, c.omega, c.Pr = 1.0, 5 / 3, 1e-3, 0.72, 1.0
    for k, v in kw.items():
        setattr(c, k, v)
    keep = US.mesh_arrays(mesh)
    if cell_type is not None:
        keep[3] = np.ascontiguousarray(cell_type, dtype=np.int32)
    vel = [np.zeros(16), np.zeros(16), np.ones(16)]
    P = ctypes.POINTER(ctypes.c_int32)
    h = ctypes.c_void_p()
    return lib.kb_us_create(ctypes.byref(c), mesh.ncell, mesh.nface,
                            *[a.ctypes.data_as(P) for a in keep[:4]],
                            *[N.ptr(a) for a in keep[4:] + vel], ctypes.byref(h))


@pytest.mark.parametrize("kw", [dict(interp_order=2), dict(flux=1), dict(flux=2),
                                dict(nf=1, collision=1), dict(dim=1)],
                         ids=["second-order", "kcu", "ugks", "1f-shakhov", "1d"])
def test_refused_configurations(kw):
    m = US.build_mesh(*US.rectangle_mesh(3, 3))
    assert _create(m, **kw) == -2
    assert N.load().kb_last_error()


def test_maxwell_wall_cells_refused():
    m = US.build_mesh(*US.rectangle_mesh(3, 3))
    assert _create(m, cell_type=np.where(m.cell_type == 1, 2, m.cell_type)) == -2
    assert b"no method" in N.load().kb_last_error()


REF_MESH = os.path.join(os.environ.get("KITBASE_REF", "/root/reference"), "test", "t1.msh")


@pytest.mark.skipif(not os.path.exists(REF_MESH), reason="the reference's test mesh is not present")
def test_reference_test_mesh():
    """The reference's own unstructured test mesh (test/t1.msh, gmsh 4.1,
    read by test/test_unstructure.jl through t1_2f.txt) loads through
    read_gmsh, builds a closed triangulation of [0, 0.1] x [0, 0.3], agrees
    with the oracle's construction, and gives the step count that test takes
    (nt = maxTime / dt with maxTime 0.001, cfl 0.8, 16 x 16 velocities on
    [-5, 5]^2, a uniform gas at rest)."""
    P, T = US.read_gmsh(REF_MESH)
    assert P.shape == (403, 2) and T.shape == (724, 3)
    for bc in ("fix", "extra"):
        m = US.build_mesh(P, T, boundary=bc)
        assert abs(m.cell_area.sum() - 0.03) < 1e-15
        nbf = m.face_cells[:, 1] == -1
        on_edge = ((np.abs(m.face_center[nbf, 0]) < 1e-12) | (np.abs(m.face_center[nbf, 0] - 0.1) < 1e-12)
                   | (np.abs(m.face_center[nbf, 1]) < 1e-12) | (np.abs(m.face_center[nbf, 1] - 0.3) < 1e-12))
        assert on_edge.all()
    KS = US.unstruct_solver_set(m, maxTime=0.001)
    vs, g = KS.vs, KS.gas
    o = OU.UnstructOracle(P, T, m.cell_type, vs.flat(vs.u), vs.flat(vs.v), vs.flat(vs.weights),
                          g.K, g.gamma, g.mu_ref, g.omega, g.Pr, "bgk")
    assert np.allclose(o.dx.min(axis=1), m.cell_dx.min(axis=1), rtol=1e-14)
    o.set_state(*US.initial_cells(KS))
    dt = o.timestep(0.8, 0.0, 0.001, vs.u1, vs.v1)
    assert int(0.001 // dt) == 6


def test_1f_setup():
    """2D1F2V: gamma from inK as heat_capacity_ratio gives it
    (src/Struct/struct_property.jl:476-492), b zero in the initial cells, the
    oracle refuses Shakhov as the device does."""
    m = US.build_mesh(*US.rectangle_mesh(4, 4))
    KS = US.unstruct_solver_set(m, nu=4, nv=4, space="2d1f2v", inK=0.0)
    assert KS.nf == 1 and KS.gas.gamma == 2.0
    w, p, h, b = US.initial_cells(KS)
    assert np.all(b == 0.0) and np.all(h > 0.0)
    with pytest.raises(ValueError):
        OU.UnstructOracle(m.points, m.cells, m.cell_type, [0.0], [0.0], [1.0], 0.0, 2.0, 1e-3,
                          0.72, 1.0, "shakhov", nf=1)
    with pytest.raises(ValueError):
        US.unstruct_solver_set(m, space="1d1f1v")


@pytest.mark.parametrize("bc,coll,space", [("fix", "bgk", "2d2f2v"), ("extra", "shakhov", "2d2f2v"),
                                           ("extra", "bgk", "2d1f2v")])
def test_c_oracle_matches_numpy_oracle(bc, coll, space):
    """The multithreaded C restatement (kb_oracle_us.c) and the numpy
    restatement of the unstructured step agree on the same mesh tables to
    FP64 round-off over 8 steps (2F BGK, 2F Shakhov, 1F BGK)."""
    P, T = US.rectangle_mesh(9, 8, jitter=0.25)
    m = US.build_mesh(P, T, boundary=bc)

    def prim_at(x, y):
        r2 = (x - 0.4) ** 2 + (y - 0.6) ** 2
        return np.array([1.0 + 0.5 * np.exp(-r2 / 0.03), 0.1, -0.05, 1.0 / (1.0 + 0.3 * np.exp(-r2 / 0.03))])

    KS = US.unstruct_solver_set(m, nu=10, nv=12, collision=coll, space=space, prim_at=prim_at,
                                inK=1.0 if space == "2d2f2v" else 0.0)
    vs, g = KS.vs, KS.gas
    orcs = []
    for c_backend in (False, True):
        o = OU.UnstructOracle(P, T, m.cell_type, vs.flat(vs.u), vs.flat(vs.v), vs.flat(vs.weights),
                              g.K, g.gamma, g.mu_ref, g.omega, g.Pr, coll, nf=KS.nf)
        o.set_state(*US.initial_cells(KS))
        if c_backend:
            o.use_c()
        orcs.append(o)
    dts = [o.timestep(KS.set.cfl, 0.0, KS.set.maxTime, vs.u1, vs.v1) for o in orcs]
    assert dts[1] == pytest.approx(dts[0], rel=1e-15)
    rs = [o.step(dts[0], 8) for o in orcs]
    (w0, p0, h0, b0), (w1, p1, h1, b1) = (o.get_state() for o in orcs)
    assert np.max(np.abs(w1 - w0)) <= 1e-13 * np.max(np.abs(w0))
    assert np.max(np.abs(h1 - h0)) <= 1e-13 * np.max(np.abs(h0))
    assert np.max(np.abs(b1 - b0)) <= 1e-13 * max(np.max(np.abs(b0)), 1e-300)
    assert np.allclose(rs[1], rs[0], rtol=1e-9, atol=1e-300)


def test_inconsistent_tables_refused():
    """kb_us_create checks the tables against each other before any CUDA
    call: a neighbour list that disagrees with face_cells, an out-of-range
    face, a stepped cell without three neighbours."""
    m = US.build_mesh(*US.rectangle_mesh(4, 3))
    lib = US._lib()
    c = N.KbConfig()
    c.dim, c.nx, c.ny, c.nu, c.nv = 2, m.ncell, 1, 4, 4
    c.flux, c.collision, c.interp_order, c.precision = 0, 0, 1, 0
    c.K, c.gamma, c.mu_ref, c.omega, c.Pr, c.nf = 1.0, 5 / 3, 1e-3, 0.72, 1.0, 2
    vel = [np.zeros(16), np.zeros(16), np.ones(16)]
    P = ctypes.POINTER(ctypes.c_int32)

    def create(keep):
        h = ctypes.c_void_p()
        return lib.kb_us_create(ctypes.byref(c), m.ncell, m.nface, *[a.ctypes.data_as(P) for a in keep[:4]],
                                *[N.ptr(a) for a in keep[4:] + vel], ctypes.byref(h))

    keep = US.mesh_arrays(m)
    inner = int(np.nonzero(m.cell_type == 0)[0][0])
    bad = [a.copy() for a in keep]
    bad[2][inner, [0, 1]] = bad[2][inner, [1, 0]]  # neighbours swapped against the faces
    assert create(bad) == -1 and b"disagree" in N.load().kb_last_error()
    bad = [a.copy() for a in keep]
    bad[1][inner, 0] = m.nface  # a face index past the end
    assert create(bad) == -1 and b"out of range" in N.load().kb_last_error()
    bad = [a.copy() for a in keep]
    bnd = int(np.nonzero(m.cell_type == 1)[0][0])
    bad[3][bnd] = 0  # a boundary cell marked as stepped
    assert create(bad) == -2 and b"three neighbours" in N.load().kb_last_error()


T1_CFG = """# unstructured setup in the reference's test-config format
matter = gas
case = cavity
space = {space}
flux = kfvs
collision = bgk
nSpecies = 1
interpOrder = 1
limiter = vanleer
boundary = {bc}
cfl = 0.8
maxTime = 0.001
hasForce = false
mesh = {mesh}
umin = -5.0
umax = 5.0
nu = 16
vmin = -4.0
vmax = 5.0
nv = 12
vMeshType = rectangle
nug = 0
nvg = 0
knudsen = 0.075
mach = 0.5
prandtl = 1.0
inK = 1.0
omega = 0.72
alphaRef = 1.0
omegaRef = 0.5
"""


def test_solver_set_from_config(tmp_path):
    """A config in the reference's format with `mesh = <gmsh file>` gives
    the unstructured solver set (mesh relative to the config's directory,
    velocity box and gas from the config, the gas at rest at the config's
    Mach number); boundary = maxwell is refused with the reason."""
    P, T = US.rectangle_mesh(6, 5, jitter=0.2)
    US.write_gmsh(str(tmp_path / "m.msh"), P, T)
    (tmp_path / "u.txt").write_text(T1_CFG.format(space="2d2f2v", bc="extra", mesh="m.msh"))
    from kitgpu.setup import read_cfg
    D = read_cfg(str(tmp_path / "u.txt"))
    KS = US.solver_set_from_config(D, str(tmp_path))
    assert KS.ps.ncell == len(T) and KS.vs.nu == 16 and KS.vs.nv == 12
    assert KS.vs.v0 == -4.0 and KS.vs.v1 == 5.0 and KS.set.cfl == 0.8 and KS.nf == 2
    w, p, h, b = US.initial_cells(KS)
    assert np.allclose(p[:, 1], 0.5 * np.sqrt(0.5 * KS.gas.gamma)) and np.all(p[:, 3] == 1.0)
    assert set(np.unique(KS.ps.cell_type)) <= {0, 1, 3}
    (tmp_path / "w.txt").write_text(T1_CFG.format(space="2d2f2v", bc="maxwell", mesh="m.msh"))
    with pytest.raises(ValueError, match="Maxwell"):
        US.solver_set_from_config(read_cfg(str(tmp_path / "w.txt")), str(tmp_path))
