"""Unstructured 2D2F2V and 2D1F2V (triangle meshes) on the GPU: host side.

The reference builds an `UnstructPSpace` (src/Geometry/geo_unstruct.jl:10-38)
from a gmsh file with FiniteMesh.jl 0.3 (`read_mesh`, `mesh_connectivity_2D`;
a dependency that is not vendored with the reference), the cells with
`init_fvm` (src/Solver/solver_init.jl:540-640) and advances them with
`evolve!` US2F (src/Solver/solver_evolution.jl:945-1035), `update!` US2F
(src/Solver/solver_update.jl:414-471), triangle `step!`
(src/Solver/step_2f.jl:256-326) and `update_boundary!` US2F
(src/Solver/update_boundary.jl:575-594).  This module reads gmsh 4.1 ASCII
meshes, builds the connectivity and geometry with the conventions below and
drives the device solver (`kb_us_*` in the C ABI).

Connectivity convention (ours; FiniteMesh's ordering is not available):
faces are the triangle edges (p1, p2), (p2, p3), (p3, p1) numbered in order
of first appearance over the cells; face_cells[f] = (first cell, second cell
or -1); cell_faces[c][j] and cell_neighbors[c][j] follow the cell's edge j.
Geometry follows the reference's helpers: face normals unit_normal(p1, p2) =
(-dy, dx) / (|d| + 1e-6) (src/Geometry/geo_general.jl:230-235), oriented from
the first to the second cell (towards the cell for a boundary face,
src/Solver/solver_init.jl:620-632); face length |p2 - p1|; centre-to-edge
distances point_distance (geo_general.jl:260-267); cell centres the vertex
means and areas half the cross product.

Cell types (the reference's `cellType`): 0 interior (stepped), 1 fixed
boundary cell (never stepped), 3 boundary cell set to the mean of its two
neighbours after each step.  Type 2 (stepped, with Maxwell wall faces) is not
offered: the reference's US2F `evolve!` calls `flux_boundary_maxwell!` with 12
arguments, which no method takes (src/Flux/flux_boundary.jl:190 needs 13).
Only first-order, KFVS is covered: the reference's US2F `evolve!` computes
fluxes for `mode == :kfvs` only, and its second-order slopes divide by the
x / y offsets of neighbouring cell centres (reconstruct4!,
src/Reconstruction/reconstruction.jl:217-235), which vanish on general meshes.

2D1F2V (space "2d1f2v": `evolve!` / `update!` / `update_boundary!` US1F,
src/Solver/solver_evolution.jl:872-947, src/Solver/solver_update.jl:359-403,
src/Solver/update_boundary.jl:546-566, with the 2D1F2V triangle `step!`,
src/Solver/step_1f.jl:228-285) runs on the same device solver with b held at
zero; it is BGK only, since that `step!` reads h and b, which a 1F cell
does not have, under Shakhov.
"""
import ctypes
import math
import os
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .setup import Setup, VSpace2D, conserve_prim, gas_property, maxwellian, prim_conserve


# ------------------------------------------------------------------ mesh IO

def read_gmsh(path):
    """Points [np, 2] and triangles [nc, 3] (0-based) of a gmsh 4.1 ASCII
    mesh, in file order; other element types are ignored."""
    with open(path) as f:
        lines = [ln.strip() for ln in f]
    i = 0
    tag_to_idx, pts, tris = {}, [], []
    while i < len(lines):
        if lines[i] == "$MeshFormat":
            ver = lines[i + 1].split()[0]
            if not ver.startswith("4"):
                raise ValueError("gmsh format %s: only 4.x ASCII meshes are read" % ver)
        elif lines[i] == "$Nodes":
            nblk = int(lines[i + 1].split()[0])
            i += 2
            for _ in range(nblk):
                n = int(lines[i].split()[3])
                tags = [int(t) for t in lines[i + 1:i + 1 + n]]
                for k, t in enumerate(tags):
                    xyz = lines[i + 1 + n + k].split()
                    tag_to_idx[t] = len(pts)
                    pts.append((float(xyz[0]), float(xyz[1])))
                i += 1 + 2 * n
            continue
        elif lines[i] == "$Elements":
            nblk = int(lines[i + 1].split()[0])
            i += 2
            for _ in range(nblk):
                _, _, etype, n = (int(t) for t in lines[i].split())
                for k in range(n):
                    ids = [int(t) for t in lines[i + 1 + k].split()]
                    if etype == 2:
                        tris.append([tag_to_idx[ids[1]], tag_to_idx[ids[2]], tag_to_idx[ids[3]]])
                i += 1 + n
            continue
        i += 1
    if not tris:
        raise ValueError("%s holds no triangles" % path)
    return np.array(pts, dtype=np.float64), np.array(tris, dtype=np.int64)


def write_gmsh(path, points, triangles):
    """A gmsh 4.1 ASCII file with the points (one node block) and triangles
    (one element block), for meshes built in code."""
    n, m = len(points), len(triangles)
    with open(path, "w") as f:
        f.write("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n")
        f.write("$Nodes\n1 %d 1 %d\n2 1 0 %d\n" % (n, n, n))
        f.write("".join("%d\n" % (k + 1) for k in range(n)))
        f.write("".join("%.17g %.17g 0\n" % (x, y) for x, y in points))
        f.write("$EndNodes\n$Elements\n1 %d 1 %d\n2 1 2 %d\n" % (m, m, m))
        f.write("".join("%d %d %d %d\n" % (k + 1, a + 1, b + 1, c + 1)
                        for k, (a, b, c) in enumerate(triangles)))
        f.write("$EndElements\n")


def rectangle_mesh(nx, ny, x0=0.0, x1=1.0, y0=0.0, y1=1.0, jitter=0.0, seed=7):
    """Triangulated rectangle: nx x ny quads split along alternating
    diagonals, interior points moved by up to `jitter` of a cell."""
    rng = np.random.default_rng(seed)
    xs, ys = np.linspace(x0, x1, nx + 1), np.linspace(y0, y1, ny + 1)
    P = np.array([(x, y) for y in ys for x in xs])
    if jitter:
        dx, dy = (x1 - x0) / nx, (y1 - y0) / ny
        for j in range(1, ny):
            for i in range(1, nx):
                k = j * (nx + 1) + i
                P[k, 0] += jitter * dx * rng.uniform(-1, 1)
                P[k, 1] += jitter * dy * rng.uniform(-1, 1)
    T = []
    for j in range(ny):
        for i in range(nx):
            a, b = j * (nx + 1) + i, j * (nx + 1) + i + 1
            c, d = a + nx + 1, b + nx + 1
            if (i + j) % 2 == 0:
                T += [[a, b, d], [a, d, c]]
            else:
                T += [[a, b, c], [b, d, c]]
    return P, np.array(T, dtype=np.int64)


# ------------------------------------------------------------ connectivity

def unit_normal(p1, p2):
    """src/Geometry/geo_general.jl:230-235"""
    d = p2 - p1
    l = math.sqrt(d[0] * d[0] + d[1] * d[1]) + 1e-6
    return np.array([-d[1] / l, d[0] / l])


def point_distance(p, p1, p2):
    """src/Geometry/geo_general.jl:260-267"""
    x0, y0 = p
    x1, y1 = p1
    x2, y2 = p2
    return abs((x2 - x1) * (y1 - y0) - (x1 - x0) * (y2 - y1)) / math.sqrt(
        (x2 - x1) ** 2 + (y2 - y1) ** 2 + 1e-6)


@dataclass
class UnstructMesh:
    points: np.ndarray          # [np, 2]
    cells: np.ndarray           # [nc, 3] point indices
    face_points: np.ndarray     # [nf, 2]
    face_cells: np.ndarray      # [nf, 2], -1 where no cell
    cell_faces: np.ndarray      # [nc, 3]
    cell_neighbors: np.ndarray  # [nc, 3], -1 where no cell
    cell_center: np.ndarray     # [nc, 2]
    cell_area: np.ndarray       # [nc]
    cell_dx: np.ndarray         # [nc, 3] centre-to-edge distances
    face_center: np.ndarray     # [nf, 2]
    face_len: np.ndarray        # [nf]
    face_n: np.ndarray          # [nf, 2]
    cell_type: np.ndarray       # [nc]

    @property
    def ncell(self):
        return len(self.cells)

    @property
    def nface(self):
        return len(self.face_points)


def build_mesh(points, cells, boundary="fix"):
    """Connectivity and geometry of a triangle mesh (see the module notes);
    boundary cells get type 1 ("fix") or 3 ("extra"; a boundary cell with a
    single neighbour stays type 1)."""
    points = np.asarray(points, dtype=np.float64)
    cells = np.asarray(cells, dtype=np.int64)
    nc = len(cells)
    # edge k = 3 c + j joins (cells[c, j], cells[c, j + 1]); faces are the
    # distinct edges numbered by their first appearance in k
    ea = cells.reshape(-1)
    eb = cells[:, [1, 2, 0]].reshape(-1)
    key = np.minimum(ea, eb) * (int(ea.max(initial=0)) + 1 if nc else 1) + np.maximum(ea, eb)
    _, first, inv, cnt = np.unique(key, return_index=True, return_inverse=True, return_counts=True)
    if (cnt > 2).any():
        raise ValueError("an edge is shared by more than two triangles")
    order = np.argsort(first, kind="stable")          # unique-key slot -> face order
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    edge_face = rank[inv.reshape(-1)]                 # edge k -> face
    cf = edge_face.reshape(nc, 3)
    fk = first[order]                                 # first edge of each face
    fp = np.stack([ea[fk], eb[fk]], axis=1)
    fc = np.full((len(fk), 2), -1, dtype=np.int64)
    fc[:, 0] = fk // 3
    k = np.arange(3 * nc)
    second = k[k != fk[edge_face]]
    fc[edge_face[second], 1] = second // 3
    nb = np.where(fc[cf, 0] == np.arange(nc)[:, None], fc[cf, 1], fc[cf, 0])
    P0, P1, P2 = points[cells[:, 0]], points[cells[:, 1]], points[cells[:, 2]]
    center = (P0 + P1 + P2) / 3.0
    area = 0.5 * np.abs((P1[:, 0] - P0[:, 0]) * (P2[:, 1] - P0[:, 1])
                        - (P2[:, 0] - P0[:, 0]) * (P1[:, 1] - P0[:, 1]))
    # point_distance of the centre to each edge (src/Geometry/geo_general.jl:260-267)
    A, B = points[ea].reshape(nc, 3, 2), points[eb].reshape(nc, 3, 2)
    x0, y0 = center[:, None, 0], center[:, None, 1]
    x1, y1, x2, y2 = A[..., 0], A[..., 1], B[..., 0], B[..., 1]
    cdx = np.abs((x2 - x1) * (y1 - y0) - (x1 - x0) * (y2 - y1)) / np.sqrt(
        (x2 - x1) ** 2 + (y2 - y1) ** 2 + 1e-6)
    pa, pb = points[fp[:, 0]], points[fp[:, 1]]
    fcen = 0.5 * (pa + pb)
    flen = np.sqrt((pa[:, 0] - pb[:, 0]) ** 2 + (pa[:, 1] - pb[:, 1]) ** 2)
    # unit_normal (src/Geometry/geo_general.jl:230-235), turned towards the
    # second cell, or into the cell at a boundary face
    d = pb - pa
    ln = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + 1e-6
    fn = np.stack([-d[:, 1] / ln, d[:, 0] / ln], axis=1)
    inner = fc[:, 1] != -1
    n0 = np.where(inner[:, None], center[np.where(inner, fc[:, 1], 0)] - center[fc[:, 0]],
                  center[fc[:, 0]] - fcen)
    fn[fn[:, 0] * n0[:, 0] + fn[:, 1] * n0[:, 1] < 0] *= -1.0
    ctype = np.zeros(nc, dtype=np.int64)
    bnd = (nb == -1).any(axis=1)
    if boundary == "fix":
        ctype[bnd] = 1
    elif boundary == "extra":
        # update_boundary! US2F takes the mean of exactly two neighbours
        # (`id1, id2 = ids`, src/Solver/update_boundary.jl:585-587), which
        # throws for a corner triangle with one; such cells are held fixed
        nn = (nb != -1).sum(axis=1)
        ctype[bnd & (nn == 2)] = 3
        ctype[bnd & (nn < 2)] = 1
    else:
        raise ValueError("unstructured boundaries: 'fix' or 'extra', not %r" % boundary)
    return UnstructMesh(points, cells, fp, fc, cf, nb, center, area, cdx, fcen, flen, fn, ctype)


# ------------------------------------------------------------------ solver

@dataclass
class UnstructSolverSet:
    set: Setup
    ps: UnstructMesh
    vs: VSpace2D
    gas: object
    ib_fw: object  # (x, y) -> w
    dim: int = 2
    nf: int = 2


def unstruct_solver_set(mesh, nu=16, nv=16, umax=5.0, vmax=5.0, vmesh="rectangle", Kn=0.075,
                        Pr=1.0, inK=1.0, omega=0.72, collision="bgk", cfl=0.8, maxTime=1.0,
                        prim_at=None, space="2d2f2v", umin=None, vmin=None, case="unstructured"):
    """The reference's unstructured test setup (test/t1_2f.txt, or
    test/t1_1f.txt with space = "2d1f2v": KFVS, first order, 16 x 16
    velocities on [-5, 5]^2, Kn 0.075, Pr 1, inK 1) on `mesh`; prim_at(x, y)
    gives the initial primitive state (default: rest, lambda 1); the velocity
    box is [umin, umax] x [vmin, vmax] (umin, vmin default to -umax, -vmax)."""
    if space not in ("2d2f2v", "2d1f2v"):
        raise ValueError("unstructured spaces: 2d2f2v or 2d1f2v, not %r" % space)
    s = Setup(matter="gas", case=case, space=space, flux="kfvs",
              collision=collision, interpOrder=1, limiter="vanleer", boundary=["fix"] * 4,
              cfl=cfl, maxTime=maxTime)
    vs = VSpace2D.build(-umax if umin is None else umin, umax, nu, -vmax if vmin is None else vmin, vmax,
                        nv, type=vmesh)
    gas = gas_property(space=space, inK=inK, knudsen=Kn, prandtl=Pr, omega=omega)
    if prim_at is None:
        def prim_at(x, y):
            return np.array([1.0, 0.0, 0.0, 1.0])

    def fw(x, y):
        return prim_conserve(prim_at(x, y), gas.gamma)

    return UnstructSolverSet(s, mesh, vs, gas, fw, nf=1 if space == "2d1f2v" else 2)


def initial_cells(KS):
    """w, prim [nc, 4] and h, b [nc, nu*nv] of init_fvm on the cell centres
    (src/Solver/solver_init.jl:594-610; 2D1F2V :512-522, with b = 0)."""
    vs, gas = KS.vs, KS.gas
    u, v = vs.flat(vs.u), vs.flat(vs.v)
    W = np.array([np.asarray(KS.ib_fw(x, y), dtype=np.float64) for x, y in KS.ps.cell_center])
    # conserve_prim and maxwellian (src/Theory/theory_macro.jl:185-206,
    # src/Theory/theory_equilibrium.jl:8-25), over all cells at once
    r, m1, m2, E = W[:, 0], W[:, 1], W[:, 2], W[:, 3]
    lam = 0.5 * r / (gas.gamma - 1.0) / (E - 0.5 * (m1 * m1 + m2 * m2) / r)
    P = np.stack([r, m1 / r, m2 / r, lam], axis=1)
    H = (P[:, 0:1] * (P[:, 3:4] / np.pi)
         * np.exp(-P[:, 3:4] * ((u[None, :] - P[:, 1:2]) ** 2 + (v[None, :] - P[:, 2:3]) ** 2)))
    B = H * gas.K / 2.0 / P[:, 3:4] if KS.nf == 2 else np.zeros_like(H)
    return W, P, H, B


_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int32)
_US_SIGS = {
    "kb_us_create": [ctypes.POINTER(N.KbConfig), ctypes.c_int32, ctypes.c_int32, _I, _I, _I, _I,
                     _D, _D, _D, _D, _D, _D, _D, ctypes.POINTER(ctypes.c_void_p)],
    "kb_us_destroy": [ctypes.c_void_p],
    "kb_us_upload": [ctypes.c_void_p, _D, _D, _D, _D],
    "kb_us_download": [ctypes.c_void_p, _D, _D, _D, _D],
    "kb_us_timestep": [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double, _D],
    "kb_us_step": [ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, _D],
    "kb_us_info": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)],
    "kb_us_stream": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)],
    "kb_us_set_tuning": [ctypes.c_void_p, ctypes.c_int32],
    "kb_us_get_tuning": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)],
}


def _lib():
    lib = N.load()
    for name, args in _US_SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    return lib


def mesh_arrays(m):
    """The index and geometry arrays kb_us_create takes, in its types."""
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    return [i32(m.face_cells), i32(m.cell_faces), i32(m.cell_neighbors), i32(m.cell_type),
            f64(m.face_n), f64(m.face_len), f64(m.cell_area), f64(m.cell_dx.min(axis=1))]


class UnstructHandle:
    """Owner of one kb_us_t (the device cells and faces of one mesh solve)."""

    def __init__(self, KS, precision="fp64"):
        self.lib = _lib()
        self.KS = KS
        m, vs, gas = KS.ps, KS.vs, KS.gas
        c = N.KbConfig()
        c.dim, c.nx, c.ny, c.nu, c.nv = 2, m.ncell, 1, vs.nu, vs.nv
        c.flux = N.FLUX[KS.set.flux]
        c.collision = N.COLLISION[KS.set.collision]
        c.interp_order = KS.set.interpOrder
        c.precision = N.PRECISION[precision]
        c.umax, c.vmax = vs.u1, vs.v1
        c.K, c.gamma, c.mu_ref, c.omega, c.Pr = gas.K, gas.gamma, gas.mu_ref, gas.omega, gas.Pr
        c.x0, c.x1, c.y0, c.y1 = 0.0, 1.0, 0.0, 1.0
        c.nf = KS.nf
        self.cfg = c
        self.nvel = vs.nu * vs.nv
        self.ncell = m.ncell
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self._keep = mesh_arrays(m) + [f64(vs.flat(vs.u)), f64(vs.flat(vs.v)),
                                        f64(vs.flat(vs.weights))]
        k = self._keep
        h = ctypes.c_void_p()
        N.check(self.lib.kb_us_create(ctypes.byref(c), m.ncell, m.nface,
                                      *[a.ctypes.data_as(_I) for a in k[:4]],
                                      *[N.ptr(a) for a in k[4:]], ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.kb_us_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, w, prim, h, b):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (w, prim, h, b)]
        for x, n in zip(a, (4, 4, self.nvel, self.nvel)):
            if x.shape != (self.ncell, n):
                raise ValueError("upload: expected [%d, %d], got %s" % (self.ncell, n, x.shape))
        N.check(self.lib.kb_us_upload(self.h, *[N.ptr(x) for x in a]))

    def download(self):
        w = np.zeros((self.ncell, 4))
        p = np.zeros((self.ncell, 4))
        h = np.zeros((self.ncell, self.nvel))
        b = np.zeros((self.ncell, self.nvel))
        N.check(self.lib.kb_us_download(self.h, N.ptr(w), N.ptr(p), N.ptr(h), N.ptr(b)))
        return dict(w=w, prim=p, h=h, b=b)

    def timestep(self, t=0.0):
        dt = ctypes.c_double()
        s = self.KS.set
        N.check(self.lib.kb_us_timestep(self.h, float(s.cfl), float(t), float(s.maxTime),
                                        ctypes.byref(dt)))
        return dt.value

    def step(self, dt, n=1):
        r = np.zeros(4)
        N.check(self.lib.kb_us_step(self.h, float(dt), int(n), N.ptr(r)))
        return r

    def set_tuning(self, cells_per_cta=0):
        """Stepped cells per CTA of the step kernel (0: the default)."""
        N.check(self.lib.kb_us_set_tuning(self.h, int(cells_per_cta)))

    def tuning(self):
        n = ctypes.c_int32()
        N.check(self.lib.kb_us_get_tuning(self.h, ctypes.byref(n)))
        return n.value

    def stream(self):
        """The cudaStream_t (as an int) the solve's kernels run on."""
        st = ctypes.c_void_p()
        N.check(self.lib.kb_us_stream(self.h, ctypes.byref(st)))
        return st.value or 0

    def launches(self):
        n = ctypes.c_int64()
        N.check(self.lib.kb_us_info(self.h, ctypes.byref(n)))
        return n.value


def init_fvm(KS, precision="fp64"):
    """Device cells of an unstructured solve in their init_fvm state."""
    hd = UnstructHandle(KS, precision)
    hd.upload(*initial_cells(KS))
    return hd


def solver_set_from_config(D, base_dir=".", prim_at=None):
    """SolverSet of a `key = value` config whose `mesh` names a gmsh file
    (set_geometry takes UnstructPSpace(mesh) when `mesh` is given,
    src/Geometry/geometry.jl:15-45, src/Geometry/geo_unstruct.jl:34-39; the
    mesh path is relative to the config's directory, as the reference's test
    runs from its own).  Boundary cells follow `boundary`: "fix" holds them,
    "extra" sets them to the mean of their neighbours; "maxwell" (type-2 wall
    cells) is refused, because the reference's unstructured evolve! calls
    flux_boundary_maxwell! with an argument list no method takes.  The
    initial state is prim_at(x, y), by default the reference's test state:
    the gas at rest at the config's Mach number, prim [1, Ma c, 0, 1]
    (test/test_unstructure.jl)."""
    bc = D.get("boundary", "fix")
    bc = bc[0] if isinstance(bc, (list, tuple)) else bc
    if bc == "maxwell":
        raise ValueError("unstructured Maxwell wall cells are not offered: the reference's US2F evolve! "
                         "calls flux_boundary_maxwell! with an argument list no method takes")
    if bc not in ("fix", "extra"):
        raise ValueError("unstructured boundaries: fix or extra, not %r" % bc)
    if str(D.get("flux", "kfvs")) != "kfvs" or int(D.get("interpOrder", 1)) != 1:
        raise ValueError("unstructured solves are first-order KFVS (flux = kfvs, interpOrder = 1)")
    path = D["mesh"] if os.path.isabs(D["mesh"]) else os.path.join(base_dir, D["mesh"])
    m = build_mesh(*read_gmsh(path), boundary=bc)
    space = D.get("space", "2d2f2v")
    gamma = gas_property(space=space, inK=float(D.get("inK", 1.0)), knudsen=float(D["knudsen"])).gamma
    if prim_at is None:
        c = (0.5 * gamma / 1.0) ** 0.5  # sound_speed(lambda = 1, gamma)
        p0 = np.array([1.0, c * float(D.get("mach", 0.0)), 0.0, 1.0])

        def prim_at(x, y):
            return p0

    return unstruct_solver_set(
        m, nu=int(D["nu"]), nv=int(D["nv"]), umin=float(D["umin"]), umax=float(D["umax"]),
        vmin=float(D["vmin"]), vmax=float(D["vmax"]), vmesh=D.get("vMeshType", "rectangle"),
        Kn=float(D["knudsen"]), Pr=float(D.get("prandtl", 1.0)), inK=float(D.get("inK", 1.0)),
        omega=float(D.get("omega", 0.72)), collision=D.get("collision", "bgk"), cfl=float(D["cfl"]),
        maxTime=float(D["maxTime"]), prim_at=prim_at, space=space, case=D.get("case", "unstructured"))


def initialize(config, precision="fp64", prim_at=None):
    """initialize(config) of an unstructured solve (src/Solver/solver_init.jl:
    10-48 with the UnstructPSpace of set_geometry): (KS, cells, t = 0), the
    cells an UnstructHandle in their init_fvm state.  `config` is a config
    file path or a dict (a dict's relative mesh path is taken from the
    current directory)."""
    from .setup import read_cfg
    if isinstance(config, str):
        D, base = read_cfg(config), os.path.dirname(os.path.abspath(config))
    else:
        D, base = dict(config), "."
    KS = solver_set_from_config(D, base, prim_at)
    return KS, init_fvm(KS, precision), 0.0
