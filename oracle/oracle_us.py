"""TEST INFRASTRUCTURE ONLY: FP64 CPU restatement of KitBase.jl's
unstructured 2D2F2V DVM step (numpy, vectorised over the velocity grid; loops
over faces and cells), the checker of kitgpu's kb_us_* solver.  Only tests/
and bench.py's CPU baseline use it; the product never imports it.  use_c()
moves the step to the multithreaded C restatement (kb_oracle_us.c) on the
same mesh tables; the numpy and C forms are held to each other by
tests/test_unstruct_mesh.py.

PARITY UNPINNED: the reference cannot run here and its unstructured test
(test/test_unstructure.jl) asserts nothing.  The mesh connectivity and
geometry of the reference come from FiniteMesh.jl 0.3 (`read_mesh`,
`mesh_connectivity_2D`, `mesh_cell_type`), which is not vendored; this file
builds its own from the points and triangles, independently of kitgpu's
host code, with the reference's own helpers (unit_normal, point_distance)
restated.

Restated (file:line of the reference):
- init_fvm US2F: cell and face normals, centre-to-edge distances
  (src/Solver/solver_init.jl:580-636, src/Geometry/geo_general.jl:230-267);
- timestep for unstructured cells (src/Solver/solver_main.jl:398-420);
- evolve! US2F, KFVS branch, first-order face states
  (src/Solver/solver_evolution.jl:945-1035) with flux_kfvs! 2F2V
  (src/Flux/flux_kfvs.jl:654-700), flux_conserve! 2F2V
  (src/Theory/theory_moments.jl:409-414) and global_frame
  (src/Geometry/geo_general.jl:6-26);
- update! US2F (src/Solver/solver_update.jl:414-471) with the triangle step!
  (src/Solver/step_2f.jl:256-326), heat_flux 2F2V and shakhov 2F2V
  (src/Theory/theory_moments.jl:567-578, src/Theory/theory_equilibrium.jl:227-238);
- update_boundary! US2F (src/Solver/update_boundary.jl:575-594).
2D1F2V (nf = 1), written from the reference's 1F functions, not from the 2F
code above:
- evolve! US1F, KFVS branch (src/Solver/solver_evolution.jl:872-947) with
  flux_kfvs! 1F2V (src/Flux/flux_kfvs.jl:615-650) and flux_conserve! 1F2V;
- update! US1F (src/Solver/solver_update.jl:359-403) with the 2D1F2V triangle
  step! (src/Solver/step_1f.jl:228-285; BGK, the only collision it can run);
- update_boundary! US1F (src/Solver/update_boundary.jl:546-566).
"""
import ctypes
import math

import numpy as np


def unit_normal(p1, p2):
    d = p2 - p1
    l = np.linalg.norm(d) + 1e-6
    return np.array([-d[1], d[0]]) / l


def point_distance(p, p1, p2):
    x0, y0 = p
    x1, y1 = p1
    x2, y2 = p2
    return abs((x2 - x1) * (y1 - y0) - (x1 - x0) * (y2 - y1)) / math.sqrt(
        (x2 - x1) ** 2 + (y2 - y1) ** 2 + 1e-6)


def conserve_prim(w, g):
    """src/Theory/theory_macro.jl:185-206 (2D)"""
    return np.array([w[0], w[1] / w[0], w[2] / w[0],
                     0.5 * w[0] / (g - 1.0) / (w[3] - 0.5 * (w[1] ** 2 + w[2] ** 2) / w[0])])


def maxwellian(u, v, p):
    return p[0] * (p[3] / np.pi) * np.exp(-p[3] * ((u - p[1]) ** 2 + (v - p[2]) ** 2))


class UnstructOracle:
    """One unstructured solve: cells from (points, triangles); cell types 0
    (stepped), 1 (fixed), 3 (mean of its two neighbours)."""

    def __init__(self, points, tris, cell_type, u, v, wt, K, gamma, mu_ref, omega, Pr, coll, nf=2):
        P = np.asarray(points, dtype=np.float64)
        T = np.asarray(tris, dtype=np.int64)
        self.u, self.v, self.wt = (np.asarray(a, dtype=np.float64) for a in (u, v, wt))
        self.K, self.g, self.mu, self.om, self.Pr, self.coll = K, gamma, mu_ref, omega, Pr, coll
        self.nf = nf
        self._c = None
        if nf == 1 and coll != "bgk":
            raise ValueError("the 2D1F2V triangle step! runs BGK only")
        self.type = np.asarray(cell_type)
        nc = len(T)
        self.center = P[T].mean(axis=1)
        e1, e2 = P[T[:, 1]] - P[T[:, 0]], P[T[:, 2]] - P[T[:, 0]]
        self.area = 0.5 * np.abs(e1[:, 0] * e2[:, 1] - e2[:, 0] * e1[:, 1])
        # faces: edges keyed by their sorted point pair, cells in order of appearance
        faces = {}
        for c in range(nc):
            for j in range(3):
                a, b = int(T[c, j]), int(T[c, (j + 1) % 3])
                faces.setdefault((min(a, b), max(a, b)), []).append((c, j, a, b))
        self.faces = []   # (c1, c2 or -1, n, len)
        self.cell_face = [[None] * 3 for _ in range(nc)]
        self.nb = [[-1] * 3 for _ in range(nc)]
        for key, lst in faces.items():
            (c1, j1, a, b) = lst[0]
            c2 = lst[1][0] if len(lst) > 1 else -1
            n = unit_normal(P[a], P[b])
            fcen = 0.5 * (P[a] + P[b])
            n0 = self.center[c2] - self.center[c1] if c2 >= 0 else self.center[c1] - fcen
            if n @ n0 < 0:
                n = -n
            ln = np.linalg.norm(P[a] - P[b])
            k = len(self.faces)
            self.faces.append((c1, c2, n, ln))
            for (c, j, pa, pb) in lst:
                self.cell_face[c][j] = k
            if c2 >= 0:
                self.nb[c1][j1] = c2
                self.nb[c2][lst[1][1]] = c1
        # outward normals of each cell's edges and the orientation signs (dirc)
        self.dirc = np.zeros((nc, 3))
        self.dx = np.zeros((nc, 3))
        for c in range(nc):
            for j in range(3):
                a, b = T[c, j], T[c, (j + 1) % 3]
                n = unit_normal(P[a], P[b])
                fcen = 0.5 * (P[a] + P[b])
                if (fcen - self.center[c]) @ n < 0:
                    n = -n
                self.dirc[c, j] = np.sign(n @ self.faces[self.cell_face[c][j]][2])
                self.dx[c, j] = point_distance(self.center[c], P[a], P[b])
        self.ncell = nc

    def set_state(self, w, prim, h, b):
        self.w, self.prim, self.h, self.b = (np.array(a, dtype=np.float64) for a in (w, prim, h, b))
        if self._c is not None:
            self._c_call("kbou_set_state", *(np.ascontiguousarray(a) for a in (self.w, self.prim, self.h, self.b)))

    def get_state(self):
        if self._c is not None:
            for a in (self.w, self.prim, self.h, self.b):
                assert a.flags.c_contiguous
            self._c_call("kbou_get_state", self.w, self.prim, self.h, self.b)
        return self.w.copy(), self.prim.copy(), self.h.copy(), self.b.copy()

    # ------------------------------------------------ C backend (kb_oracle_us.c)

    def use_c(self):
        """Step through the multithreaded C restatement (kb_oracle_us.c) on
        this oracle's own mesh tables; returns self."""
        import oracle as O
        L = ctypes.CDLL(O.build())
        D, I = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)
        L.kbou_create.restype = ctypes.c_void_p
        L.kbou_create.argtypes = [ctypes.c_int, ctypes.c_int] + [I] * 4 + [D] * 5 + [ctypes.c_int] + [D] * 3 + \
            [ctypes.c_double] * 5 + [ctypes.c_int] * 2
        L.kbou_timestep.restype = ctypes.c_double
        L.kbou_timestep.argtypes = [ctypes.c_void_p] + [ctypes.c_double] * 5
        for name in ("kbou_set_state", "kbou_get_state"):
            getattr(L, name).argtypes = [ctypes.c_void_p] + [D] * 4
        L.kbou_step.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, D]
        L.kbou_destroy.argtypes = [ctypes.c_void_p]
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        nf = len(self.faces)
        self._keep = [
            i32([[c1, c2] for c1, c2, n, ln in self.faces]), i32(self.cell_face), i32(self.nb),
            i32(self.type), f64([n for c1, c2, n, ln in self.faces]), f64([ln for c1, c2, n, ln in self.faces]),
            f64(self.dirc), f64(self.area), f64(self.dx.min(axis=1)), f64(self.u), f64(self.v), f64(self.wt)]
        k = self._keep
        ptr = lambda a: a.ctypes.data_as(I if a.dtype == np.int32 else D)
        self._L = L
        self._c = L.kbou_create(self.ncell, nf, *[ptr(a) for a in k[:9]], len(self.u),
                                *[ptr(a) for a in k[9:]], self.K, self.g, self.mu, self.om, self.Pr,
                                1 if self.coll == "shakhov" else 0, self.nf)
        if hasattr(self, "w"):
            self.set_state(self.w, self.prim, self.h, self.b)
        return self

    def _c_call(self, name, *arrays):
        D = ctypes.POINTER(ctypes.c_double)
        getattr(self._L, name)(self._c, *[a.ctypes.data_as(D) for a in arrays])

    def __del__(self):
        if getattr(self, "_c", None):
            self._L.kbou_destroy(self._c)
            self._c = None

    def timestep(self, cfl, t, tmax_time, umax, vmax):
        if self._c is not None:
            return self._L.kbou_timestep(self._c, cfl, t, tmax_time, umax, vmax)
        tmax = 0.0
        for c in range(self.ncell):
            sos = (0.5 * self.g / self.prim[c, 3]) ** 0.5
            um, vm = umax + sos, vmax + sos
            tmax = max(tmax, math.sqrt(um ** 2 + vm ** 2) / self.dx[c].min())
        dt = cfl / tmax
        return dt if dt < tmax_time - t else tmax_time - t

    def evolve(self, dt):
        if self.nf == 1:
            return self._evolve_1f(dt)
        nv = len(self.u)
        self.fw = np.zeros((len(self.faces), 4))
        self.fh = np.zeros((len(self.faces), nv))
        self.fb = np.zeros((len(self.faces), nv))
        for k, (c1, c2, n, ln) in enumerate(self.faces):
            if c2 < 0:
                continue
            vn = self.u * n[0] + self.v * n[1]
            vt = self.v * n[0] - self.u * n[1]
            d = np.where(vn >= 0.0, 1.0, 0.0)
            h = self.h[c1] * d + self.h[c2] * (1.0 - d)
            b = self.b[c1] * d + self.b[c2] * (1.0 - d)
            fh = (dt * vn * h - 0.5 * dt ** 2 * vn ** 2 * 0.0) * ln
            fb = (dt * vn * b - 0.5 * dt ** 2 * vn ** 2 * 0.0) * ln
            fw = np.array([np.sum(self.wt * fh), np.sum(vn * self.wt * fh), np.sum(vt * self.wt * fh),
                           0.5 * (np.sum((vn ** 2 + vt ** 2) * self.wt * fh) + np.sum(self.wt * fb))])
            self.fw[k] = [fw[0], fw[1] * n[0] - fw[2] * n[1], fw[1] * n[1] + fw[2] * n[0], fw[3]]
            self.fh[k], self.fb[k] = fh, fb

    def update(self, dt):
        if self.nf == 1:
            return self._update_1f(dt)
        sumR, sumA = np.zeros(4), np.zeros(4)
        u, v, wt, K, Pr = self.u, self.v, self.wt, self.K, self.Pr
        for c in range(self.ncell):
            if self.type[c] not in (0, 2):
                continue
            fs = self.cell_face[c]
            dc = self.dirc[c]
            w, p, h, b = self.w[c], self.prim[c], self.h[c], self.b[c]
            w_old = w.copy()
            if self.coll == "shakhov":
                cu, cv = u - p[1], v - p[2]
                c2 = cu ** 2 + cv ** 2
                q = 0.5 * np.array([np.sum(wt * cu * c2 * h) + np.sum(wt * cu * b),
                                    np.sum(wt * cv * c2 * h) + np.sum(wt * cv * b)])
                MHo = maxwellian(u, v, p)
                MBo = MHo * K / (2.0 * p[3])
                fac = 0.8 * (1.0 - Pr) * p[3] ** 2 / p[0] * (cu * q[0] + cv * q[1])
                SH = fac * (2.0 * p[3] * c2 + K - 5.0) * MHo
                SB = fac * (2.0 * p[3] * c2 + K - 3.0) * MBo
            else:
                SH, SB = 0.0, 0.0
            w -= (self.fw[fs[0]] * dc[0] + self.fw[fs[1]] * dc[1] + self.fw[fs[2]] * dc[2]) / self.area[c]
            p[:] = conserve_prim(w, self.g)
            sumR += (w - w_old) ** 2
            sumA += np.abs(w)
            MH = maxwellian(u, v, p)
            MB = MH * K / (2.0 * p[3])
            MH = MH + SH
            MB = MB + SB
            tau = self.mu * 2.0 * p[3] ** (1.0 - self.om) / p[0]
            h[:] = (h - (self.fh[fs[0]] * dc[0] + self.fh[fs[1]] * dc[1] + self.fh[fs[2]] * dc[2])
                    / self.area[c] + dt / tau * MH) / (1.0 + dt / tau)
            b[:] = (b - (self.fb[fs[0]] * dc[0] + self.fb[fs[1]] * dc[1] + self.fb[fs[2]] * dc[2])
                    / self.area[c] + dt / tau * MB) / (1.0 + dt / tau)
        res = np.sqrt(sumR * self.ncell) / (sumA + 1.e-7)
        for c in range(self.ncell):
            if self.type[c] == 3:
                ids = [i for i in self.nb[c] if i != -1][:2]
                self.w[c] = 0.5 * (self.w[ids[0]] + self.w[ids[1]])
                self.h[c] = 0.5 * (self.h[ids[0]] + self.h[ids[1]])
                self.b[c] = 0.5 * (self.b[ids[0]] + self.b[ids[1]])
                self.prim[c] = conserve_prim(self.w[c], self.g)
        return res

    # ------------------------------------------------------------ 2D1F2V

    def _evolve_1f(self, dt):
        """evolve! US1F: ff = (dt vn f - 0.5 dt^2 vn^2 sf) len with sf = 0
        (first order), fw = (sum w ff, sum w vn ff, sum w vt ff,
        0.5 sum w (vn^2 + vt^2) ff), rotated by global_frame."""
        nv = len(self.u)
        self.fw = np.zeros((len(self.faces), 4))
        self.fh = np.zeros((len(self.faces), nv))
        self.fb = np.zeros((len(self.faces), nv))
        for k, (c1, c2, n, ln) in enumerate(self.faces):
            if c2 < 0:
                continue
            vn = self.u * n[0] + self.v * n[1]
            vt = self.v * n[0] - self.u * n[1]
            delta = np.where(vn >= 0.0, 1.0, 0.0)
            f = self.h[c1] * delta + self.h[c2] * (1.0 - delta)
            ff = (dt * vn * f) * ln
            a = np.sum(self.wt * ff)
            bn = np.sum(self.wt * vn * ff)
            bt = np.sum(self.wt * vt * ff)
            e = 0.5 * np.sum(self.wt * (vn * vn + vt * vt) * ff)
            self.fw[k] = [a, bn * n[0] - bt * n[1], bn * n[1] + bt * n[0], e]
            self.fh[k] = ff

    def _update_1f(self, dt):
        sumR, sumA = np.zeros(4), np.zeros(4)
        for c in range(self.ncell):
            if self.type[c] not in (0, 2):
                continue
            fs, dc = self.cell_face[c], self.dirc[c]
            w, p, f = self.w[c], self.prim[c], self.h[c]
            w_old = w.copy()
            w -= (self.fw[fs[0]] * dc[0] + self.fw[fs[1]] * dc[1] + self.fw[fs[2]] * dc[2]) / self.area[c]
            p[:] = conserve_prim(w, self.g)
            sumR += (w - w_old) ** 2
            sumA += np.abs(w)
            M = maxwellian(self.u, self.v, p)
            tau = self.mu * 2.0 * p[3] ** (1.0 - self.om) / p[0]
            f[:] = (f - (self.fh[fs[0]] * dc[0] + self.fh[fs[1]] * dc[1] + self.fh[fs[2]] * dc[2])
                    / self.area[c] + dt / tau * M) / (1.0 + dt / tau)
        res = np.sqrt(sumR * self.ncell) / (sumA + 1.e-7)
        for c in range(self.ncell):
            if self.type[c] == 3:
                i1, i2 = [i for i in self.nb[c] if i != -1][:2]
                self.w[c] = 0.5 * (self.w[i1] + self.w[i2])
                self.h[c] = 0.5 * (self.h[i1] + self.h[i2])
                self.prim[c] = conserve_prim(self.w[c], self.g)
        return res

    def step(self, dt, n=1):
        if self._c is not None:
            r = np.zeros(4)
            self._L.kbou_step(self._c, dt, n, r.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            return r
        res = None
        for _ in range(n):
            self.evolve(dt)
            res = self.update(dt)
        return res
