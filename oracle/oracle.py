"""CPU ORACLE -- test infrastructure, not the product.

A restatement of the reference's BEM path (squirmer-bem-3dtube):
  * geometry and panel quadrature in C (``bem_oracle.c`` -> ``_build/liboracle.so``),
  * the solver logic of ``src/swimmer.hpp``, ``src/duct_flow.hpp`` and
    ``src/trajectory.hpp`` here, with the dense algebra on scipy's LAPACK
    (``dgetrf``/``dgetrs``/``dgesv``/``dgemm``) -- the same LAPACK calls the
    reference makes through ``src/utils/linalg.hpp:17-26``.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module, and only as the checker.  It is pinned against fixtures the
reference itself wrote (``tests/golden/``, checked by ``tests/test_oracle.py``).
"""
import ctypes
import math
import os
import subprocess

import numpy as np
import scipy.linalg as sla

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
EIGHT_PI = 8.0 * math.pi
WALL, INLET, OUTLET, SPHERE = 0, 1, 2, 10


def build():
    """Compile the C restatement (make -C oracle port)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def _load():
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "bem_oracle.c")):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    D = ctypes.POINTER(ctypes.c_double)
    I = ctypes.POINTER(ctypes.c_int)
    c_d, c_i = ctypes.c_double, ctypes.c_int
    sig = {
        "orc_rule": (c_i, [c_i, D, D]),
        "orc_gauss_legendre01": (None, [c_i, D, D]),
        "orc_panel_integrals": (None, [c_i, D, D, I, D, D]),
        "orc_rule_of": (c_i, [D, D, c_i]),
        "orc_block": (None, [c_i, D, c_i, D, c_i, c_d, D, D, D]),
        "orc_velocity_at": (None, [c_i, D, D, D, c_d, c_i, D, D]),
        "orc_uniform_z": (c_i, [c_d, c_d, c_i, D]),
        "orc_graded_z": (c_i, [c_d, c_d, c_d, c_d, c_d, D, c_i]),
        "orc_tube_mesh": (c_i, [c_d, D, c_i, c_i, c_i, D, I, c_i]),
        "orc_swimmer_tube_mesh": (c_i, [c_d, c_d, c_d, c_i, c_i, D, I, c_i]),
        "orc_icosphere": (c_i, [c_d, c_i, c_d, c_d, c_d, c_i, D, I, c_i]),
        "orc_geometry": (None, [c_i, D, D, D, D, D]),
        "orc_squirmer_slip": (None, [c_i, D, D, D, c_d, c_d, D]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = _load()
    return _LIB


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _v(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


# ---------------------------------------------------------------- meshes
class Mesh:
    """Flat-triangle mesh as per-panel vertices, tags and derived geometry
    (mesh.hpp:50-91)."""

    def __init__(self, V, tags):
        self.V = np.ascontiguousarray(V, dtype=np.float64).reshape(-1, 9)
        self.tags = np.ascontiguousarray(tags, dtype=np.int32)
        self.geometry()

    def geometry(self):
        P = self.P
        self.normal = np.zeros((P, 3))
        self.centroid = np.zeros((P, 3))
        self.area = np.zeros(P)
        self.h = np.zeros(P)
        lib().orc_geometry(P, _dp(self.V), _dp(self.normal), _dp(self.centroid), _dp(self.area),
                           _dp(self.h))

    @property
    def P(self):
        return self.V.shape[0]

    def translate(self, d):
        """mesh.hpp:82-85 (nodes + d, per vertex)."""
        d = np.asarray(d, dtype=np.float64)
        self.V = self.V + np.tile(d, 3)[None, :]
        self.geometry()

    def copy(self):
        return Mesh(self.V.copy(), self.tags.copy())

    def total_area(self):
        return float(sum(self.area))


def merge(a, b):
    """mesh.hpp:95-103."""
    return Mesh(np.vstack([a.V, b.V]), np.concatenate([a.tags, b.tags]))


def _mesh_from(fn, *args):
    n = fn(*args, None, None, 0)
    V = np.zeros((n, 9))
    tags = np.zeros(n, dtype=np.int32)
    fn(*args, _dp(V), _ip(tags), n)
    return Mesh(V, tags)


def uniform_z(z0, z1, nz):
    z = np.zeros(nz + 1)
    lib().orc_uniform_z(z0, z1, nz, _dp(z))
    return z


def graded_z(L, dzmin, dzmax, core, growth=1.25):
    n = lib().orc_graded_z(L, dzmin, dzmax, core, growth, None, 0)
    z = np.zeros(n)
    lib().orc_graded_z(L, dzmin, dzmax, core, growth, _dp(z), n)
    return z


def tube_mesh(R, z, n_theta, n_r):
    z = _v(z)
    return _mesh_from(lib().orc_tube_mesh, R, _dp(z), len(z), n_theta, n_r)


def swimmer_tube_mesh(R, L, a, n_theta, n_r=4):
    return _mesh_from(lib().orc_swimmer_tube_mesh, R, L, a, n_theta, n_r)


def icosphere(a, level, center=(0.0, 0.0, 0.0), tag=SPHERE):
    return _mesh_from(lib().orc_icosphere, a, level, float(center[0]), float(center[1]),
                      float(center[2]), tag)


# ---------------------------------------------------------------- kernels
def panel_integrals(V9, x0, self_flag):
    """kernels.hpp:67-82 for arrays of (panel, target, self): returns SL, DL (n, 9)."""
    V9 = _v(V9).reshape(-1, 9)
    n = V9.shape[0]
    x0 = _v(x0).reshape(n, 3)
    sf = np.ascontiguousarray(np.broadcast_to(np.asarray(self_flag, dtype=np.int32), (n,)))
    SL = np.zeros((n, 9))
    DL = np.zeros((n, 9))
    lib().orc_panel_integrals(n, _dp(V9), _dp(x0), _ip(sf), _dp(SL), _dp(DL))
    return SL, DL


def rule_of(V9, x0, self_flag=0):
    return lib().orc_rule_of(_dp(_v(V9)), _dp(_v(x0)), int(self_flag))


def quadrature_rule(level):
    L = np.zeros((448, 3))
    W = np.zeros(448)
    n = lib().orc_rule(level, _dp(L), _dp(W))
    return L[:n].copy(), W[:n].copy()


def gauss_legendre01(n):
    x, w = np.zeros(n), np.zeros(n)
    lib().orc_gauss_legendre01(n, _dp(x), _dp(w))
    return x, w


def block(T, S, same_mesh, mu, want_S=True, want_D=True, want_sum=False):
    """One coupling block (targets = centroids of T, sources = panels of S)."""
    nT, nS = T.P, S.P
    Sb = np.zeros((3 * nT, 3 * nS), order="F") if want_S else None
    Db = np.zeros((3 * nT, 3 * nS), order="F") if want_D else None
    ds = np.zeros((nT, 9)) if want_sum else None
    lib().orc_block(nT, _dp(T.V), nS, _dp(S.V), int(same_mesh), mu, _dp(Sb), _dp(Db), _dp(ds))
    return Sb, Db, ds


def velocity_at(M, u, f, mu, points):
    """field.hpp:18-34."""
    pts = _v(points).reshape(-1, 3)
    u = _v(u).reshape(-1, 3)
    f = _v(f).reshape(-1, 3)
    out = np.zeros_like(pts)
    lib().orc_velocity_at(M.P, _dp(M.V), _dp(u), _dp(f), mu, pts.shape[0], _dp(pts), _dp(out))
    return out


def squirmer_slip(x, center, e, B1, B2):
    x = _v(x).reshape(-1, 3)
    out = np.zeros_like(x)
    lib().orc_squirmer_slip(x.shape[0], _dp(x), _dp(_v(center)), _dp(_v(e)), B1, B2, _dp(out))
    return out


# ---------------------------------------------------------------- tube
def deflate(M, p0, npan, A, off, mu):
    """Tube::deflate, swimmer.hpp:64-74 (rank-one Wielandt term)."""
    At = float(np.sum(M.area[p0:p0 + npan]))
    sc = 1.0 / (EIGHT_PI * mu * math.sqrt(At))
    n = M.normal[p0:p0 + npan].reshape(-1)
    na = (M.normal[p0:p0 + npan] * M.area[p0:p0 + npan, None]).reshape(-1)
    A[off:off + 3 * npan, off:off + 3 * npan] += sc * np.outer(n, na)


class Tube:
    """swimmer.hpp:33-75: tube mesh, single-layer block T, deflation, dgetrf."""

    def __init__(self, R, L, a, n_theta, n_r=4, mu=1.0, keep_matrix=False):
        self.R, self.L, self.mu = R, L, mu
        self.mesh = swimmer_tube_mesh(R, L, a, n_theta, n_r)
        self.Nt = self.mesh.P
        T, _, _ = block(self.mesh, self.mesh, True, mu, True, False)
        deflate(self.mesh, 0, self.Nt, T, 0, mu)
        if keep_matrix:
            self.T = T.copy(order="F")
        self.lu = sla.lu_factor(T, overwrite_a=True, check_finite=False)

    def solve(self, B):
        return sla.lu_solve(self.lu, B, check_finite=False)


# ---------------------------------------------------------------- swimmer
class SwimmerSolution:
    def __init__(self, U, Om, f_sphere, f_tube):
        self.U, self.Om, self.f_sphere, self.f_tube = U, Om, f_sphere, f_tube


class SwimmerSolver:
    """swimmer.hpp:83-289: blocks, rigid map, Schur complement and solves."""

    def __init__(self, tube, sphere, center, mu=1.0, keep_blocks=False):
        self.tube, self.S, self.xc, self.mu = tube, sphere, np.asarray(center, float), mu
        self.Ns = sphere.P
        self.Nt = tube.Nt if tube else 0
        self._build(keep_blocks)

    def slip(self, e, B1, B2):
        """swimmer.hpp:100-104."""
        return squirmer_slip(self.S.centroid, self.xc, e, B1, B2)

    def _K(self):
        Ns = self.Ns
        K = np.zeros((3 * Ns, 6), order="F")
        r = self.S.centroid - self.xc[None, :]
        i = 3 * np.arange(Ns)
        K[i, 0] = 1; K[i + 1, 1] = 1; K[i + 2, 2] = 1
        K[i + 0, 4] = r[:, 2]; K[i + 0, 5] = -r[:, 1]
        K[i + 1, 3] = -r[:, 2]; K[i + 1, 5] = r[:, 0]
        K[i + 2, 3] = r[:, 1]; K[i + 2, 4] = -r[:, 0]
        return K

    def _build(self, keep):
        """swimmer.hpp:180-251."""
        mu, Ns, Nt, S = self.mu, self.Ns, self.Nt, self.S
        ns = 3 * Ns
        dls = np.zeros((Ns, 9))
        if self.tube:
            B, AuBt, _ = block(self.tube.mesh, S, False, mu, True, True)
            D, _, dsum_t = block(S, self.tube.mesh, False, mu, True, False, True)
            dls += dsum_t
        E, AuBs, dsum_s = block(S, S, True, mu, True, True, True)
        dls += dsum_s
        ext = 0.0 if self.tube else 1.0
        for i in range(Ns):
            AuBs[3 * i:3 * i + 3, 3 * i:3 * i + 3] += dls[i].reshape(3, 3) / EIGHT_PI - ext * np.eye(3)
        deflate(S, 0, Ns, E, 0, mu)
        K = self._K()
        Cs = AuBs @ K
        self.Gs, self.Gc = E.copy(order="F"), Cs.copy(order="F")
        self.AuBs = AuBs
        if keep:
            self.E = E
            self.K = K
        if self.tube:
            Ct = AuBt @ K
            self.AuBt, self.D = AuBt, D
            self.Y = self.tube.solve(np.hstack([B, Ct]))
            DY = D @ self.Y
            self.Gs -= DY[:, :ns]
            self.Gc -= DY[:, ns:]
            if keep:
                self.B, self.Ct = B, Ct
        if keep:
            self.Cs = Cs

    def _constraint_matrix(self):
        """swimmer.hpp:108-125: [Gs | Gc] with the scaled force/torque rows."""
        ns = 3 * self.Ns
        n = ns + 6
        M = np.zeros((n, n), order="F")
        M[:ns, :ns] = self.Gs
        M[:ns, ns:] = self.Gc
        amax = float(np.max(np.abs(self.Gs)))
        Amax = float(np.max(5.0 * self.S.area))
        sc = amax / Amax
        r = self.S.centroid - self.xc[None, :]
        A = self.S.area * sc
        p = 3 * np.arange(self.Ns)
        for a in range(3):
            M[ns + a, p + a] = A
        M[ns + 3, p + 1] = -A * r[:, 2]; M[ns + 3, p + 2] = A * r[:, 1]
        M[ns + 4, p + 0] = A * r[:, 2]; M[ns + 4, p + 2] = -A * r[:, 0]
        M[ns + 5, p + 0] = -A * r[:, 1]; M[ns + 5, p + 1] = A * r[:, 0]
        return M

    def reduced_rhs(self, us):
        """swimmer.hpp:256-269: returns (r_s - D T^-1 r_t, T^-1 r_t)."""
        u = np.asarray(us, float).reshape(-1)
        rs = -(self.AuBs @ u)
        rt = np.zeros(3 * self.Nt)
        if self.tube:
            rt = self.tube.solve(-(self.AuBt @ u))
            rs = rs - self.D @ rt
        return rs, rt

    def unpack(self, x, rt):
        """swimmer.hpp:274-288."""
        ns = 3 * self.Ns
        U = x[ns:ns + 3].copy()
        Om = x[ns + 3:ns + 6].copy()
        fs = x[:ns].reshape(-1, 3).copy()
        ft = np.zeros((0, 3))
        if self.tube:
            ft = (rt - self.Y @ x).reshape(-1, 3)
        return SwimmerSolution(U, Om, fs, ft)

    def solve_free(self, slips):
        """swimmer.hpp:107-139."""
        ns = 3 * self.Ns
        M = self._constraint_matrix()
        Rh = np.zeros((ns + 6, len(slips)), order="F")
        rts = []
        for k, sl in enumerate(slips):
            rs, rt = self.reduced_rhs(sl)
            Rh[:ns, k] = rs
            rts.append(rt)
        X = sla.solve(M, Rh, check_finite=False)
        return [self.unpack(X[:, k], rts[k]) for k in range(len(slips))]

    def solve_prescribed(self, U, Om):
        """swimmer.hpp:142-153."""
        ns = 3 * self.Ns
        w = np.concatenate([np.asarray(U, float), np.asarray(Om, float)])
        rhs = sla.solve(self.Gs, -(self.Gc @ w), check_finite=False)
        x = np.concatenate([rhs, w])
        return self.unpack(x, np.zeros(3 * self.Nt))

    def force(self, s):
        """swimmer.hpp:156-160."""
        return -np.sum(self.S.area[:, None] * s.f_sphere, axis=0)

    def velocity(self, s, slip_field, pts):
        """swimmer.hpp:163-173."""
        allm = merge(self.tube.mesh, self.S) if self.tube else self.S
        u = np.zeros((allm.P, 3))
        f = np.zeros((allm.P, 3))
        Nt = self.Nt
        if Nt:
            f[:Nt] = s.f_tube
        r = self.S.centroid - self.xc[None, :]
        u[Nt:] = s.U[None, :] + np.cross(s.Om[None, :], r) + np.asarray(slip_field).reshape(-1, 3)
        f[Nt:] = s.f_sphere
        return velocity_at(allm, u, f, self.mu, pts)


# ---------------------------------------------------------------- duct flow
class DuctFlow:
    """duct_flow.hpp:22-109: mixed-BC completed BIE, LU once, one RHS per dP."""

    class Solution:
        def __init__(self, u, f, Q):
            self.u, self.f, self.Q = u, f, Q

    def __init__(self, R, L, n_theta, n_z, n_r, mu=1.0, keep_matrix=False):
        self.R, self.L, self.mu = R, L, mu
        self.mesh = tube_mesh(R, uniform_z(0, L, n_z), n_theta, n_r)
        self._assemble(keep_matrix)

    def u_known(self, p, b):
        return not (self.mesh.tags[p] != WALL and b == 2)

    def _assemble(self, keep):
        P = self.mesh.P
        tags = self.mesh.tags
        self.cap = [p for p in range(P) if tags[p] != WALL]
        Sb, Db, dls = block(self.mesh, self.mesh, True, self.mu, True, True, True)
        unknown_u = np.zeros(3 * P, dtype=bool)
        for p in self.cap:
            unknown_u[3 * p + 2] = True
        M = np.where(unknown_u[None, :], Db, Sb)
        M = np.asfortranarray(M)
        self.Fk = np.asfortranarray(Sb[:, [3 * p + 2 for p in self.cap]])
        for i in self.cap:
            M[3 * i:3 * i + 3, 3 * i + 2] += dls[i].reshape(3, 3)[:, 2] / EIGHT_PI
        if keep:
            self.M = M.copy(order="F")
        self.lu = sla.lu_factor(M, overwrite_a=True, check_finite=False)

    def solve(self, p_in, p_out):
        P = self.mesh.P
        fk = np.array([p_in if self.mesh.tags[p] == INLET else -p_out for p in self.cap])
        x = sla.lu_solve(self.lu, -(self.Fk @ fk), check_finite=False)
        u = np.zeros((P, 3))
        f = x.reshape(P, 3).copy()
        Q = 0.0
        for k, p in enumerate(self.cap):
            u[p, 2] = f[p, 2]
            f[p, 2] = fk[k]
            if self.mesh.tags[p] == OUTLET:
                Q += u[p, 2] * self.mesh.area[p]
        return DuctFlow.Solution(u, f, Q)

    def velocity(self, s, pts):
        return velocity_at(self.mesh, s.u, s.f, self.mu, pts)

    def exact_uz(self, r, dP):
        return dP / self.L * (self.R * self.R - r * r) / (4 * self.mu)

    def exact_Q(self, dP):
        return math.pi * self.R ** 4 * dP / self.L / (8 * self.mu)


# ---------------------------------------------------------------- trajectory
class TrajectoryParams:
    """trajectory.hpp:23-36 (defaults as in the reference)."""

    def __init__(self, **kw):
        self.alpha = 0.0
        self.a_over_R = 0.3
        self.beta0 = 0.5
        self.pitch0_deg = 0.0
        self.yaw0_deg = 0.0
        self.dt = 0.5
        self.t_max = 100.0
        self.L_over_R = 4.0
        self.n_theta = 30
        self.sphere_level = 2
        self.beta_stop = 0.95
        self.budget_s = 0.0
        for k, v in kw.items():
            if not hasattr(self, k):
                raise KeyError(k)
            setattr(self, k, v)


def fmt10(v):
    return "%.10g" % v


def run_trajectory(P, steps_max=None):
    """trajectory.hpp:42-151 without the file I/O: returns (rows, status), each
    row = t, x, y, z, ex, ey, ez, Ux, Uy, Uz, Omx, Omy, Omz, beta."""
    a = 1.0
    R = a / P.a_over_R
    tube = Tube(R, P.L_over_R * R, a, P.n_theta)
    sph0 = icosphere(a, P.sphere_level)

    def evaluate(y):
        c = np.array([y[0], y[1], 0.0])
        e = np.array(y[3:6]) / np.linalg.norm(y[3:6])
        S = sph0.copy()
        S.translate(c)
        s = SwimmerSolver(tube, S, c)
        k = s.solve_free([s.slip(e, 1, 0), s.slip(e, 0, 1)])
        U = k[0].U + P.alpha * k[1].U
        Om = k[0].Om + P.alpha * k[1].Om
        de = np.cross(Om, e)
        return np.concatenate([U, de]), U, Om

    def beta_of(y):
        return math.hypot(y[0], y[1]) / (R - a)

    b = P.beta0 * (R - a)
    xi, chi = P.pitch0_deg * math.pi / 180, P.yaw0_deg * math.pi / 180
    y = np.array([-b, 0, 0, math.cos(chi) * math.sin(xi), math.sin(chi), math.cos(chi) * math.cos(xi)])
    t, step, hist, rows = 0.0, 0, [], []
    status = "finished"
    while t < P.t_max - 1e-9:
        if beta_of(y) > P.beta_stop:
            status = "wall contact"
            break
        if steps_max is not None and step >= steps_max:
            status = "paused"
            break
        d, U, Om = evaluate(y)
        rows.append([t, *y, *U, *Om, beta_of(y)])
        if len(hist) < 3:
            k2 = evaluate(y + P.dt / 2 * d)[0]
            k3 = evaluate(y + P.dt / 2 * k2)[0]
            k4 = evaluate(y + P.dt * k3)[0]
            y = y + P.dt / 6 * (d + 2 * k2 + 2 * k3 + k4)
        else:
            f1, f2, f3 = hist[2], hist[1], hist[0]
            y = y + P.dt / 24 * (55 * d - 59 * f1 + 37 * f2 - 9 * f3)
        n = math.sqrt(y[3] ** 2 + y[4] ** 2 + y[5] ** 2)
        y[3:6] /= n
        hist.append(d)
        if len(hist) > 3:
            hist.pop(0)
        t += P.dt
        step += 1
    return np.array(rows), status
