"""Python host mirror of the squirmer BEM hot path, over the C ABI (include/sqbem.h).

Same names and argument meaning as the reference's header API
(src/duct_flow.hpp, src/swimmer.hpp, src/trajectory.hpp, src/utils/mesh.hpp,
src/utils/field.hpp): ``Tube``, ``SwimmerSolver`` (``slip``, ``solve_free``,
``solve_prescribed``, ``force``, ``velocity``), ``DuctFlow`` (``solve``,
``velocity``, ``exact_uz``, ``exact_Q``), ``velocity_at``, ``panel_integrals`` and
the mesh generators.  Every compute call runs in the CUDA library
``lib/libsqbem.so``; there is no CPU fallback -- if the library is missing or no
GPU is present the call raises.
"""
import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "lib", "libsqbem.so")

OK, ERR_ARG, ERR_SINGULAR, ERR_CUDA, ERR_NOT_CONVERGED, ERR_NO_DEVICE, ERR_ALLOC, ERR_TIMEOUT = range(8)
FP64, MIXED = 0, 1
WALL, INLET, OUTLET, SPHERE = 0, 1, 2, 10
EIGHT_PI = 8.0 * math.pi


class BEMError(RuntimeError):
    """A failed library call; ``code`` is the sqbem status code."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_VP = ctypes.c_void_p
_c_d, _c_i = ctypes.c_double, ctypes.c_int

# name -> (restype, argtypes); every entry point declared in include/sqbem.h
SIGNATURES = {
    "sqbem_last_error": (ctypes.c_char_p, []),
    "sqbem_version": (ctypes.c_char_p, []),
    "sqbem_launch_count": (ctypes.c_longlong, []),
    "sqbem_set_limits": (_c_i, [ctypes.c_longlong, _c_i]),
    "sqbem_test_gemm_stall": (_c_i, [_c_i]),
    "sqbem_pipe_rates": (_c_i, [_D, _D]),
    "sqbem_tube_mesh": (_c_i, [_c_d, _D, _c_i, _c_i, _c_i, _D, _I, _c_i, _I]),
    "sqbem_swimmer_tube_mesh": (_c_i, [_c_d, _c_d, _c_d, _c_i, _c_i, _D, _I, _c_i, _I]),
    "sqbem_uniform_z": (_c_i, [_c_d, _c_d, _c_i, _D]),
    "sqbem_icosphere": (_c_i, [_c_d, _c_i, _D, _c_i, _D, _I, _c_i, _I]),
    "sqbem_geometry": (_c_i, [_c_i, _D, _D, _D, _D, _D]),
    "sqbem_panel_integrals": (_c_i, [_c_i, _D, _D, _I, _D, _D]),
    "sqbem_solve_dense": (_c_i, [_c_i, _c_i, _D, _D, _I]),
    "sqbem_velocity_at": (_c_i, [_c_i, _D, _D, _D, _c_d, _c_i, _D, _D, _c_i]),
    "sqbem_velocity_at_noalloc": (_c_i, [_c_i, _VP, _VP, _VP, _c_d, _c_i, _VP, _VP, _c_i, _VP]),
    "sqbem_tube_create": (_c_i, [_c_d, _c_d, _c_d, _c_i, _c_i, _c_d, _c_i, ctypes.POINTER(_VP)]),
    "sqbem_tube_panels": (_c_i, [_VP, _I]),
    "sqbem_tube_mesh_get": (_c_i, [_VP, _D, _I]),
    "sqbem_tube_destroy": (None, [_VP]),
    "sqbem_tube_symmetry": (_c_i, [_c_d, _c_d, _c_d, _c_i, _c_i, _I, _I, _I]),
    "sqbem_tube_block_f32": (_c_i, [_c_d, _c_d, _c_d, _c_i, _c_i, _c_d, _c_i, _VP]),
    "sqbem_tube_fourier_solve": (_c_i, [_c_d, _c_d, _c_d, _c_i, _c_i, _c_d, _c_i, _D, _D]),
    "sqbem_swimmer_create": (_c_i, [_VP, _c_i, _D, _I, _D, _c_d, _c_i, ctypes.POINTER(_VP)]),
    "sqbem_swimmer_solve_free": (_c_i, [_VP, _c_i, _D, _D, _D, _D, _D]),
    "sqbem_swimmer_solve_prescribed": (_c_i, [_VP, _D, _D, _D, _D]),
    "sqbem_swimmer_timings": (_c_i, [_VP, _D, _D]),
    "sqbem_swimmer_refinement": (_c_i, [_VP, _I, _D]),
    "sqbem_swimmer_adjoint": (_c_i, [_VP, _c_i, _D, _D, _D, _D, _D]),
    "sqbem_swimmer_destroy": (None, [_VP]),
    "sqbem_duct_create": (_c_i, [_c_d, _c_d, _c_i, _c_i, _c_i, _c_d, _c_i, ctypes.POINTER(_VP)]),
    "sqbem_duct_panels": (_c_i, [_VP, _I]),
    "sqbem_duct_mesh_get": (_c_i, [_VP, _D, _I]),
    "sqbem_duct_solve": (_c_i, [_VP, _c_d, _c_d, _D, _D, _D]),
    "sqbem_duct_destroy": (None, [_VP]),
    "sqbem_transfer_bytes": (_c_i, [ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
    "sqbem_kernel_stats_enable": (_c_i, [_c_i]),
    "sqbem_kernel_stats": (_c_i, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_longlong), _D, _D, _D]),
    "sqbem_kernel_stats_classes": (_c_i, [ctypes.c_char_p, _c_i]),
    "sqbem_trim_pool": (_c_i, []),
    "sqbem_kinematics_batch": (_c_i, [_c_i, _VP, _c_i, _D, _D]),
    "sqbem_kinematics_batch_tractions": (_c_i, [_c_i, _VP, _c_i, _D, ctypes.POINTER(_D), ctypes.POINTER(_D), _D]),
    "sqbem_adjoint_batch": (_c_i, [_c_i, _VP, _c_i, _D, _D]),
    "sqbem_trajectory_defaults": (_c_i, [_VP]),
    "sqbem_tube_cache_stats": (_c_i, [ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), _I]),
    "sqbem_tube_cache_clear": (_c_i, []),
    "sqbem_run_trajectory": (_c_i, [_VP, ctypes.c_char_p, _c_i, _c_i, ctypes.c_char_p, _c_i]),
    "sqbem_trajectory_ensemble": (_c_i, [_c_i, _D, _D, _VP, _c_i, _c_i, _c_i, _D, _D, _D, _I, _D]),
    "sqbem_ensemble_field": (_c_i, [_c_i, _D, _D, _VP, _c_i, _c_i, _c_i, _c_d, _c_i, _D, _D]),
    "sqbem_gemm_mixed": (_c_i, [_c_i, _c_i, _c_i, ctypes.c_float, ctypes.POINTER(ctypes.c_float), _c_i,
                                ctypes.POINTER(ctypes.c_float), _c_i, ctypes.c_float,
                                ctypes.POINTER(ctypes.c_float), _c_i]),
    "sqbem_gemm_mixed_ex": (_c_i, [_c_i, _c_i, _c_i, _c_i, _c_i, ctypes.c_float, ctypes.POINTER(ctypes.c_float), _c_i,
                                   ctypes.POINTER(ctypes.c_float), _c_i, ctypes.c_float,
                                   ctypes.POINTER(ctypes.c_float), _c_i]),
    "sqbem_gemm_variants": (_c_i, [_I]),
    "sqbem_gemm_timing": (_c_i, [_c_i, _c_i, _c_i, _c_i, _c_i, _c_i, ctypes.c_float, _c_i, _D]),
}


def gemm_mixed(A, B, C=None, alpha=1.0, beta=0.0, variant=-1, products=3):
    """linalg.hpp:42-48 gemm on the tensor cores, split-BF16 operands: returns
    alpha A B + beta C as FP32.  variant: the kernel's tile variant (-1: the
    tuning table's choice); products: 3 (hi*hi + hi*lo + lo*hi) or 2 (A rounded
    to BF16)."""
    A = np.asfortranarray(np.asarray(A, dtype=np.float32))
    B = np.asfortranarray(np.asarray(B, dtype=np.float32))
    M, K = A.shape
    N = B.shape[1]
    Cm = np.asfortranarray(np.zeros((M, N), np.float32) if C is None else np.asarray(C, dtype=np.float32).copy())
    fp = ctypes.POINTER(ctypes.c_float)
    if variant == -1 and products == 3:
        _check(lib().sqbem_gemm_mixed(M, N, K, alpha, A.ctypes.data_as(fp), M, B.ctypes.data_as(fp), K, beta,
                                      Cm.ctypes.data_as(fp), M))
    else:
        _check(lib().sqbem_gemm_mixed_ex(variant, products, M, N, K, alpha, A.ctypes.data_as(fp), M,
                                         B.ctypes.data_as(fp), K, beta, Cm.ctypes.data_as(fp), M))
    return Cm


class TrajParams(ctypes.Structure):
    """sqbem_traj_params = TrajectoryParams (src/trajectory.hpp:23-36)."""
    _fields_ = [("alpha", ctypes.c_double), ("a_over_R", ctypes.c_double), ("beta0", ctypes.c_double),
                ("pitch0_deg", ctypes.c_double), ("yaw0_deg", ctypes.c_double), ("dt", ctypes.c_double),
                ("t_max", ctypes.c_double), ("L_over_R", ctypes.c_double), ("n_theta", ctypes.c_int),
                ("sphere_level", ctypes.c_int), ("beta_stop", ctypes.c_double), ("budget_s", ctypes.c_double)]

    def __init__(self, **kw):
        super().__init__()
        _check(lib().sqbem_trajectory_defaults(ctypes.byref(self)))
        for k, v in kw.items():
            if k not in dict(self._fields_):
                raise KeyError(k)
            setattr(self, k, v)


def run_trajectory(P, out_prefix, verbose=False, precision=FP64):
    """trajectory.hpp:42-151 on the GPU; writes <out_prefix>.csv / .ckpt, returns the status."""
    buf = ctypes.create_string_buffer(64)
    _check(lib().sqbem_run_trajectory(ctypes.byref(P), out_prefix.encode(), int(verbose), precision, buf, 64))
    return buf.value.decode()


def trajectory_ensemble(y0, alpha, P, steps, scheme=1, precision=MIXED):
    """n swimmers in one tube: returns (states (n, steps+1, 6), U (n, steps, 3),
    Om (n, steps, 3), status (n,), device seconds)."""
    y0 = _f64(y0).reshape(-1, 6)
    n = y0.shape[0]
    al = _f64(np.broadcast_to(np.asarray(alpha, dtype=np.float64), (n,)))
    states = np.zeros((n, steps + 1, 6))
    U = np.zeros((n, steps, 3))
    Om = np.zeros((n, steps, 3))
    status = np.zeros(n, dtype=np.int32)
    secs = ctypes.c_double(0)
    _check(lib().sqbem_trajectory_ensemble(n, _dp(y0), _dp(al), ctypes.byref(P), steps, scheme, precision,
                                           _dp(states), _dp(U), _dp(Om), _ip(status), ctypes.byref(secs)))
    return states, U, Om, status, secs.value


def ensemble_field(states, alpha, P, nx=25, ny=25, nz=41, z_extent=7.0, precision=MIXED):
    """Velocity on an nx x ny x nz grid per swimmer (x, y in [-0.97 R, 0.97 R],
    z in [-z_extent, z_extent] around the sphere; NaN outside the tube section and
    within 1.03 a of the centre).  Returns (u (n, nx, ny, nz, 3), device seconds)."""
    st = _f64(states).reshape(-1, 6)
    n = st.shape[0]
    al = _f64(np.broadcast_to(np.asarray(alpha, dtype=np.float64), (n,)))
    u = np.zeros((n, nx, ny, nz, 3))
    secs = ctypes.c_double(0)
    _check(lib().sqbem_ensemble_field(n, _dp(st), _dp(al), ctypes.byref(P), nx, ny, nz, z_extent, precision, _dp(u),
                                      ctypes.byref(secs)))
    return u, secs.value


def field_grid(R, c, nx=25, ny=25, nz=41, z_extent=7.0, a=1.0):
    """The points of ensemble_field's grid (n, 3) and its mask (True = evaluated)."""
    lim = 0.97 * R
    x = -lim + 2 * lim * np.arange(nx) / (nx - 1)
    y = -lim + 2 * lim * np.arange(ny) / (ny - 1)
    z = -z_extent + 2 * z_extent * np.arange(nz) / (nz - 1)
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    pts = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)
    d = np.sqrt(np.sum((pts - np.asarray(c, float)[None, :]) ** 2, axis=1))
    mask = (pts[:, 0] ** 2 + pts[:, 1] ** 2 <= lim * lim) & (d >= 1.03 * a)
    return pts, mask


class Instance(ctypes.Structure):
    """sqbem_instance (include/sqbem.h): one kinematics case of a batch."""
    _fields_ = [("a_over_R", ctypes.c_double), ("beta", ctypes.c_double), ("L_over_R", ctypes.c_double),
                ("e", ctypes.c_double * 3), ("n_theta", ctypes.c_int), ("n_r", ctypes.c_int),
                ("sphere_level", ctypes.c_int), ("towed", ctypes.c_int)]


RESULT_STRIDE = 16
ADJOINT_STRIDE = 48

_LIB = None


def lib():
    """The loaded CUDA library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise BEMError(ERR_NO_DEVICE, "libsqbem.so not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def _check(rc):
    if rc != OK:
        raise BEMError(rc, lib().sqbem_last_error().decode())


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _ip(a):
    return None if a is None else a.ctypes.data_as(_I)


def _f64(x, shape=None):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    return a.reshape(shape) if shape is not None else a


def launch_count():
    return int(lib().sqbem_launch_count())


def transfer_bytes():
    """(host->device, device->host) bytes copied by the library so far"""
    h, d = ctypes.c_longlong(0), ctypes.c_longlong(0)
    _check(lib().sqbem_transfer_bytes(ctypes.byref(h), ctypes.byref(d)))
    return h.value, d.value


def trim_pool():
    """return the library's cached device memory to the driver"""
    _check(lib().sqbem_trim_pool())


def kernel_stats_enable(on=True):
    _check(lib().sqbem_kernel_stats_enable(1 if on else 0))


def kernel_stats(cls):
    """(launches, seconds, flops, bytes) of one kernel class since enabling"""
    n, s, f, b = ctypes.c_longlong(0), ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
    _check(lib().sqbem_kernel_stats(cls.encode(), ctypes.byref(n), ctypes.byref(s), ctypes.byref(f), ctypes.byref(b)))
    return n.value, s.value, f.value, b.value


def kernel_stats_classes():
    buf = ctypes.create_string_buffer(4096)
    _check(lib().sqbem_kernel_stats_classes(buf, 4096))
    return [c for c in buf.value.decode().split(",") if c]


def _instances(instances):
    n = len(instances)
    arr = (Instance * n)()
    for k, d in enumerate(instances):
        arr[k].a_over_R = d["a_over_R"]
        arr[k].beta = d["beta"]
        arr[k].L_over_R = d.get("L_over_R", 4.0)
        e = d.get("e", (0.0, 0.0, 1.0))
        for c in range(3):
            arr[k].e[c] = e[c]
        arr[k].n_theta = d.get("n_theta", 24)
        arr[k].n_r = d.get("n_r", 4)
        arr[k].sphere_level = d["sphere_level"]
        arr[k].towed = int(d.get("towed", 0))
    return arr


def kinematics_batch(instances, precision=MIXED, tractions=False):
    """sqbem_kinematics_batch: instances = list of dicts with a_over_R, beta,
    L_over_R, e, n_theta, n_r, sphere_level, towed.  Returns (results
    (n x RESULT_STRIDE), device seconds); with tractions=True
    (sqbem_kinematics_batch_tractions) also the lists f_sphere and f_tube of
    (2, N, 3) arrays per instance (slip modes B1 = 1 and B2 = 1)."""
    n = len(instances)
    arr = _instances(instances)
    res = np.zeros((n, RESULT_STRIDE))
    secs = ctypes.c_double(0)
    if not tractions:
        _check(lib().sqbem_kinematics_batch(n, ctypes.cast(arr, _VP), precision, _dp(res), ctypes.byref(secs)))
        return res, secs.value
    fs = [np.zeros((2, 20 * 4 ** int(d["sphere_level"]), 3)) for d in instances]
    ft = [np.zeros((2, _tube_panels(d), 3)) for d in instances]
    ps = (_D * max(n, 1))(*[_dp(a) for a in fs])
    pt = (_D * max(n, 1))(*[_dp(a) for a in ft])
    _check(lib().sqbem_kinematics_batch_tractions(n, ctypes.cast(arr, _VP), precision, _dp(res), ps, pt,
                                                  ctypes.byref(secs)))
    return res, secs.value, fs, ft


def _tube_panels(d):
    """panel count of an instance's tube (0 for the unbounded fluid)"""
    if d["a_over_R"] <= 0:
        return 0
    R = 1.0 / d["a_over_R"]
    P = ctypes.c_int(0)
    _check(lib().sqbem_swimmer_tube_mesh(R, d.get("L_over_R", 4.0) * R, 1.0, int(d.get("n_theta", 24)),
                                         int(d.get("n_r", 4)), None, None, 0, ctypes.byref(P)))
    return P.value


def tube_cache_stats():
    """(tubes built, cache hits, entries held) of the trajectory calls' tube cache"""
    b, h, e = ctypes.c_longlong(0), ctypes.c_longlong(0), ctypes.c_int(0)
    _check(lib().sqbem_tube_cache_stats(ctypes.byref(b), ctypes.byref(h), ctypes.byref(e)))
    return b.value, h.value, e.value


def tube_cache_clear():
    _check(lib().sqbem_tube_cache_clear())


def set_limits(gemm_wait_cycles=-1, refine_max_iterations=-1):
    """sqbem_set_limits: bounded-wait length of the tensor-core GEMM (SM cycles)
    and the refinement cap; -1 restores a default."""
    _check(lib().sqbem_set_limits(int(gemm_wait_cycles), int(refine_max_iterations)))


def pipe_rates():
    """(FP64, FP32) FMA throughput of this GPU in TFLOP/s, measured now."""
    a, b = ctypes.c_double(0), ctypes.c_double(0)
    _check(lib().sqbem_pipe_rates(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def adjoint_batch(instances, precision=FP64):
    """sqbem_adjoint_batch: per instance and slip mode m (0: B1, 1: B2) the
    free-swimming U, Om and their derivatives with respect to the sphere centre.
    Returns (dict of arrays U (n, 2, 3), Om (n, 2, 3), dU_dc (n, 2, 3, 3),
    dOm_dc (n, 2, 3, 3); device seconds)."""
    n = len(instances)
    arr = _instances(instances)
    res = np.zeros((n, ADJOINT_STRIDE))
    secs = ctypes.c_double(0)
    _check(lib().sqbem_adjoint_batch(n, ctypes.cast(arr, _VP), precision, _dp(res), ctypes.byref(secs)))
    r = res.reshape(n, 2, 24)
    out = dict(U=r[:, :, 0:3].copy(), Om=r[:, :, 3:6].copy(), dU_dc=r[:, :, 6:15].reshape(n, 2, 3, 3).copy(),
               dOm_dc=r[:, :, 15:24].reshape(n, 2, 3, 3).copy())
    return out, secs.value


# ---------------------------------------------------------------- meshes
class Mesh:
    """Per-panel vertices, tags and geometry (src/utils/mesh.hpp:50-91)."""

    def __init__(self, V, tags):
        self.V = _f64(V).reshape(-1, 9).copy()
        self.tags = np.ascontiguousarray(tags, dtype=np.int32).copy()
        self.geometry()

    @property
    def P(self):
        return self.V.shape[0]

    def geometry(self):
        P = self.P
        self.normal = np.zeros((P, 3))
        self.centroid = np.zeros((P, 3))
        self.area = np.zeros(P)
        self.h = np.zeros(P)
        _check(lib().sqbem_geometry(P, _dp(self.V), _dp(self.normal), _dp(self.centroid), _dp(self.area),
                                    _dp(self.h)))

    def translate(self, d):
        self.V = self.V + np.tile(_f64(d), 3)[None, :]
        self.geometry()

    def copy(self):
        return Mesh(self.V, self.tags)

    def total_area(self):
        return float(sum(self.area))


def merge(a, b):
    return Mesh(np.vstack([a.V, b.V]), np.concatenate([a.tags, b.tags]))


def _make_mesh(fn, *args):
    P = ctypes.c_int(0)
    _check(fn(*args, None, None, 0, ctypes.byref(P)))
    V = np.zeros((P.value, 9))
    tags = np.zeros(P.value, dtype=np.int32)
    _check(fn(*args, _dp(V), _ip(tags), P.value, ctypes.byref(P)))
    return Mesh(V, tags)


def uniform_z(z0, z1, nz):
    z = np.zeros(nz + 1)
    _check(lib().sqbem_uniform_z(z0, z1, nz, _dp(z)))
    return z


def tube_mesh(R, z, n_theta, n_r):
    z = _f64(z)
    return _make_mesh(lib().sqbem_tube_mesh, R, _dp(z), len(z), n_theta, n_r)


def swimmer_tube_mesh(R, L, a, n_theta, n_r=4):
    return _make_mesh(lib().sqbem_swimmer_tube_mesh, R, L, a, n_theta, n_r)


def tube_symmetry(R, L, a, n_theta, n_r=4):
    """sqbem_tube_symmetry: (nb, sector, rep) of the swimmer tube mesh -- panel
    p is sector-0 representative rep[p] rotated by sector[p] sectors of 2 pi /
    n_theta; nb = 0 (and None, None) if the mesh has no such symmetry."""
    nb = ctypes.c_int(0)
    _check(lib().sqbem_tube_symmetry(R, L, a, n_theta, n_r, ctypes.byref(nb), None, None))
    if nb.value == 0:
        return 0, None, None
    n = nb.value * n_theta
    sector = np.zeros(n, dtype=np.int32)
    rep = np.zeros(n, dtype=np.int32)
    _check(lib().sqbem_tube_symmetry(R, L, a, n_theta, n_r, ctypes.byref(nb), _ip(sector), _ip(rep)))
    return nb.value, sector, rep


def tube_block_f32(R, L, a, n_theta, n_r=4, mu=1.0, symmetric=True):
    """sqbem_tube_block_f32: the mixed path's deflated FP32 tube block (3 Nt x
    3 Nt), assembled from the rows of one sector or directly."""
    Nt = swimmer_tube_mesh(R, L, a, n_theta, n_r).P
    T = np.zeros((3 * Nt, 3 * Nt), dtype=np.float32, order="F")
    _check(lib().sqbem_tube_block_f32(R, L, a, n_theta, n_r, mu, 1 if symmetric else 0,
                                      T.ctypes.data_as(_VP)))
    return T


def tube_fourier_solve(R, L, a, n_theta, X, n_r=4, mu=1.0):
    """sqbem_tube_fourier_solve: T^{-1} X through the tube's Fourier blocks (X:
    3 Nt x nc)."""
    X = np.asfortranarray(X, dtype=np.float64)
    Y = np.zeros_like(X, order="F")
    _check(lib().sqbem_tube_fourier_solve(R, L, a, n_theta, n_r, mu, X.shape[1], _dp(X), _dp(Y)))
    return Y


def icosphere(a, level, center=(0.0, 0.0, 0.0), tag=SPHERE):
    c = _f64(center)
    return _make_mesh(lib().sqbem_icosphere, a, level, _dp(c), tag)


# ---------------------------------------------------------------- kernels
def panel_integrals(V9, x0, self_flag):
    """kernels.hpp:67-82 on the GPU for arrays of (panel, target, self)."""
    V9 = _f64(V9).reshape(-1, 9)
    n = V9.shape[0]
    x0 = _f64(x0).reshape(n, 3)
    sf = np.ascontiguousarray(np.broadcast_to(np.asarray(self_flag, dtype=np.int32), (n,)))
    SL = np.zeros((n, 9))
    DL = np.zeros((n, 9))
    _check(lib().sqbem_panel_integrals(n, _dp(V9), _dp(x0), _ip(sf), _dp(SL), _dp(DL)))
    return SL, DL


def squirmer_slip(x, center, e, B1, B2):
    """kernels.hpp:107-111: u_s = (B1 + B2 cos) (cos rhat - e), host arithmetic."""
    x = _f64(x).reshape(-1, 3)
    r = x - _f64(center)[None, :]
    rh = r * (1.0 / np.sqrt(np.sum(r * r, axis=1)))[:, None]
    ct = rh @ _f64(e)
    return (B1 + B2 * ct)[:, None] * (ct[:, None] * rh - _f64(e)[None, :])


def solve_dense(A, B):
    """linalg.hpp:53-58 (dgesv) on the GPU: returns (A^{-1} B, pivoted)."""
    A = np.asfortranarray(np.asarray(A, dtype=np.float64))
    B = np.asarray(B, dtype=np.float64)
    vec = B.ndim == 1
    X = np.asfortranarray(B.reshape(B.shape[0], -1).copy())
    piv = ctypes.c_int(0)
    _check(lib().sqbem_solve_dense(A.shape[0], X.shape[1], A.ctypes.data_as(_D), X.ctypes.data_as(_D),
                                   ctypes.byref(piv)))
    return (X[:, 0] if vec else X), bool(piv.value)


def velocity_at(M, u, f, mu, points, precision=FP64):
    """field.hpp:18-34 on the GPU."""
    pts = _f64(points).reshape(-1, 3)
    u = _f64(u).reshape(-1, 3)
    f = _f64(f).reshape(-1, 3)
    out = np.zeros_like(pts)
    _check(lib().sqbem_velocity_at(M.P, _dp(M.V), _dp(u), _dp(f), mu, pts.shape[0], _dp(pts), _dp(out), precision))
    return out


# ---------------------------------------------------------------- tube / swimmer
class Tube:
    """Tube (src/swimmer.hpp:33-75): mesh, T, deflation and LU on the GPU."""

    def __init__(self, R, L, a, n_theta, n_r=4, mu=1.0, precision=FP64):
        self.R, self.L, self.mu, self.precision = R, L, mu, precision
        h = _VP()
        _check(lib().sqbem_tube_create(R, L, a, n_theta, n_r, mu, precision, ctypes.byref(h)))
        self._h = h
        n = ctypes.c_int(0)
        _check(lib().sqbem_tube_panels(h, ctypes.byref(n)))
        self.Nt = n.value
        V = np.zeros((self.Nt, 9))
        tags = np.zeros(self.Nt, dtype=np.int32)
        _check(lib().sqbem_tube_mesh_get(h, _dp(V), _ip(tags)))
        self.mesh = Mesh(V, tags)

    def close(self):
        if getattr(self, "_h", None):
            lib().sqbem_tube_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SwimmerSolution:
    def __init__(self, U, Om, f_sphere, f_tube):
        self.U, self.Om, self.f_sphere, self.f_tube = U, Om, f_sphere, f_tube


class SwimmerSolver:
    """SwimmerSolver (src/swimmer.hpp:83-289) on the GPU.  tube=None is the
    unbounded fluid; the tube must outlive the solver."""

    def __init__(self, tube, sphere, center, mu=1.0, precision=FP64):
        self.tube, self.S, self.xc, self.mu = tube, sphere, _f64(center).copy(), mu
        self.precision = precision
        self.Ns = sphere.P
        self.Nt = tube.Nt if tube else 0
        h = _VP()
        _check(lib().sqbem_swimmer_create(tube._h if tube else None, self.Ns, _dp(sphere.V), _ip(sphere.tags),
                                          _dp(self.xc), mu, precision, ctypes.byref(h)))
        self._h = h
        ta, ts = ctypes.c_double(0), ctypes.c_double(0)
        _check(lib().sqbem_swimmer_timings(h, ctypes.byref(ta), ctypes.byref(ts)))
        self.t_assembly, self.t_schur = ta.value, ts.value

    def slip(self, e, B1, B2):
        return squirmer_slip(self.S.centroid, self.xc, e, B1, B2)

    def solve_free(self, slips):
        nr = len(slips)
        sl = _f64(np.stack([np.asarray(s, float).reshape(-1, 3) for s in slips]))
        U = np.zeros((nr, 3))
        Om = np.zeros((nr, 3))
        fs = np.zeros((nr, self.Ns, 3))
        ft = np.zeros((nr, self.Nt, 3))
        _check(lib().sqbem_swimmer_solve_free(self._h, nr, _dp(sl), _dp(U), _dp(Om), _dp(fs),
                                              _dp(ft) if self.Nt else None))
        return [SwimmerSolution(U[k], Om[k], fs[k], ft[k]) for k in range(nr)]

    def solve_prescribed(self, U, Om):
        fs = np.zeros((self.Ns, 3))
        ft = np.zeros((self.Nt, 3))
        _check(lib().sqbem_swimmer_solve_prescribed(self._h, _dp(_f64(U)), _dp(_f64(Om)), _dp(fs),
                                                    _dp(ft) if self.Nt else None))
        return SwimmerSolution(_f64(U).copy(), _f64(Om).copy(), fs, ft)

    def adjoint(self, slips):
        """solve_free plus the derivatives of U and Omega with respect to a rigid
        translation of the sphere: returns U (nr, 3), Om (nr, 3), dU_dc
        (nr, 3, 3) and dOm_dc (nr, 3, 3), [k, a, j] = d(.)_a / dc_j."""
        nr = len(slips)
        sl = _f64(np.stack([np.asarray(s, float).reshape(-1, 3) for s in slips]))
        U = np.zeros((nr, 3))
        Om = np.zeros((nr, 3))
        dU = np.zeros((nr, 3, 3))
        dOm = np.zeros((nr, 3, 3))
        _check(lib().sqbem_swimmer_adjoint(self._h, nr, _dp(sl), _dp(U), _dp(Om), _dp(dU), _dp(dOm)))
        return U, Om, dU, dOm

    def refinement(self):
        it, res = ctypes.c_int(0), ctypes.c_double(0)
        _check(lib().sqbem_swimmer_refinement(self._h, ctypes.byref(it), ctypes.byref(res)))
        return it.value, res.value

    def force(self, s):
        """swimmer.hpp:156-160: F = -sum f dA."""
        return -np.sum(self.S.area[:, None] * s.f_sphere, axis=0)

    def velocity(self, s, slip_field, pts):
        """swimmer.hpp:163-173."""
        allm = merge(self.tube.mesh, self.S) if self.tube else self.S
        u = np.zeros((allm.P, 3))
        f = np.zeros((allm.P, 3))
        if self.Nt:
            f[:self.Nt] = s.f_tube
        r = self.S.centroid - self.xc[None, :]
        u[self.Nt:] = s.U[None, :] + np.cross(s.Om[None, :], r) + np.asarray(slip_field).reshape(-1, 3)
        f[self.Nt:] = s.f_sphere
        return velocity_at(allm, u, f, self.mu, pts, self.precision)

    def close(self):
        if getattr(self, "_h", None):
            lib().sqbem_swimmer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- duct flow
class DuctFlow:
    """DuctFlow (src/duct_flow.hpp:22-109) on the GPU."""

    class Solution:
        def __init__(self, u, f, Q):
            self.u, self.f, self.Q = u, f, Q

    def __init__(self, R, L, n_theta, n_z, n_r, mu=1.0, precision=FP64):
        self.R, self.L, self.mu, self.precision = R, L, mu, precision
        h = _VP()
        _check(lib().sqbem_duct_create(R, L, n_theta, n_z, n_r, mu, precision, ctypes.byref(h)))
        self._h = h
        n = ctypes.c_int(0)
        _check(lib().sqbem_duct_panels(h, ctypes.byref(n)))
        V = np.zeros((n.value, 9))
        tags = np.zeros(n.value, dtype=np.int32)
        _check(lib().sqbem_duct_mesh_get(h, _dp(V), _ip(tags)))
        self.mesh = Mesh(V, tags)

    def solve(self, p_in, p_out):
        P = self.mesh.P
        u = np.zeros((P, 3))
        f = np.zeros((P, 3))
        Q = ctypes.c_double(0)
        _check(lib().sqbem_duct_solve(self._h, p_in, p_out, _dp(u), _dp(f), ctypes.byref(Q)))
        return DuctFlow.Solution(u, f, Q.value)

    def velocity(self, s, pts):
        return velocity_at(self.mesh, s.u, s.f, self.mu, pts, self.precision)

    def exact_uz(self, r, dP):
        return dP / self.L * (self.R * self.R - r * r) / (4 * self.mu)

    def exact_Q(self, dP):
        return math.pi * self.R ** 4 * dP / self.L / (8 * self.mu)

    def close(self):
        if getattr(self, "_h", None):
            lib().sqbem_duct_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
